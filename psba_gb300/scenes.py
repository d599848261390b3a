"""Seeded synthetic bundle-adjustment scenes.

The reference ships small text scenes and points at public datasets
(Dubrovnik, Venice, Ladybug, ...) whose point files are not available here;
these generators stand in for them with the same shapes: camera counts,
point counts, observations per point and value ranges.

Conventions match the solver (and the reference, PSBA/main.cpp:131-149):

* ``K``      (C, 5)  fx, cx, cy, aspect, skew  -- held fixed
* ``q0``     (C, 4)  initial rotation quaternion s, v1, v2, v3 (s >= 0)
* ``cams``   (C, 6)  local rotation vector part v (starts at 0) and translation t
* ``pts``    (P, 3)
* ``meas``   (O, 2)  observations sorted by (point, camera)
* ``obs_pt``, ``obs_cam`` (O,) int32

A camera maps X to Xc = R(q(v) (x) q0) X + t and projects
x = (fx Xc + skew Yc + cx Zc) / Zc, y = (fx ar Yc + cy Zc) / Zc.
"""
from dataclasses import dataclass, field
from typing import Optional

import numpy as np


@dataclass
class Scene:
    name: str
    K: np.ndarray
    q0: np.ndarray
    cams: np.ndarray
    pts: np.ndarray
    meas: np.ndarray
    obs_pt: np.ndarray
    obs_cam: np.ndarray
    cams_true: Optional[np.ndarray] = None
    pts_true: Optional[np.ndarray] = None
    q_true: Optional[np.ndarray] = None
    meta: dict = field(default_factory=dict)
    cnp: int = 6  # parameters per camera: 6 (fixed K), 11 (+ K), 16 (+ K + distortion)

    @property
    def n_cams(self):
        return int(self.K.shape[0])

    @property
    def n_pts(self):
        return int(self.pts.shape[0])

    @property
    def n_obs(self):
        return int(self.meas.shape[0])

    def copy(self):
        sc = Scene(self.name, self.K.copy(), self.q0.copy(), self.cams.copy(), self.pts.copy(),
                   self.meas.copy(), self.obs_pt.copy(), self.obs_cam.copy(),
                   None if self.cams_true is None else self.cams_true.copy(),
                   None if self.pts_true is None else self.pts_true.copy(),
                   None if self.q_true is None else self.q_true.copy(), dict(self.meta), self.cnp)
        cov = getattr(self, "cov", None)
        sc.cov = None if cov is None else cov.copy()
        return sc

    def validate(self):
        C, P, O = self.n_cams, self.n_pts, self.n_obs
        assert self.K.shape == (C, 5) and self.q0.shape == (C, 4) and self.cams.shape == (C, self.cnp)
        assert self.cnp in (6, 11, 16)
        assert self.pts.shape == (P, 3) and self.meas.shape == (O, 2)
        assert self.obs_pt.shape == (O,) and self.obs_cam.shape == (O,)
        key = self.obs_pt.astype(np.int64) * C + self.obs_cam
        assert np.all(np.diff(key) > 0), "observations must be sorted by (point, camera), no repeats"
        assert self.obs_pt.min() >= 0 and self.obs_pt.max() < P
        assert self.obs_cam.min() >= 0 and self.obs_cam.max() < C
        return True


# ---------------------------------------------------------------------------
# quaternion helpers

def quat_mul(a, b):
    """Hamilton product of (..., 4) arrays, scalar first."""
    s1, v1 = a[..., :1], a[..., 1:]
    s2, v2 = b[..., :1], b[..., 1:]
    s = s1 * s2 - np.sum(v1 * v2, axis=-1, keepdims=True)
    v = s1 * v2 + s2 * v1 + np.cross(v1, v2)
    return np.concatenate([s, v], axis=-1)


def quat_from_rotvec(w):
    th = np.linalg.norm(w, axis=-1, keepdims=True)
    half = 0.5 * th
    with np.errstate(invalid="ignore", divide="ignore"):
        k = np.where(th > 1e-300, np.sin(half) / np.where(th > 0, th, 1.0), 0.5)
    return np.concatenate([np.cos(half), w * k], axis=-1)


def quat_from_matrix(R):
    """Rotation matrices (..., 3, 3) -> unit quaternions with s >= 0."""
    R = np.asarray(R, dtype=np.float64)
    out = np.empty(R.shape[:-2] + (4,))
    for idx in np.ndindex(R.shape[:-2]):
        m = R[idx]
        tr = m[0, 0] + m[1, 1] + m[2, 2]
        if tr > 0:
            s = np.sqrt(tr + 1.0) * 2
            q = [0.25 * s, (m[2, 1] - m[1, 2]) / s, (m[0, 2] - m[2, 0]) / s, (m[1, 0] - m[0, 1]) / s]
        elif m[0, 0] > m[1, 1] and m[0, 0] > m[2, 2]:
            s = np.sqrt(1.0 + m[0, 0] - m[1, 1] - m[2, 2]) * 2
            q = [(m[2, 1] - m[1, 2]) / s, 0.25 * s, (m[0, 1] + m[1, 0]) / s, (m[0, 2] + m[2, 0]) / s]
        elif m[1, 1] > m[2, 2]:
            s = np.sqrt(1.0 + m[1, 1] - m[0, 0] - m[2, 2]) * 2
            q = [(m[0, 2] - m[2, 0]) / s, (m[0, 1] + m[1, 0]) / s, 0.25 * s, (m[1, 2] + m[2, 1]) / s]
        else:
            s = np.sqrt(1.0 + m[2, 2] - m[0, 0] - m[1, 1]) * 2
            q = [(m[1, 0] - m[0, 1]) / s, (m[0, 2] + m[2, 0]) / s, (m[1, 2] + m[2, 1]) / s, 0.25 * s]
        q = np.array(q)
        q /= np.linalg.norm(q)
        if q[0] < 0:
            q = -q
        out[idx] = q
    return out


def quat_to_matrix(q):
    s, a, b, c = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
    R = np.empty(q.shape[:-1] + (3, 3))
    R[..., 0, 0] = 1 - 2 * (b * b + c * c)
    R[..., 0, 1] = 2 * (a * b - s * c)
    R[..., 0, 2] = 2 * (a * c + s * b)
    R[..., 1, 0] = 2 * (a * b + s * c)
    R[..., 1, 1] = 1 - 2 * (a * a + c * c)
    R[..., 1, 2] = 2 * (b * c - s * a)
    R[..., 2, 0] = 2 * (a * c - s * b)
    R[..., 2, 1] = 2 * (b * c + s * a)
    R[..., 2, 2] = 1 - 2 * (a * a + b * b)
    return R


def look_at(center, target, up=(0.0, 0.0, 1.0)):
    """World-to-camera rotation whose +Z axis points from center to target."""
    z = np.asarray(target, float) - np.asarray(center, float)
    z /= np.linalg.norm(z)
    x = np.cross(z, up)
    if np.linalg.norm(x) < 1e-9:
        x = np.cross(z, (1.0, 0.0, 0.0))
    x /= np.linalg.norm(x)
    y = np.cross(z, x)
    return np.stack([x, y, z])


def project(K, q, t, X):
    """Pinhole projection of points X (n,3) by per-row cameras (n,...)."""
    R = quat_to_matrix(q)
    Xc = np.einsum("nij,nj->ni", R, X) + t
    iz = 1.0 / Xc[:, 2]
    x = (K[:, 0] * Xc[:, 0] + K[:, 4] * Xc[:, 1] + K[:, 1] * Xc[:, 2]) * iz
    y = (K[:, 0] * K[:, 3] * Xc[:, 1] + K[:, 2] * Xc[:, 2]) * iz
    return np.stack([x, y], axis=1), Xc[:, 2]


def distort(kc, x, y):
    """Bouguet distortion of normalised coordinates; kc (n, 5) = k1, k2, p1, p2, k3."""
    r2 = x * x + y * y
    radial = 1.0 + r2 * (kc[:, 0] + r2 * (kc[:, 1] + r2 * kc[:, 4]))
    xd = radial * x + 2.0 * kc[:, 2] * x * y + kc[:, 3] * (r2 + 2.0 * x * x)
    yd = radial * y + kc[:, 2] * (r2 + 2.0 * y * y) + 2.0 * kc[:, 3] * x * y
    return xd, yd


def project_full(K, kc, q, t, X):
    """Projection with per-row intrinsics K (n, 5) and distortion kc (n, 5) or None."""
    if kc is None:
        return project(K, q, t, X)
    R = quat_to_matrix(q)
    Xc = np.einsum("nij,nj->ni", R, X) + t
    x, y = Xc[:, 0] / Xc[:, 2], Xc[:, 1] / Xc[:, 2]
    xd, yd = distort(kc, x, y)
    u = K[:, 0] * xd + K[:, 4] * yd + K[:, 1]
    v = K[:, 0] * K[:, 3] * yd + K[:, 2]
    return np.stack([u, v], axis=1), Xc[:, 2]


def powerlaw_pmf(kmin, kmax, alpha):
    k = np.arange(kmin, kmax + 1)
    w = k.astype(np.float64) ** (-alpha)
    return k, w / w.sum()


# ---------------------------------------------------------------------------

def _finish(name, rng, K, q_true, t_true, X_true, obs_pt, obs_cam, noise_px, outlier_frac,
            rot_sigma, trans_frac, pt_frac, width, height, meta):
    C = K.shape[0]
    order = np.lexsort((obs_cam, obs_pt))
    obs_pt = obs_pt[order].astype(np.int32)
    obs_cam = obs_cam[order].astype(np.int32)
    xy, depth = project(K[obs_cam], q_true[obs_cam], t_true[obs_cam], X_true[obs_pt])
    meas = xy + rng.normal(0.0, noise_px, size=xy.shape)
    if outlier_frac > 0:
        m = rng.random(len(meas)) < outlier_frac
        meas[m, 0] = rng.uniform(0, width, size=m.sum())
        meas[m, 1] = rng.uniform(0, height, size=m.sum())
    # initial estimate: rotation perturbed into q0 (the local part v starts at 0, as the
    # reference does, main.cpp:131-136), translations and points perturbed
    dq = quat_from_rotvec(rng.normal(0.0, rot_sigma, size=(C, 3)))
    q0 = quat_mul(dq, q_true)
    q0 /= np.linalg.norm(q0, axis=1, keepdims=True)
    q0[q0[:, 0] < 0] *= -1
    tn = np.linalg.norm(t_true, axis=1, keepdims=True)
    t0 = t_true + trans_frac * tn * rng.normal(0.0, 1.0, size=t_true.shape) / np.sqrt(3.0)
    # mean depth of each point over its observations
    dsum = np.bincount(obs_pt, weights=depth, minlength=X_true.shape[0])
    dcnt = np.bincount(obs_pt, minlength=X_true.shape[0])
    dmean = dsum / np.maximum(dcnt, 1)
    X0 = X_true + pt_frac * dmean[:, None] * rng.normal(0.0, 1.0, size=X_true.shape) / np.sqrt(3.0)
    cams = np.zeros((C, 6))
    cams[:, 3:] = t0
    cams_true = np.zeros((C, 6))
    cams_true[:, 3:] = t_true
    meta = dict(meta, noise_px=noise_px, outlier_frac=outlier_frac)
    sc = Scene(name, K.copy(), q0, cams, X0, meas, obs_pt, obs_cam, cams_true, X_true.copy(),
               q_true.copy(), meta)
    sc.validate()
    return sc


def arc_scene(seed=0, n_cams=7, n_pts=500, arc_deg=30.0, k_range=None, noise_px=0.5,
              outlier_frac=0.0, rot_sigma=0.01, trans_frac=0.01, pt_frac=0.02,
              name="arc", min_views=3, fan=1.6):
    """Small scene: cameras on an arc looking outward over a 2x2x2 box 5-8 units away.

    fx = fy = 800, cx = 320, cy = 240, 640x480 frames.  A point is observed by every
    camera it projects into (k_range=None), or by a uniformly drawn number of them in
    k_range (the batched workload's 3-8 views per point)."""
    rng = np.random.default_rng(seed)
    C, P = int(n_cams), int(n_pts)
    W, H = 640.0, 480.0
    K = np.tile(np.array([800.0, 320.0, 240.0, 1.0, 0.0]), (C, 1))
    ang = np.deg2rad(np.linspace(-arc_deg / 2, arc_deg / 2, C))
    # camera centers on a unit-radius arc about the origin, optical axes fanned out past the arc
    # radii (fan x arc angle) so that the outer frames see only part of the box
    centers = np.stack([np.sin(ang), np.zeros(C), -np.cos(ang)], axis=1)
    R = np.stack([look_at(centers[j], centers[j] + np.array([np.sin(fan * a), 0.0, np.cos(fan * a)]),
                          up=(0.0, -1.0, 0.0)) for j, a in enumerate(ang)])
    q_true = quat_from_matrix(R)
    t_true = -np.einsum("nij,nj->ni", quat_to_matrix(q_true), centers)
    need = max(min_views, k_range[0] if k_range else min_views)
    Xs, opt, ocam = [], [], []
    got = 0
    R_all = quat_to_matrix(q_true)
    while got < P:
        m = min(4 * (P - got) + 16, max(4096, 4_000_000 // C))  # bounded candidate chunk
        X = np.stack([rng.uniform(-1.0, 1.0, m), rng.uniform(-1.0, 1.0, m), rng.uniform(5.0, 7.0, m)], 1)
        Xc = np.einsum("cij,mj->mci", R_all, X) + t_true[None]
        z = Xc[..., 2]
        with np.errstate(divide="ignore", invalid="ignore"):
            u = K[0, 0] * Xc[..., 0] / z + K[0, 1]
            v = K[0, 0] * K[0, 3] * Xc[..., 1] / z + K[0, 2]
        vis = (z > 0.1) & (u >= 0) & (u < W) & (v >= 0) & (v < H)
        cnt = vis.sum(1)
        keep = np.nonzero(cnt >= need)[0][: P - got]
        vis, cnt, X = vis[keep], cnt[keep], X[keep]
        if k_range is not None:
            k = np.minimum(rng.integers(k_range[0], k_range[1] + 1, size=len(keep)), cnt)
            start = (rng.random(len(keep)) * (cnt - k + 1)).astype(np.int64)
            pos = np.cumsum(vis, axis=1) - 1
            vis = vis & (pos >= start[:, None]) & (pos < (start + k)[:, None])
        rows, cols = np.nonzero(vis)
        Xs.append(X)
        opt.append(rows + got)
        ocam.append(cols)
        got += len(keep)
    X_true = np.concatenate(Xs)
    return _finish(name, rng, K, q_true, t_true, X_true, np.concatenate(opt), np.concatenate(ocam),
                   noise_px, outlier_frac, rot_sigma, trans_frac, pt_frac, W, H,
                   {"seed": seed, "generator": "arc", "k_range": k_range})


def circle_scene(seed=0, n_cams=88, n_pts=64298, radius=200.0, volume=(300.0, 300.0, 50.0),
                 kmin=2, kmax=40, alpha=1.835, noise_px=1.0, outlier_frac=0.02, rot_sigma=0.01,
                 trans_frac=0.01, pt_frac=0.02, name="circle", chunk=8192):
    """Large scene: cameras on a circle around a point volume, power-law views per point.

    Every point draws k from a truncated discrete power law on [kmin, kmax] and is
    observed by the k cameras nearest (in angle) to a random camera that sees it
    in-frame; pixel noise N(0, noise_px), outlier_frac of the observations replaced by
    uniform image positions."""
    rng = np.random.default_rng(seed)
    C, P = int(n_cams), int(n_pts)
    W, H = 640.0, 480.0
    K = np.tile(np.array([800.0, 320.0, 240.0, 1.0, 0.0]), (C, 1))
    phi = 2 * np.pi * np.arange(C) / C
    centers = np.stack([radius * np.cos(phi), radius * np.sin(phi), np.full(C, 30.0)], 1)
    R = np.stack([look_at(centers[j], np.array([0.0, 0.0, 0.0])) for j in range(C)])
    q_true = quat_from_matrix(R)
    t_true = -np.einsum("nij,nj->ni", quat_to_matrix(q_true), centers)
    kvals, pmf = powerlaw_pmf(kmin, kmax, alpha)
    pts, opt, ocam = [], [], []
    got = 0
    while got < P:
        m = min(chunk, 2 * (P - got) + 64)
        X = np.stack([rng.uniform(-volume[0] / 2, volume[0] / 2, m),
                      rng.uniform(-volume[1] / 2, volume[1] / 2, m),
                      rng.uniform(-volume[2] / 2, volume[2] / 2, m)], 1)
        Xc = np.einsum("cij,mj->mci", quat_to_matrix(q_true), X) + t_true[None]
        z = Xc[..., 2]
        with np.errstate(divide="ignore", invalid="ignore"):
            u = 800.0 * Xc[..., 0] / z + 320.0
            v = 800.0 * Xc[..., 1] / z + 240.0
        vis = (z > 1.0) & (u >= 0) & (u < W) & (v >= 0) & (v < H)
        ks = rng.choice(kvals, size=m, p=pmf)
        for r in range(m):
            cams_r = np.nonzero(vis[r])[0]
            if len(cams_r) < kmin:
                continue
            k = min(int(ks[r]), len(cams_r))
            c0 = cams_r[int(rng.integers(0, len(cams_r)))]
            dist = np.abs(((cams_r - c0) + C // 2) % C - C // 2)
            sel = np.sort(cams_r[np.argsort(dist, kind="stable")[:k]])
            pts.append(X[r])
            opt.append(np.full(k, got))
            ocam.append(sel)
            got += 1
            if got == P:
                break
    X_true = np.array(pts)
    return _finish(name, rng, K, q_true, t_true, X_true, np.concatenate(opt), np.concatenate(ocam),
                   noise_px, outlier_frac, rot_sigma, trans_frac, pt_frac, W, H,
                   {"seed": seed, "generator": "circle", "alpha": alpha})


def small_lm_scene(seed=0):
    """7 cameras on a 30 degree arc, 500 points: the CPU-runnable plain FP64 LM case."""
    return arc_scene(seed=seed, n_cams=7, n_pts=500, name="arc7x500")


def large_lm_scene(seed=0, n_pts=64298):
    """88 cameras on a 200 m circle, 64,298 points, power-law views (mean about 6)."""
    return circle_scene(seed=seed, n_cams=88, n_pts=n_pts, name="circle88x%d" % n_pts)


def batch_scenes(n_problems=1024, seed=0, cams=(5, 30), pts=(200, 3000), views=(3, 8)):
    """Independent small problems of uneven size, one seed each."""
    rng = np.random.default_rng(seed)
    out = []
    for b in range(n_problems):
        C = int(rng.integers(cams[0], cams[1] + 1))
        P = int(rng.integers(pts[0], pts[1] + 1))
        out.append(arc_scene(seed=int(rng.integers(0, 2**31 - 1)), n_cams=C, n_pts=P,
                             arc_deg=max(30.0, 4.0 * C), k_range=views,
                             name="batch%d_%dx%d" % (b, C, P)))
    return out


def serving_scenes(n_problems=32, seed=0, cams=(5, 138), pts=(500, 60000), views=(4, 6)):
    """Requests of the serving workload: cameras and points log-uniform on the
    given ranges, 4-6 views per point, the small-scene generator with a
    per-request seed (the arc widens with the camera count, up to 160 deg)."""
    rng = np.random.default_rng(seed)
    out = []
    for b in range(n_problems):
        C = int(round(np.exp(rng.uniform(np.log(cams[0]), np.log(cams[1])))))
        P = int(round(np.exp(rng.uniform(np.log(pts[0]), np.log(pts[1])))))
        out.append(arc_scene(seed=int(rng.integers(0, 2**31 - 1)), n_cams=C, n_pts=P,
                             arc_deg=float(min(max(30.0, 2.0 * C), 160.0)), k_range=views,
                             name="serve%d_%dx%d" % (b, C, P)))
    return out


def with_intrinsics(scene, cnp, seed=0, k_off=0.05, k_sigma=0.05, p_sigma=0.001, noise_px=None,
                    outlier_frac=None):
    """The same geometry with variable intrinsics: cnp 11 optimises fx, cx, cy,
    aspect, skew per camera (true values spread around the scene's K, the
    initial estimate k_off relative off: fx, cx, cy, fy each times
    1 + N(0, k_off)); cnp 16 adds distortion k1, k2, p1, p2, k3 with true k's
    from N(0, k_sigma) and p's from N(0, p_sigma), starting at 0.  The
    observations are re-drawn from the true model with the scene's noise and
    outlier fractions."""
    assert cnp in (11, 16) and scene.cams_true is not None
    rng = np.random.default_rng(seed)
    C = scene.n_cams
    Kt = scene.K.copy()
    Kt[:, 0] *= 1.0 + 0.02 * rng.normal(size=C)
    Kt[:, 1] += 4.0 * rng.normal(size=C)
    Kt[:, 2] += 4.0 * rng.normal(size=C)
    Kt[:, 3] *= 1.0 + 0.005 * rng.normal(size=C)
    kc_t = None
    if cnp == 16:
        kc_t = np.zeros((C, 5))
        kc_t[:, [0, 1, 4]] = rng.normal(0.0, k_sigma, size=(C, 3))
        kc_t[:, [2, 3]] = rng.normal(0.0, p_sigma, size=(C, 2))
    meta = dict(scene.meta)
    noise = meta.get("noise_px", 1.0) if noise_px is None else noise_px
    out_frac = meta.get("outlier_frac", 0.0) if outlier_frac is None else outlier_frac
    j, i = scene.obs_cam, scene.obs_pt
    xy, _ = project_full(Kt[j], None if kc_t is None else kc_t[j], scene.q_true[j], scene.cams_true[j, 3:],
                         scene.pts_true[i])
    meas = xy + rng.normal(0.0, noise, size=xy.shape)
    if out_frac > 0:
        m = rng.random(len(meas)) < out_frac
        meas[m, 0] = rng.uniform(0, 640.0, size=m.sum())
        meas[m, 1] = rng.uniform(0, 480.0, size=m.sum())
    fx0 = Kt[:, 0] * (1.0 + k_off * rng.normal(size=C))
    fy0 = Kt[:, 0] * Kt[:, 3] * (1.0 + k_off * rng.normal(size=C))
    K0 = np.stack([fx0, Kt[:, 1] * (1.0 + k_off * rng.normal(size=C)),
                   Kt[:, 2] * (1.0 + k_off * rng.normal(size=C)), fy0 / fx0, Kt[:, 4]], axis=1)
    cams = np.zeros((C, cnp))
    cams[:, :6] = scene.cams
    cams[:, 6:11] = K0
    cams_true = np.zeros((C, cnp))
    cams_true[:, :6] = scene.cams_true
    cams_true[:, 6:11] = Kt
    if cnp == 16:
        cams_true[:, 11:16] = kc_t
    meta.update({"cnp": cnp, "intrinsics_seed": seed})
    sc = Scene(scene.name + "_cnp%d" % cnp, Kt, scene.q0.copy(), cams, scene.pts.copy(), meas,
               scene.obs_pt.copy(), scene.obs_cam.copy(), cams_true, scene.pts_true.copy(), scene.q_true.copy(),
               meta, cnp)
    sc.validate()
    return sc


def varcam_scene(cnp, seed=0, n_cams=52, n_pts=64053, alpha=None):
    """The variable-intrinsics workload: 52 cameras on the 200 m circle,
    64,053 points, power-law views with the exponent re-fitted for a mean of
    5.42 views per point, cnp 11 or 16."""
    if alpha is None:
        alpha = fit_powerlaw_alpha(5.42)
    base = circle_scene(seed=seed, n_cams=n_cams, n_pts=n_pts, alpha=alpha, name="circle%d" % n_cams)
    return with_intrinsics(base, cnp, seed=seed + 1000)


def fit_powerlaw_alpha(mean, kmin=2, kmax=40):
    """Exponent of the truncated power law on [kmin, kmax] with the given mean."""
    lo, hi = 0.5, 4.0
    for _ in range(60):
        a = 0.5 * (lo + hi)
        k, p = powerlaw_pmf(kmin, kmax, a)
        if (k * p).sum() > mean:
            lo = a
        else:
            hi = a
    return 0.5 * (lo + hi)


def with_covariance(scene, seed=0, sigma=(0.3, 1.5), corr=0.6):
    """The scene with a random SPD 2x2 measurement covariance per observation
    (standard deviations uniform on sigma, correlation uniform on [-corr, corr])
    in ``cov`` (O, 2, 2); the measurements are left as they are."""
    rng = np.random.default_rng(seed)
    O = scene.n_obs
    sx = rng.uniform(*sigma, size=O)
    sy = rng.uniform(*sigma, size=O)
    rho = rng.uniform(-corr, corr, size=O)
    cov = np.empty((O, 2, 2))
    cov[:, 0, 0] = sx * sx
    cov[:, 1, 1] = sy * sy
    cov[:, 0, 1] = cov[:, 1, 0] = rho * sx * sy
    sc = scene.copy()
    sc.cov = cov
    sc.name = scene.name + "_cov"
    return sc
