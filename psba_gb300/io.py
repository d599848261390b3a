"""Problems in the reference's text format (the sba camera / point files).

Camera file: one camera per line, ``#`` comments; 7 fields (quaternion s,
v1, v2, v3 and translation), 12 fields (K = fu, u0, v0, aspect, skew first)
or 17 fields (K, five distortion terms, quaternion, translation) --
``data/7cams.txt``, ``data/*camsvarK.txt``, ``data/54camsvarKD.txt`` of the
reference.  Point file: ``X Y Z nframes frame0 x0 y0 [cov0] frame1 x1 y1
[cov1] ...`` where a projection's covariance, when present, is the full 2x2
(4 values, row-major) or its upper triangle (3 values), detected from the
first line as the reference's reader does (PSBA/readparams.cpp:237-283).

The reading follows readInitialSBAEstimate (PSBA/readparams.cpp:444-519)
with quat2vec (PSBA/misc.cpp:21-49) as the input filter and the split of
PSBA/main.cpp:131-149: each file quaternion is normalised with a
non-negative scalar part, becomes the camera's initial rotation q0, and the
local rotation vector starts at 0; K (and distortion) are split off.  Unlike
the reference's reader (which assumes it), frames need not be listed in
ascending camera order: observations are sorted by (point, camera), and a
repeated (point, camera) pair is an error.  Nothing here calls exit(): bad
input raises ValueError.
"""
import numpy as np

from .scenes import Scene, quat_mul

__all__ = ["read_cameras", "read_points", "load_scene", "write_scene"]


def _lines(path):
    with open(path) as f:
        for ln in f:
            s = ln.strip()
            if s and not s.startswith("#"):
                yield s


def read_cameras(path):
    """(C, F) array of the camera lines; F is 7, 12 or 17."""
    rows = [[float(v) for v in s.split()] for s in _lines(path)]
    if not rows:
        raise ValueError("%s: no cameras" % path)
    F = len(rows[0])
    if F not in (7, 12, 17):
        raise ValueError("%s: %d fields per camera (expected 7, 12 or 17)" % (path, F))
    for k, r in enumerate(rows):
        if len(r) != F:
            raise ValueError("%s: camera %d has %d fields, the first has %d" % (path, k, len(r), F))
    return np.array(rows)


def read_points(path, n_cams=None):
    """Points (P, 3), observations (point, camera, x, y) in file order and the
    per-observation 2x2 covariances (O, 2, 2) or None."""
    pts, obs, cov = [], [], []
    cov_len = None
    for p, s in enumerate(_lines(path)):
        v = s.split()
        if len(v) < 4:
            raise ValueError("%s: point %d: short line" % (path, p))
        X = [float(a) for a in v[:3]]
        nf = int(v[3])
        rest = v[4:]
        if cov_len is None:
            if nf <= 0 or len(rest) % nf:
                raise ValueError("%s: point %d: %d values for %d frames" % (path, p, len(rest), nf))
            per = len(rest) // nf
            if per not in (3, 6, 7):
                raise ValueError("%s: point %d: %d values per projection (3, 6 or 7)" % (path, p, per))
            cov_len = per - 3
        per = 3 + cov_len
        if len(rest) != nf * per:
            raise ValueError("%s: point %d: %d values for %d frames of %d" % (path, p, len(rest), nf, per))
        pts.append(X)
        for f in range(nf):
            q = rest[f * per:(f + 1) * per]
            cam = int(q[0])
            if cam < 0 or (n_cams is not None and cam >= n_cams):
                raise ValueError("%s: point %d: camera index %d out of range" % (path, p, cam))
            obs.append((p, cam, float(q[1]), float(q[2])))
            if cov_len == 4:
                c = [float(a) for a in q[3:7]]
                cov.append([[c[0], c[1]], [c[2], c[3]]])
            elif cov_len == 3:
                c = [float(a) for a in q[3:6]]
                cov.append([[c[0], c[1]], [c[1], c[2]]])
    return np.array(pts).reshape(-1, 3), obs, (np.array(cov) if cov_len else None)


def _quat_in(q):
    """quat2vec (PSBA/misc.cpp:33-44) then the rebuilt unit quaternion of
    readCameraParams (PSBA/readparams.cpp:221-225)."""
    mag = np.sqrt((q * q).sum(axis=1))
    sg = np.where(q[:, 0] >= 0.0, 1.0, -1.0)
    v = q[:, 1:] * (sg / mag)[:, None]
    # the reference's order of operations: 1 - v1^2 - v2^2 - v3^2
    s = np.sqrt(((1.0 - v[:, 0] * v[:, 0]) - v[:, 1] * v[:, 1]) - v[:, 2] * v[:, 2])
    return np.concatenate([s[:, None], v], axis=1)


def load_scene(cams_path, pts_path, cnp=6, K=None, name=None):
    """A Scene from the reference's files.

    cnp 6: pose only; K from the 12/17-field file, or the K argument (5
    values or (C, 5)) for 7-field files.  cnp 11: the file's K is the
    initial estimate of per-camera intrinsics.  cnp 16: also the distortion
    (zero when the file has none).  The scene's ``cov`` attribute holds the
    observation covariances (or None)."""
    camf = read_cameras(cams_path)
    C, F = camf.shape
    pts, obs, cov = read_points(pts_path, n_cams=C)
    if F == 7:
        if cnp != 6 and K is None:
            raise ValueError("7-field camera file: intrinsics must be given (K=...)")
        Kf = None if K is None else np.broadcast_to(np.asarray(K, dtype=np.float64), (C, 5)).copy()
        kc = np.zeros((C, 5))
        qt = camf
    else:
        Kf = camf[:, :5].copy()
        kc = camf[:, 5:10].copy() if F == 17 else np.zeros((C, 5))
        qt = camf[:, F - 7:]
    if Kf is None:
        raise ValueError("no intrinsics: the camera file has none and K was not given")
    if cnp not in (6, 11, 16):
        raise ValueError("cnp must be 6, 11 or 16")
    q0 = _quat_in(qt[:, :4])
    t = qt[:, 4:7]
    arr = np.array(obs, dtype=np.float64).reshape(-1, 4)
    opt, ocam = arr[:, 0].astype(np.int64), arr[:, 1].astype(np.int64)
    order = np.lexsort((ocam, opt))
    key = opt[order] * C + ocam[order]
    if len(key) > 1 and np.any(np.diff(key) == 0):
        raise ValueError("%s: a point is observed twice by the same camera" % pts_path)
    meas = arr[order, 2:4].copy()
    cams = np.zeros((C, cnp))
    cams[:, 3:6] = t
    if cnp >= 11:
        cams[:, 6:11] = Kf
    if cnp == 16:
        cams[:, 11:16] = kc
    sc = Scene(name or str(cams_path), Kf, q0, cams, pts, meas, opt[order].astype(np.int32),
               ocam[order].astype(np.int32), meta={"source": (str(cams_path), str(pts_path))}, cnp=cnp)
    sc.cov = None if cov is None else cov[order]
    sc.validate()
    return sc


def write_scene(cams_path, pts_path, scene, cams=None, pts=None, cov=None):
    """Write a Scene (optionally with other parameters, e.g. a solution) in
    the reference's format: 12 fields per camera (17 for cnp 16), the
    rotation written as the composed quaternion q(v) (x) q0."""
    cams = scene.cams if cams is None else np.asarray(cams)
    pts = scene.pts if pts is None else np.asarray(pts)
    C = scene.n_cams
    v = cams[:, :3]
    s = np.sqrt(1.0 - (v * v).sum(axis=1))
    q = quat_mul(np.concatenate([s[:, None], v], axis=1), scene.q0)
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    q[q[:, 0] < 0] *= -1
    K = cams[:, 6:11] if scene.cnp >= 11 else scene.K
    with open(cams_path, "w") as f:
        if scene.cnp == 16:
            f.write("# fu, u0, v0, ar, s   kc(1:5)   quaternion translation\n")
        else:
            f.write("# fu, u0, v0, ar, s   quaternion translation\n")
        for j in range(C):
            vals = list(K[j])
            if scene.cnp == 16:
                vals += list(cams[j, 11:16])
            vals += list(q[j]) + list(cams[j, 3:6])
            f.write(" ".join("%.17g" % x for x in vals) + "\n")
    starts = np.searchsorted(scene.obs_pt, np.arange(scene.n_pts + 1))
    with open(pts_path, "w") as f:
        f.write("# X Y Z  nframes  frame0 x0 y0%s  frame1 x1 y1 ...\n" % (" covx0^2 covx0y0 covx0y0 covy0^2"
                                                                         if cov is not None else ""))
        for i in range(scene.n_pts):
            a, b = starts[i], starts[i + 1]
            parts = ["%.17g %.17g %.17g" % tuple(pts[i]), str(b - a)]
            for o in range(a, b):
                parts.append("%d %.17g %.17g" % (scene.obs_cam[o], scene.meas[o, 0], scene.meas[o, 1]))
                if cov is not None:
                    parts.append(" ".join("%.17g" % x for x in np.asarray(cov[o]).ravel()))
            f.write(" ".join(parts) + "\n")
