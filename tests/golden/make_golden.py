"""Regenerate the golden fixtures from the reference's own kernels.

Runs the reference's OpenCL kernels and CPU Jacobian (compiled for the CPU by
oracle/build.py from the reference checkout, see oracle/ref_shim.cpp) on a
small seeded scene and stores every stage's output.  The tests compare the
oracle (and through it the GPU path) against these arrays on machines where
the reference sources are absent.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle.ref as ref  # noqa: E402
from psba_gb300 import scenes  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_arc7.npz")


def main():
    if not ref.available():
        raise SystemExit("reference sources not available here")
    sc = scenes.arc_scene(seed=11, n_cams=7, n_pts=60, name="golden")
    rng = np.random.default_rng(5)
    cams = sc.cams.copy()
    cams[:, :3] = rng.normal(0.0, 0.01, size=(sc.n_cams, 3))  # nonzero local rotations
    pts = sc.pts
    ex = ref.compute_exQT(sc, cams, pts)
    JA, JB = ref.compute_jacobiQT(sc, cams, pts)
    out = dict(K=sc.K, q0=sc.q0, meas=sc.meas, obs_pt=sc.obs_pt, obs_cam=sc.obs_cam, cams=cams, pts=pts,
               ex=ex, JA=JA, JB=JB)
    for tag, coeff in (("c1", 1.0), ("c2", 2.0), ("cm2", -2.0)):
        U, V, W, g, d = ref.normal_blocks(sc, JA, JB, ex, coeff)
        out.update({"U_" + tag: U, "V_" + tag: V, "W_" + tag: W, "g_" + tag: g, "uvdiag_" + tag: d})
    U, V, W, g, d = ref.normal_blocks(sc, JA, JB, ex, 1.0)
    mu = 1e-3 * d.max()
    Vinv, Y, S, ea = ref.trial(sc, U, V, W, g, mu)
    out.update(mu=np.array(mu), Vinv=Vinv, Y=Y, S=S, ea=ea)
    # reduced-camera solve with the reference's matVec_mul on numpy's inverse of
    # the (lower-defined) S, then its compute_eb / compute_dpb
    Sl = np.tril(S)
    Sfull = Sl + np.tril(Sl, -1).T
    Sinv = np.linalg.inv(Sfull)
    dpa = ref.matvec(Sinv, ea)
    Vstore = V.copy()
    for i in range(sc.n_pts):
        for r in range(3):
            for c in range(r + 1):
                Vstore[i, r, c] = Vinv[i, r, c]
    eb, dpb = ref.back_substitute(sc, W, Vstore, g, dpa)
    out.update(Sinv=Sinv, dpa=dpa, eb=eb, dpb=dpb)
    x = rng.normal(size=6 * sc.n_cams + 3 * sc.n_pts)
    jx = ref.jmultiply(sc, JA, JB, x)
    out.update(jx_in=x, jx_dense=jx)
    # CPU Jacobian of PSBA/levmar_func_cpu.cpp for the first observations
    cpuA, cpuB = [], []
    for o in range(8):
        j, i = sc.obs_cam[o], sc.obs_pt[o]
        A, B = ref.calc_img_proj_jac(sc.K[j], sc.q0[j], cams[j, :3], cams[j, 3:], pts[i])
        cpuA.append(A)
        cpuB.append(B)
    out.update(cpu_JA=np.array(cpuA), cpu_JB=np.array(cpuB))
    np.savez_compressed(OUT, **out)
    print(OUT, os.path.getsize(OUT), "bytes", sc.n_obs, "observations")


if __name__ == "__main__":
    main()
