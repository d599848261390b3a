"""Binding of the reference's own kernels compiled for the CPU (oracle/_ref).

TEST INFRASTRUCTURE ONLY.  ``build.build_ref()`` compiles the reference's
barrier-free OpenCL kernels and ``PSBA/levmar_func_cpu.cpp`` where they lie;
this module runs them with the reference's dense index tables so that the
oracle's restatement can be compared with the reference's arithmetic, and so
that golden fixtures can be generated.  It is unavailable where the
reference checkout is absent (the GPU machine): tests that need it skip there and
use the committed fixtures instead.
"""
import ctypes as C

import numpy as np

from . import build as _build

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_lib = None


def available():
    return _build.reference_available()


def lib():
    global _lib
    if _lib is None:
        path = _build.build_ref()
        if path is None:
            raise RuntimeError("reference sources are not available on this machine")
        _lib = C.CDLL(path)
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class DenseIndex:
    """The reference's index tables (generate_idxs, PSBA/misc.cpp:178-218):
    iidx/jidx per observation, blk_idx[P*C] (observation or -1) and the
    common-point table comm3DIdx[C*C*P] with counts comm3DIdxCnt[C*C]."""

    def __init__(self, scene, with_common=True):
        C_, P = scene.n_cams, scene.n_pts
        self.iidx = np.ascontiguousarray(scene.obs_pt, dtype=np.int32)
        self.jidx = np.ascontiguousarray(scene.obs_cam, dtype=np.int32)
        blk = -np.ones(P * C_, dtype=np.int32)
        blk[self.iidx.astype(np.int64) * C_ + self.jidx] = np.arange(scene.n_obs, dtype=np.int32)
        self.blk = blk
        if with_common:
            cnt = np.zeros(C_ * C_, dtype=np.int32)
            com = np.zeros(C_ * C_ * P, dtype=np.int32)
            starts = np.searchsorted(self.iidx, np.arange(P + 1))
            for i in range(P):
                cams = self.jidx[starts[i]:starts[i + 1]]
                for j in cams:
                    for k in cams:
                        if k <= j:
                            t = cnt[j * C_ + k]
                            cnt[j * C_ + k] += 1
                            com[j * C_ * P + k * P + t] = i
                            if k != j:
                                cnt[k * C_ + j] += 1
                                com[k * C_ * P + j * P + t] = i
            self.cnt = cnt
            self.com = com


def compute_exQT(scene, cams, pts):
    ex = np.empty(2 * scene.n_obs)
    ix = DenseIndex(scene, with_common=False)
    lib().ref_compute_exQT(C.c_int(scene.n_obs), _d(_f(scene.K)), _d(_f(scene.meas)), _d(_f(scene.q0)),
                           _d(_f(cams)), _d(_f(pts)), _i(ix.iidx), _i(ix.jidx), _d(ex))
    return ex.reshape(-1, 2)


def compute_jacobiQT(scene, cams, pts):
    JA = np.empty((scene.n_obs, 2, 6))
    JB = np.empty((scene.n_obs, 2, 3))
    ix = DenseIndex(scene, with_common=False)
    lib().ref_compute_jacobiQT(C.c_int(scene.n_obs), _d(_f(scene.K)), _d(_f(scene.meas)),
                               _d(_f(scene.q0)), _d(_f(cams)), _d(_f(pts)), _i(ix.iidx), _i(ix.jidx),
                               _d(JA), _d(JB))
    return JA, JB


def calc_img_proj_jac(K5, q0, v, t, M):
    """PSBA/levmar_func_cpu.cpp:227 calcImgProjJacRTS for one camera/point."""
    A = np.empty((2, 6))
    B = np.empty((2, 3))
    lib().ref_calcImgProjJacRTS(_d(_f(K5)), _d(_f(q0)), _d(_f(v)), _d(_f(t)), _d(_f(M)), _d(A), _d(B))
    return A, B


def normal_blocks(scene, JA, JB, ex, coeff):
    C_, P, O = scene.n_cams, scene.n_pts, scene.n_obs
    ix = DenseIndex(scene, with_common=False)
    U = np.empty((C_, 6, 6))
    V = np.empty((P, 3, 3))
    W = np.empty((O, 6, 3))
    g = np.empty(6 * C_ + 3 * P)
    d = np.empty(6 * C_ + 3 * P)
    JA, JB, ex = _f(JA), _f(JB), _f(ex)
    L = lib()
    L.ref_compute_U(C_, P, O, _d(JA), _i(ix.blk), _d(U), _d(d), C.c_double(coeff))
    L.ref_compute_V(C_, P, O, _d(JB), _i(ix.blk), _d(V), _d(d), C.c_double(coeff))
    L.ref_compute_Wblks(C_, P, O, _d(JA), _d(JB), _i(ix.iidx), _i(ix.jidx), _d(W), C.c_double(coeff))
    L.ref_compute_g(C_, P, O, C.c_double(coeff), _d(JA), _d(JB), _i(ix.blk), _d(ex), _d(g))
    return U, V, W, g, d


def trial(scene, U, V, W, g, mu):
    """One damping trial of levmar.cpp:126-131 on the reference kernels:
    update_UV, compute_Vinv, compute_Yblks, compute_S, compute_ea.
    Returns the symmetric V^-1 (from its lower storage), Y, S (full) and ea."""
    C_, P, O = scene.n_cams, scene.n_pts, scene.n_obs
    ix = DenseIndex(scene, with_common=True)
    U = _f(U).copy()
    V = _f(V).copy()
    W = _f(W)
    g = _f(g)
    L = lib()
    L.ref_update_UV(C_, P, _d(U), _d(V), C.c_double(mu))
    ret = np.zeros(1)
    L.ref_compute_Vinv(P, _d(V), _d(ret))
    Y = np.empty((O, 6, 3))
    L.ref_compute_Yblks(C_, P, O, _i(ix.iidx), _d(W), _d(V), _d(Y))
    N = 6 * C_
    S = np.empty((N, N))
    L.ref_compute_S(C_, P, _i(ix.blk), _d(U), _d(Y), _d(W), _i(ix.com), _i(ix.cnt), _d(S))
    ea = np.empty(N)
    L.ref_compute_ea(C_, P, O, _i(ix.blk), _d(Y), _d(g), _d(ea))
    Vl = V.reshape(P, 3, 3)
    Vinv = np.tril(Vl) + np.transpose(np.tril(Vl, -1), (0, 2, 1))
    return Vinv, Y, S, ea


def back_substitute(scene, W, Vstore, g, dpa):
    """compute_eb + compute_dpb (sba_func.cpp:1001-1117) given dpa.  Vstore is
    the reference's V buffer after compute_Vinv (V^-1 in its lower triangle)."""
    C_, P, O = scene.n_cams, scene.n_pts, scene.n_obs
    ix = DenseIndex(scene, with_common=False)
    nt = 6 * C_ + 3 * P
    dp = np.zeros(nt)
    dp[:6 * C_] = dpa
    eab = np.zeros(nt)
    L = lib()
    L.ref_compute_eb(C_, P, O, _i(ix.blk), _d(_f(W)), _d(dp), _d(_f(g)), _d(eab))
    L.ref_compute_dpb(C_, P, _d(_f(Vstore)), _d(eab), _d(dp))
    return eab[6 * C_:], dp[6 * C_:]


def jmultiply(scene, JA, JB, x):
    """Dense J x over the (point, camera) grid, compute_Jmultiply.cl."""
    C_, P, O = scene.n_cams, scene.n_pts, scene.n_obs
    ix = DenseIndex(scene, with_common=False)
    out = np.empty(2 * C_ * P)
    lib().ref_compute_Jmultiply(C_, P, O, _d(_f(JA)), _d(_f(JB)), _i(ix.blk), _d(_f(x)), _d(out))
    return out


def matvec(M, v):
    M = _f(M)
    out = np.empty(M.shape[0])
    lib().ref_matVec_mul(M.shape[0], _d(M), _d(_f(v)), _d(out))
    return out


# ---------------------------------------------------------------- the reader

_reader = None


def reader_available():
    return _build.build_ref_reader() is not None


def read_sba(cams_path, pts_path, cnp=11, filecnp=12):
    """readInitialSBAEstimate (PSBA/readparams.cpp:444-519) with quat2vec as
    its input filter, compiled from the reference: returns (motstruct
    (ncams * cnp + npts * 3), initrot (4 per camera), imgpts (2 per
    projection, file order), cov (4 per projection) or None, vmask (npts x
    ncams)), the arrays as the reference's main() receives them
    (PSBA/main.cpp:102-110)."""
    global _reader
    if _reader is None:
        path = _build.build_ref_reader()
        if path is None:
            raise RuntimeError("reference sources are not available on this machine")
        _reader = C.CDLL(path)
        _reader.ref_read_sba.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_int, _ip, _ip, _ip,
                                         C.POINTER(_dp), C.POINTER(_dp), C.POINTER(_dp), C.POINTER(_dp),
                                         C.POINTER(C.POINTER(C.c_char))]
        _reader.ref_reader_free.argtypes = [C.c_void_p]
    nc, npt, npr = C.c_int(), C.c_int(), C.c_int()
    ms, ir, ip, cv = _dp(), _dp(), _dp(), _dp()
    vm = C.POINTER(C.c_char)()
    _reader.ref_read_sba(str(cams_path).encode(), str(pts_path).encode(), cnp, filecnp, C.byref(nc), C.byref(npt),
                         C.byref(npr), C.byref(ms), C.byref(ir), C.byref(ip), C.byref(cv), C.byref(vm))
    n_ms = nc.value * cnp + npt.value * 3
    out = (np.ctypeslib.as_array(ms, (n_ms,)).copy(), np.ctypeslib.as_array(ir, (4 * nc.value,)).copy(),
           np.ctypeslib.as_array(ip, (2 * npr.value,)).copy(),
           np.ctypeslib.as_array(cv, (4 * npr.value,)).copy() if cv else None,
           np.frombuffer(C.string_at(vm, npt.value * nc.value), dtype=np.int8).reshape(npt.value, nc.value).copy())
    for p in (ms, ir, ip, cv):
        if p:
            _reader.ref_reader_free(C.cast(p, C.c_void_p))
    _reader.ref_reader_free(C.cast(vm, C.c_void_p))
    return out
