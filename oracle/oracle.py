"""ctypes front end of the oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
import this module; the product package never does.

Point clouds are numpy arrays of shape (n, 3); they are passed to C as SoA
float32 ``[x0..xn-1, y0.., z0..]`` (the reference's cloud2data layout,
src/cloud2data.cpp:29-46).  R is row-major 3x3, t has 3 entries
(README.md:205-214 of the reference).
"""
import ctypes
import os

import numpy as np

from . import build as _build

TRACE_STRIDE = 32
# trace record fields (see oracle_impl.h)
T_STEP, T_SCHED, T_SUM = 0, 1, 2
T_XC, T_YC, T_S, T_R, T_T, T_GAP, T_LMAX = slice(3, 6), slice(6, 9), slice(9, 18), slice(18, 27), slice(27, 30), 30, 31

_lib = None
_ref = None
_ref_gpu = None

_f = ctypes.c_float
_i = ctypes.c_int
_p = ctypes.c_void_p


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def lib():
    global _lib
    if _lib is None:
        so = _build.build_oracle()
        _lib = ctypes.CDLL(so)
        L = _lib
        L.oracle_find_rt_from_s.restype = _i
        L.oracle_find_rt_from_s.argtypes = [_p] * 8
        L.oracle_eig4.restype = None
        L.oracle_eig4.argtypes = [_p] * 3
        for sfx in ("_f64", "_f32"):
            fn = getattr(L, "oracle_emicp" + sfx)
            fn.restype = _i
            fn.argtypes = [_p, _i, _p, _i, _p, _p, _f, _f, _f, _f, _p, _i]
            fn = getattr(L, "oracle_emicp_step" + sfx)
            fn.restype = ctypes.c_double
            fn.argtypes = [_p, _i, _p, _i, _p, _p, _f, _f, _p, _p, _p, _p, _p, _p]
            fn = getattr(L, "oracle_softassign" + sfx)
            fn.restype = _i
            fn.argtypes = [_p, _i, _p, _i, _p, _p, _i, _i, _i, _f, _f, _f, _f, _p, _i]
            fn = getattr(L, "oracle_softassign_step" + sfx)
            fn.restype = ctypes.c_double
            fn.argtypes = [_p, _i, _p, _i, _p, _p, _f, _f, _i, _p, _p, _p, _p, _p, _p, _p, _p]
            fn = getattr(L, "oracle_icp" + sfx)
            fn.restype = _i
            fn.argtypes = [_p, _i, _p, _i, _p, _p, _i, _p, _p, _i]
        L.oracle_set_threads.argtypes = [_i]
        L.oracle_max_threads.restype = _i
    return _lib


def ref():
    """The reference's own emicp_cpu/findRTfromS, or None where it cannot be built."""
    global _ref
    if _ref is None:
        so = None
        try:
            so = _build.build_reference()
        except Exception:  # noqa: BLE001 -- optional
            so = None
        if so is None or not os.path.exists(so):
            return None
        os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
        _ref = ctypes.CDLL(so)
        _ref.ref_emicp_cpu.restype = _i
        _ref.ref_emicp_cpu.argtypes = [_p, _i, _p, _i, _p, _p, _f, _f, _f, _f, _i]
        _ref.ref_find_rt_from_s.restype = None
        _ref.ref_find_rt_from_s.argtypes = [_p] * 5
    return _ref


def ref_gpu():
    """The reference's own GPU code (softassign(), emicp()) run on the host
    (oracle/emu), or None where it cannot be built."""
    global _ref_gpu
    if _ref_gpu is None:
        so = None
        try:
            so = _build.build_reference_gpu()
        except Exception:  # noqa: BLE001 -- optional
            so = None
        if so is None or not os.path.exists(so):
            return None
        os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
        _ref_gpu = ctypes.CDLL(so)
        _ref_gpu.ref_softassign.restype = _i
        _ref_gpu.ref_softassign.argtypes = [_p, _i, _p, _i, _p, _p, _i, _i, _i, _f, _f, _f, _f, _p, _i, _i]
        _ref_gpu.ref_emicp_gpu.restype = _i
        _ref_gpu.ref_emicp_gpu.argtypes = [_p, _i, _p, _i, _p, _p, _f, _f, _f, _f, _p, _i, _i]
    return _ref_gpu


def set_threads(n):
    lib().oracle_set_threads(int(n))


def max_threads():
    return lib().oracle_max_threads()


def soa(P):
    P = np.asarray(P, dtype=np.float32)
    assert P.ndim == 2 and P.shape[1] == 3
    return np.ascontiguousarray(P.T).reshape(-1)


def _dt(precision):
    return (np.float64, "_f64") if precision == "f64" else (np.float32, "_f32")


def find_rt_from_s(Xc, Yc, S, q_prev=None):
    """Horn's pose (FP64). S in the reference's h_S layout (9 values)."""
    Xc = np.ascontiguousarray(Xc, dtype=np.float64)
    Yc = np.ascontiguousarray(Yc, dtype=np.float64)
    S = np.ascontiguousarray(np.asarray(S, dtype=np.float64).reshape(-1))
    R = np.zeros(9)
    t = np.zeros(3)
    qp = np.array([1.0, 0, 0, 0]) if q_prev is None else np.ascontiguousarray(q_prev, dtype=np.float64)
    gap = np.zeros(1)
    lmax = np.zeros(1)
    used_prev = lib().oracle_find_rt_from_s(_ptr(Xc), _ptr(Yc), _ptr(S), _ptr(R), _ptr(t), _ptr(qp),
                                            _ptr(gap), _ptr(lmax))
    return R.reshape(3, 3), t, dict(q=qp, gap=gap[0], lmax=lmax[0], used_prev=bool(used_prev))


def eig4(N):
    N = np.asfortranarray(np.asarray(N, dtype=np.float64).reshape(4, 4))
    vals = np.zeros(4)
    vecs = np.zeros(16)
    lib().oracle_eig4(_ptr(np.ascontiguousarray(N.reshape(-1, order="F"))), _ptr(vals), _ptr(vecs))
    return vals, vecs.reshape(4, 4, order="F")


def emicp(X, Y, R0=None, t0=None, sigma_p2=0.01, sigma_inf=1e-5, sigma_factor=0.9, d_02=0.01,
          precision="f64", trace=True, max_steps=100000):
    """Annealed EM-ICP (src/emicp_cpu.cpp:186-547). Returns (R, t, trace[steps, 32])."""
    dt, sfx = _dt(precision)
    Xs, Ys = soa(X), soa(Y)
    R = np.ascontiguousarray(np.eye(3) if R0 is None else R0, dtype=dt).reshape(-1).copy()
    t = np.ascontiguousarray(np.zeros(3) if t0 is None else t0, dtype=dt).reshape(-1).copy()
    tr = np.zeros((max_steps if trace else 0, TRACE_STRIDE))
    n = getattr(lib(), "oracle_emicp" + sfx)(_ptr(Xs), len(X), _ptr(Ys), len(Y), _ptr(R), _ptr(t),
                                            sigma_p2, sigma_inf, sigma_factor, d_02,
                                            _ptr(tr) if trace else None, tr.shape[0])
    if n < 0:
        raise ValueError("oracle_emicp: invalid arguments")
    return R.reshape(3, 3).astype(np.float64), t.astype(np.float64), tr[: min(n, tr.shape[0])]


def emicp_step(X, Y, R, t, sigma_p2, d_02, precision="f64"):
    """One EM-ICP E-step + moments. Returns dict with C, lam, U (M x 3), Xc, Yc, S, sum."""
    dt, sfx = _dt(precision)
    Xs, Ys = soa(X), soa(Y)
    M = len(Y)
    R = np.ascontiguousarray(R, dtype=dt).reshape(-1)
    t = np.ascontiguousarray(t, dtype=dt).reshape(-1)
    C = np.zeros(M, dt)
    lam = np.zeros(M, dt)
    U = np.zeros(3 * M, dt)
    Xc, Yc, S = np.zeros(3, dt), np.zeros(3, dt), np.zeros(9, dt)
    s = getattr(lib(), "oracle_emicp_step" + sfx)(_ptr(Xs), len(X), _ptr(Ys), M, _ptr(R), _ptr(t),
                                                 sigma_p2, d_02, _ptr(C), _ptr(lam), _ptr(U),
                                                 _ptr(Xc), _ptr(Yc), _ptr(S))
    return dict(C=C, lam=lam, U=U.reshape(M, 3), Xc=Xc, Yc=Yc, S=S, sum=s)


def softassign(X, Y, R0=None, t0=None, JMAX=100, I0=5, I1=3, alpha=3.0, T_0=100.0, TFACTOR=0.95,
               moutlier=None, precision="f64", trace=True):
    """Annealed Softassign (src/softassign.cu:256-886). Returns (R, t, trace)."""
    dt, sfx = _dt(precision)
    if moutlier is None:
        moutlier = float(np.float32(1.0 / np.sqrt(np.float32(T_0)) * np.exp(np.float32(-1.0))))
    Xs, Ys = soa(X), soa(Y)
    R = np.ascontiguousarray(np.eye(3) if R0 is None else R0, dtype=dt).reshape(-1).copy()
    t = np.ascontiguousarray(np.zeros(3) if t0 is None else t0, dtype=dt).reshape(-1).copy()
    cap = max(JMAX * I0, 1)
    tr = np.zeros((cap if trace else 0, TRACE_STRIDE))
    n = getattr(lib(), "oracle_softassign" + sfx)(_ptr(Xs), len(X), _ptr(Ys), len(Y), _ptr(R), _ptr(t),
                                                 JMAX, I0, I1, alpha, T_0, TFACTOR, moutlier,
                                                 _ptr(tr) if trace else None, tr.shape[0])
    if n < 0:
        raise ValueError("oracle_softassign: invalid arguments")
    return R.reshape(3, 3).astype(np.float64), t.astype(np.float64), tr[: min(n, tr.shape[0])]


def softassign_step(X, Y, R, t, T, alpha, I1, s, u, precision="f64"):
    """One Softassign inner iteration; s (N) and u (M) slack are updated in place copies."""
    dt, sfx = _dt(precision)
    Xs, Ys = soa(X), soa(Y)
    N, M = len(X), len(Y)
    R = np.ascontiguousarray(R, dtype=dt).reshape(-1)
    t = np.ascontiguousarray(t, dtype=dt).reshape(-1)
    s = np.array(s, dtype=dt).reshape(-1).copy()
    u = np.array(u, dtype=dt).reshape(-1).copy()
    rs, cs, w = np.zeros(N, dt), np.zeros(M, dt), np.zeros(N, dt)
    Xc, Yc, S = np.zeros(3, dt), np.zeros(3, dt), np.zeros(9, dt)
    sm = getattr(lib(), "oracle_softassign_step" + sfx)(_ptr(Xs), N, _ptr(Ys), M, _ptr(R), _ptr(t), T,
                                                       alpha, I1, _ptr(s), _ptr(u), _ptr(rs), _ptr(cs),
                                                       _ptr(w), _ptr(Xc), _ptr(Yc), _ptr(S))
    return dict(s=s, u=u, rs=rs, cs=cs, w=w, Xc=Xc, Yc=Yc, S=S, sum=sm)


def icp(X, Y, R0=None, t0=None, maxIteration=30, precision="f64", trace=True):
    """ICP with exhaustive nearest neighbours (src/icp.cpp:122-290; the
    reference's FLANN search is approximate). Returns (R, t, trace, nn) with
    nn the matches of the last iteration."""
    dt, sfx = _dt(precision)
    Xs, Ys = soa(X), soa(Y)
    R = np.ascontiguousarray(np.eye(3) if R0 is None else R0, dtype=dt).reshape(-1).copy()
    t = np.ascontiguousarray(np.zeros(3) if t0 is None else t0, dtype=dt).reshape(-1).copy()
    tr = np.zeros((max(maxIteration, 1) if trace else 0, TRACE_STRIDE))
    nn = np.zeros(len(Y), np.int32)
    n = getattr(lib(), "oracle_icp" + sfx)(_ptr(Xs), len(X), _ptr(Ys), len(Y), _ptr(R), _ptr(t), maxIteration,
                                          _ptr(nn), _ptr(tr) if trace else None, tr.shape[0])
    if n < 0:
        raise ValueError("oracle_icp: invalid arguments")
    return R.reshape(3, 3).astype(np.float64), t.astype(np.float64), tr[: min(n, tr.shape[0])], nn


def ref_emicp_cpu(X, Y, R0=None, t0=None, sigma_p2=0.01, sigma_inf=1e-5, sigma_factor=0.9, d_02=0.01):
    """The reference's own emicp_cpu() (FP32 + OpenBLAS). Returns (R, t) or None."""
    L = ref()
    if L is None:
        return None
    Xs, Ys = soa(X), soa(Y)
    R = np.ascontiguousarray(np.eye(3) if R0 is None else R0, dtype=np.float32).reshape(-1).copy()
    t = np.ascontiguousarray(np.zeros(3) if t0 is None else t0, dtype=np.float32).reshape(-1).copy()
    L.ref_emicp_cpu(_ptr(Xs), len(X), _ptr(Ys), len(Y), _ptr(R), _ptr(t), sigma_p2, sigma_inf,
                    sigma_factor, d_02, 1)
    return R.reshape(3, 3).astype(np.float64), t.astype(np.float64)


def ref_find_rt_from_s(Xc, Yc, S):
    """The reference's own findRTfromS() (dsyev_). Returns (R, t) or None."""
    L = ref()
    if L is None:
        return None
    Xc = np.ascontiguousarray(Xc, dtype=np.float32)
    Yc = np.ascontiguousarray(Yc, dtype=np.float32)
    S = np.ascontiguousarray(np.asarray(S, dtype=np.float32).reshape(-1))
    R = np.zeros(9, np.float32)
    t = np.zeros(3, np.float32)
    L.ref_find_rt_from_s(_ptr(Xc), _ptr(Yc), _ptr(S), _ptr(R), _ptr(t))
    return R.reshape(3, 3).astype(np.float64), t.astype(np.float64)


def ref_softassign(X, Y, R0=None, t0=None, JMAX=100, I0=5, I1=3, alpha=3.0, T_0=100.0, TFACTOR=0.95,
                   moutlier=None):
    """The reference's own softassign() (src/softassign.cu:256-886; its CUDA
    kernels and cuBLAS calls run on the host by oracle/emu). Returns (R, t,
    trace) with the reference's own per-update record (Xc, Yc, S, R, t, as
    passed to and returned by its findRTfromS), or None where unavailable."""
    L = ref_gpu()
    if L is None:
        return None
    if moutlier is None:
        moutlier = float(np.float32(1.0 / np.sqrt(np.float32(T_0)) * np.exp(np.float32(-1.0))))
    Xs, Ys = soa(X), soa(Y)
    R = np.ascontiguousarray(np.eye(3) if R0 is None else R0, dtype=np.float32).reshape(-1).copy()
    t = np.ascontiguousarray(np.zeros(3) if t0 is None else t0, dtype=np.float32).reshape(-1).copy()
    cap = max(JMAX * I0, 1)
    tr = np.zeros((cap, TRACE_STRIDE))
    n = L.ref_softassign(_ptr(Xs), len(X), _ptr(Ys), len(Y), _ptr(R), _ptr(t), JMAX, I0, I1, alpha, T_0, TFACTOR,
                         moutlier, _ptr(tr), cap, 1)
    # the record's schedule field: T of each update (T_0 * TFACTOR^j in FP32, src/softassign.cu:820)
    T = np.float32(T_0)
    for j in range(JMAX):
        for i in range(I0):
            if j * I0 + i < cap:
                tr[j * I0 + i, 1] = float(T)
        T = np.float32(T * np.float32(TFACTOR))
    return R.reshape(3, 3).astype(np.float64), t.astype(np.float64), tr[: min(n, cap)]


def ref_emicp_gpu(X, Y, R0=None, t0=None, sigma_p2=0.01, sigma_inf=1e-5, sigma_factor=0.9, d_02=0.01):
    """The reference's own GPU emicp() (src/emicp.cu:247-716; its CUDA kernels
    and cuBLAS calls run on the host by oracle/emu). Returns (R, t, trace)
    with the reference's own per-step record, or None where unavailable."""
    L = ref_gpu()
    if L is None:
        return None
    Xs, Ys = soa(X), soa(Y)
    R = np.ascontiguousarray(np.eye(3) if R0 is None else R0, dtype=np.float32).reshape(-1).copy()
    t = np.ascontiguousarray(np.zeros(3) if t0 is None else t0, dtype=np.float32).reshape(-1).copy()
    sig = []
    s = np.float32(sigma_p2)
    while s > np.float32(sigma_inf):
        sig.append(float(s))
        s = np.float32(s * np.float32(sigma_factor))
    cap = max(len(sig), 1)
    tr = np.zeros((cap, TRACE_STRIDE))
    n = L.ref_emicp_gpu(_ptr(Xs), len(X), _ptr(Ys), len(Y), _ptr(R), _ptr(t), sigma_p2, sigma_inf, sigma_factor,
                        d_02, _ptr(tr), cap, 1)
    tr[: len(sig), 1] = sig
    return R.reshape(3, 3).astype(np.float64), t.astype(np.float64), tr[: min(n, cap)]
