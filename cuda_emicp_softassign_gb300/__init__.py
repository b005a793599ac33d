"""GB300-native soft-correspondence rigid registration (EM-ICP and Softassign).

Python mirror of the reference's registration API (src/3dregistration.h:39-99):
``emicp(X, Y, R, t, param)`` and ``softassign(X, Y, R, t, param)`` align point
set Y (source) to X (target) so that X ~ R Y + t. Both run the sm_103a kernels
of ``libcesa.so`` through its C ABI (include/cesa.h). There is no CPU path: if
the library is missing or no GPU is present, the calls raise.

Point clouds are ``(n, 3)`` float arrays. R is 3x3 (row-major when flattened),
t has 3 entries.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libcesa.so")

CESA_OK = 0
CESA_ERR_INVALID_ARGUMENT = 1
CESA_ERR_CUDA = 2
CESA_ERR_TIMEOUT = 3
CESA_ERR_NO_DEVICE = 4
CESA_ERR_OUT_OF_MEMORY = 5
CESA_ERR_UNSUPPORTED = 6
CESA_ERR_NOALLOC_LIMIT = 7
CESA_ERR_INTERNAL = 8

LAYOUT_AUTO = 0
LAYOUT_SLICES = 1
LAYOUT_RANGED = 2
SA_BACKWARD_AUTO = 0
SA_BACKWARD_PERSISTENT = 1
SA_BACKWARD_LAUNCHES = 2
SINKHORN_AUTO = 0
SINKHORN_MATRIX_FREE = 1
SINKHORN_MATERIALISED = 2
SINKHORN_BANDED = 3
ICP_SEARCH_AUTO = 0
ICP_SEARCH_EXHAUSTIVE = 1
ICP_SEARCH_GRID = 2
POINTS_BY_NAME = 0
POINTS_PCD = 1
POINTS_PLY = 2
POINTS_TEXT = 3

TRACE_STRIDE = 32
# trace record fields
T_STEP, T_SCHED, T_SUM = 0, 1, 2
T_XC, T_YC, T_S, T_R, T_T = slice(3, 6), slice(6, 9), slice(9, 18), slice(18, 27), slice(27, 30)
T_GAP, T_LMAX = 30, 31


class CesaError(RuntimeError):
    def __init__(self, code, what=""):
        self.code = code
        super().__init__("%s: %s (%d)" % (what or "cesa", status_string(code) if _lib else code, code))


class Params(ctypes.Structure):
    """Mirror of ``cesa_params`` (registrationParameters fields first)."""
    _fields_ = [
        ("JMAX", ctypes.c_int), ("I0", ctypes.c_int), ("I1", ctypes.c_int),
        ("alpha", ctypes.c_float), ("T_0", ctypes.c_float), ("TFACTOR", ctypes.c_float),
        ("moutlier", ctypes.c_float),
        ("sigma_p2", ctypes.c_float), ("sigma_inf", ctypes.c_float),
        ("sigma_factor", ctypes.c_float), ("d_02", ctypes.c_float),
        ("maxIteration", ctypes.c_int),
        ("sinkhorn_form", ctypes.c_int), ("timeout_ms", ctypes.c_int), ("device", ctypes.c_int),
        ("icp_search", ctypes.c_int), ("emicp_backward_layout", ctypes.c_int),
        ("softassign_backward_form", ctypes.c_int), ("reserved", ctypes.c_int * 2),
    ]

    @classmethod
    def default(cls, **kw):
        """Reference defaults (src/main.cpp:280-315), overridden by keyword."""
        p = cls()
        lib().cesa_params_default(ctypes.byref(p))
        for k, v in kw.items():
            if not hasattr(p, k):
                raise AttributeError(k)
            setattr(p, k, v)
        if "T_0" in kw and "moutlier" not in kw:
            p.moutlier = float(np.float32(1.0 / np.sqrt(np.float32(p.T_0)) * np.exp(np.float32(-1.0))))
        return p


# registrationParameters is the reference's name for the same record
registrationParameters = Params

ALGO_EMICP = 0
ALGO_SOFTASSIGN = 1
MAX_BATCH = 1024


class Pair(ctypes.Structure):
    """Mirror of ``cesa_pair``: one registration of a batch."""
    _fields_ = [
        ("algorithm", ctypes.c_int), ("N", ctypes.c_int), ("M", ctypes.c_int),
        ("X", ctypes.c_void_p), ("Y", ctypes.c_void_p), ("Rt", ctypes.c_void_p),
        ("params", Params),
    ]


class Report(ctypes.Structure):
    _fields_ = [
        ("trace", ctypes.c_void_p), ("trace_capacity", ctypes.c_int), ("steps", ctypes.c_int),
        ("sinkhorn_form", ctypes.c_int), ("grid_blocks", ctypes.c_int), ("device_ms", ctypes.c_float),
        ("timeline", ctypes.c_void_p), ("timeline_capacity", ctypes.c_int), ("timeline_written", ctypes.c_int),
    ]


_lib = None

_p = ctypes.c_void_p
_i = ctypes.c_int
_f = ctypes.c_float


def lib():
    """The loaded libcesa.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libcesa.so is not built (run: python -m cuda_emicp_softassign_gb300.build)")
        L = ctypes.CDLL(LIB_PATH)
        L.cesa_params_default.argtypes = [_p]
        L.cesa_params_default.restype = None
        for name in ("cesa_emicp", "cesa_softassign", "cesa_icp"):
            fn = getattr(L, name)
            fn.argtypes = [_p, _i, _p, _i, _p, _p, _p, _p]
            fn.restype = _i
        L.cesa_icp_device.argtypes = [_p, _i, _p, _i, _p, _p, _p, _p, _p]
        L.cesa_icp_device.restype = _i
        L.cesa_load_points.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.POINTER(ctypes.c_float)),
                                       ctypes.POINTER(_i)]
        L.cesa_load_points.restype = _i
        L.cesa_free.argtypes = [_p]
        L.cesa_free.restype = None
        L.cesa_points_reduction.argtypes = [_p, ctypes.POINTER(_i), ctypes.c_float, ctypes.c_ulonglong]
        L.cesa_points_reduction.restype = _i
        L.cesa_align_scale_once.argtypes = [_p, _i, _p, _i]
        L.cesa_align_scale_once.restype = _i
        L.cesa_save_rt.argtypes = [ctypes.c_char_p, _p, _p]
        L.cesa_save_rt.restype = _i
        L.cesa_load_rt.argtypes = [ctypes.c_char_p, _p, _p]
        L.cesa_load_rt.restype = _i
        L.cesa_save_points.argtypes = [ctypes.c_char_p, _p, _i, _i]
        L.cesa_save_points.restype = _i
        L.cesa_transform_points.argtypes = [_p, _i, _p, _p]
        L.cesa_transform_points.restype = _i
        for name in ("cesa_emicp_device", "cesa_softassign_device"):
            fn = getattr(L, name)
            fn.argtypes = [_p, _i, _p, _i, _p, _p, _p, _p]
            fn.restype = _i
        L.cesa_stream_status.argtypes = [_p]
        L.cesa_stream_status.restype = _i
        L.cesa_emicp_step_device.argtypes = [_p, _i, _p, _i, _p, _p, _f, _f, _p, _p, _p]
        L.cesa_emicp_step_device.restype = _i
        L.cesa_softassign_step_device.argtypes = [_p, _i, _p, _i, _p, _p, _f, _f, _i, _i,
                                                  _p, _p, _p, _p, _p, _p, _p]
        L.cesa_softassign_step_device.restype = _i
        L.cesa_find_rt_from_s.argtypes = [_p] * 6
        L.cesa_find_rt_from_s.restype = _i
        L.cesa_cloud2data.argtypes = [_p, _i, _i, _p]
        L.cesa_cloud2data.restype = _i
        L.cesa_release_workspaces.argtypes = []
        L.cesa_release_workspaces.restype = None
        L.cesa_status_string.argtypes = [_i]
        L.cesa_status_string.restype = ctypes.c_char_p
        L.cesa_version.restype = _i
        L.cesa_register_batch_device.argtypes = [_p, _i, _p, _p]
        L.cesa_register_batch_device.restype = _i
        L.cesa_register_batch.argtypes = [_p, _i, _p]
        L.cesa_register_batch.restype = _i
        L.cesa_emicp_tape_bytes.argtypes = [_i, _i, _p]
        L.cesa_emicp_tape_bytes.restype = ctypes.c_size_t
        L.cesa_emicp_forward_device.argtypes = [_p, _i, _p, _i, _p, _p, _p, _p, _p]
        L.cesa_emicp_forward_device.restype = _i
        L.cesa_emicp_backward_device.argtypes = [_i, _i, _p, _p, _p, _p, _p, _p, _p, _p]
        L.cesa_emicp_backward_device.restype = _i
        L.cesa_softassign_tape_bytes.argtypes = [_i, _i, _p]
        L.cesa_softassign_tape_bytes.restype = ctypes.c_size_t
        L.cesa_softassign_forward_device.argtypes = [_p, _i, _p, _i, _p, _p, _p, _p, _p]
        L.cesa_softassign_forward_device.restype = _i
        L.cesa_softassign_backward_device.argtypes = [_i, _i, _p, _p, _p, _p, _p, _p, _p, _p]
        L.cesa_softassign_backward_device.restype = _i
        L.cesa_tune_sinkhorn.argtypes = [_i, _i, _p, _p, _p, _p]
        L.cesa_tune_sinkhorn.restype = _i
        L.cesa_self_test_waits.argtypes = [_i, _i, _p, _p]
        L.cesa_self_test_waits.restype = _i
        _lib = L
    return _lib


def status_string(code):
    return lib().cesa_status_string(int(code)).decode()


def _check(rc, what):
    if rc != CESA_OK:
        raise CesaError(rc, what)


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def cloud2data(points):
    """(n, 3) points -> SoA float32 [x..., y..., z...] (src/cloud2data.cpp:29-46)."""
    P = np.ascontiguousarray(points, dtype=np.float32)
    if P.ndim != 2 or P.shape[1] < 3:
        raise ValueError("points must be (n, 3)")
    out = np.empty(3 * P.shape[0], np.float32)
    _check(lib().cesa_cloud2data(_ptr(P), P.shape[0], P.shape[1], _ptr(out)), "cloud2data")
    return out


def _pose_in(R, t):
    Rh = np.ascontiguousarray(np.eye(3) if R is None else R, dtype=np.float32).reshape(-1).copy()
    th = np.ascontiguousarray(np.zeros(3) if t is None else t, dtype=np.float32).reshape(-1).copy()
    if Rh.size != 9 or th.size != 3:
        raise ValueError("R must be 3x3 and t must have 3 entries")
    return Rh, th


def _host_call(fn_name, X, Y, R, t, param, trace, timeline=0):
    Xs, Ys = cloud2data(X), cloud2data(Y)
    Rh, th = _pose_in(R, t)
    rep = Report()
    tl = None
    if timeline:
        tl = np.zeros(int(timeline), np.uint64)
        rep.timeline = tl.ctypes.data
        rep.timeline_capacity = int(timeline)
    tr = None
    if trace:
        cap = int(trace) if not isinstance(trace, bool) else 100000
        tr = np.zeros((cap, TRACE_STRIDE))
        rep.trace = tr.ctypes.data
        rep.trace_capacity = cap
    rc = getattr(lib(), fn_name)(_ptr(Xs), len(X), _ptr(Ys), len(Y), _ptr(Rh), _ptr(th),
                                 ctypes.byref(param), ctypes.byref(rep))
    _check(rc, fn_name)
    out = (Rh.reshape(3, 3).astype(np.float64), th.astype(np.float64))
    if timeline:
        return out + (tl, rep)
    if trace:
        return out + (tr[: min(rep.steps, tr.shape[0])], rep)
    return out


def timeline_table(tl, grid_blocks=1, block=None):
    """Decodes a phase timeline into rows (block, phase, ns since the earliest
    entry of any block); `block` selects one block's rows."""
    tl = np.asarray(tl, dtype=np.uint64)
    per = len(tl) // max(grid_blocks, 1)
    tl = tl[: per * grid_blocks].reshape(grid_blocks, per)
    blk = np.repeat(np.arange(grid_blocks), per).reshape(grid_blocks, per)
    used = tl != 0
    phase = (tl >> np.uint64(56)).astype(np.int64)[used]
    t = (tl & np.uint64((1 << 56) - 1)).astype(np.int64)[used]
    b = blk[used]
    rows = np.stack([b, phase, t - (t.min() if len(t) else 0)], axis=1)
    return rows if block is None else rows[rows[:, 0] == block][:, 1:]


def emicp(X, Y, R=None, t=None, param=None, trace=False, timeline=0):
    """Annealed EM-ICP on the GPU (replaces emicp(), src/emicp.cu:247-716).

    Returns (R, t); (R, t, trace, report) when ``trace`` is set; (R, t,
    timeline, report) when ``timeline`` (a capacity) is given.
    """
    return _host_call("cesa_emicp", X, Y, R, t, param or Params.default(), trace, timeline)


def softassign(X, Y, R=None, t=None, param=None, trace=False, timeline=0):
    """Annealed Softassign on the GPU (replaces softassign(), src/softassign.cu:256-886)."""
    return _host_call("cesa_softassign", X, Y, R, t, param or Params.default(), trace, timeline)


def find_rt_from_s(Xc, Yc, S, q_prev=None):
    """Horn's pose from centres and cross-covariance (replaces findRTfromS)."""
    xc = np.ascontiguousarray(Xc, dtype=np.float32)
    yc = np.ascontiguousarray(Yc, dtype=np.float32)
    s = np.ascontiguousarray(np.asarray(S, dtype=np.float32).reshape(-1))
    R = np.zeros(9, np.float32)
    t = np.zeros(3, np.float32)
    qp = None if q_prev is None else np.ascontiguousarray(q_prev, dtype=np.float32)
    _check(lib().cesa_find_rt_from_s(_ptr(xc), _ptr(yc), _ptr(s), _ptr(R), _ptr(t),
                                     _ptr(qp) if qp is not None else None), "find_rt_from_s")
    return R.reshape(3, 3).astype(np.float64), t.astype(np.float64)


# ----------------------------------------------------------------- device API
# These take torch CUDA tensors (torch only provides the device memory and the
# stream; the work runs in libcesa.so).

def _stream_handle(stream):
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    return getattr(stream, "cuda_stream", stream)


def _dptr(t):
    return ctypes.c_void_p(t.data_ptr())


def icp(X, Y, R=None, t=None, param=None, trace=False):
    """ICP on the GPU, maxIteration iterations of exact nearest-neighbour
    matching (a uniform grid over the target, or exhaustive: param.icp_search)
    and Horn's pose (replaces icp(), src/icp.cpp:122-290, whose FLANN search is
    approximate). Returns (R, t), or (R, t, trace, report)."""
    return _host_call("cesa_icp", X, Y, R, t, param or Params.default(), trace)


def icp_device(dX, dY, dRt, param=None, d_nn=None, d_status=None, stream=None):
    """Enqueue ICP on device SoA tensors; dRt (12 floats) is in/out; d_nn
    (optional int32 tensor of M) receives the last iteration's matches."""
    p = param or Params.default()
    rc = lib().cesa_icp_device(_dptr(dX), dX.numel() // 3, _dptr(dY), dY.numel() // 3, _dptr(dRt), ctypes.byref(p),
                               _dptr(d_nn) if d_nn is not None else None,
                               _dptr(d_status) if d_status is not None else None,
                               ctypes.c_void_p(_stream_handle(stream)))
    _check(rc, "icp_device")


def load_points(path):
    """Points of a PLY (ASCII / binary), PCD (ascii / binary /
    binary_compressed) or text file as an (n, 3) float32 array, non-finite
    points dropped (the reference CLI's loadFile)."""
    L = lib()
    buf = ctypes.POINTER(ctypes.c_float)()
    n = _i(0)
    _check(L.cesa_load_points(os.fsencode(path), ctypes.byref(buf), ctypes.byref(n)), "load_points")
    try:
        out = np.ctypeslib.as_array(buf, shape=(n.value * 3,)).reshape(-1, 3).copy() if n.value else \
            np.zeros((0, 3), np.float32)
    finally:
        L.cesa_free(ctypes.cast(buf, _p))
    return out


def points_reduction(P, percent, seed=0):
    """Keeps each point with probability percent / 100, in order (seeded)."""
    a = np.ascontiguousarray(P, dtype=np.float32).copy()
    n = _i(len(a))
    _check(lib().cesa_points_reduction(_ptr(a), ctypes.byref(n), float(percent), int(seed)), "points_reduction")
    return a[: n.value]


def align_scale_once(X, Y):
    """Both clouds scaled about the origin to a covariance trace of 0.003."""
    a = np.ascontiguousarray(X, dtype=np.float32).copy()
    b = np.ascontiguousarray(Y, dtype=np.float32).copy()
    _check(lib().cesa_align_scale_once(_ptr(a), len(a), _ptr(b), len(b)), "align_scale_once")
    return a, b


def save_points(path, P, fmt=POINTS_BY_NAME):
    """Writes (n, 3) points as ASCII PCD (PCL's savePCDFileASCII layout), ASCII
    PLY or text; POINTS_BY_NAME picks by the extension."""
    a = np.ascontiguousarray(P, dtype=np.float32).reshape(-1, 3)
    _check(lib().cesa_save_points(os.fsencode(path), _ptr(a), len(a), int(fmt)), "save_points")


def transform_points(P, R, t):
    """R P + t per point in FP32 (the reference tools' pcl::transformPointCloud)."""
    a = np.ascontiguousarray(P, dtype=np.float32).reshape(-1, 3).copy()
    Rh, th = _pose_in(R, t)
    _check(lib().cesa_transform_points(_ptr(a), len(a), _ptr(Rh), _ptr(th)), "transform_points")
    return a


def save_rt(path, R, t):
    Rh, th = _pose_in(R, t)
    _check(lib().cesa_save_rt(os.fsencode(path), _ptr(Rh), _ptr(th)), "save_rt")


def load_rt(path):
    Rh = np.zeros(9, np.float32)
    th = np.zeros(3, np.float32)
    _check(lib().cesa_load_rt(os.fsencode(path), _ptr(Rh), _ptr(th)), "load_rt")
    return Rh.reshape(3, 3).astype(np.float64), th.astype(np.float64)


def emicp_device(dX, dY, dRt, param=None, d_status=None, stream=None):
    """Enqueue EM-ICP on device SoA tensors; dRt (12 floats, R then t) is in/out."""
    p = param or Params.default()
    rc = lib().cesa_emicp_device(_dptr(dX), dX.numel() // 3, _dptr(dY), dY.numel() // 3, _dptr(dRt),
                                 ctypes.byref(p), _dptr(d_status) if d_status is not None else None,
                                 ctypes.c_void_p(_stream_handle(stream)))
    _check(rc, "emicp_device")


def softassign_device(dX, dY, dRt, param=None, d_status=None, stream=None):
    p = param or Params.default()
    rc = lib().cesa_softassign_device(_dptr(dX), dX.numel() // 3, _dptr(dY), dY.numel() // 3,
                                      _dptr(dRt), ctypes.byref(p),
                                      _dptr(d_status) if d_status is not None else None,
                                      ctypes.c_void_p(_stream_handle(stream)))
    _check(rc, "softassign_device")


def emicp_device_noalloc(dX, dY, dRt, param=None, d_status=None, stream=None):
    """EM-ICP on device tensors without any device allocation (fixed 16 MiB
    scratch inside libcesa.so); for callers that cannot call cudaMalloc.
    Returns the C status code instead of raising, so callers can test the
    size limit (CESA_ERR_NOALLOC_LIMIT)."""
    p = param or Params.default()
    fn = lib().cesa_emicp_device_noalloc
    fn.argtypes = [_p, _i, _p, _i, _p, _p, _p, _p]
    fn.restype = _i
    return fn(_dptr(dX), dX.numel() // 3, _dptr(dY), dY.numel() // 3, _dptr(dRt), ctypes.byref(p),
              _dptr(d_status) if d_status is not None else None, ctypes.c_void_p(_stream_handle(stream)))


def register_batch(pairs, report=False):
    """Batched registration on host clouds, one persistent launch.

    pairs: sequence of (algorithm, X, Y, params) or (algorithm, X, Y, params,
    R0, t0), with algorithm ALGO_EMICP or ALGO_SOFTASSIGN and X, Y (n, 3).
    Returns a list of (R, t); with ``report`` also the Report.
    """
    n = len(pairs)
    arr = (Pair * n)()
    keep = []
    for i, pr in enumerate(pairs):
        algo, X, Y, prm = pr[:4]
        R0, t0 = (pr[4], pr[5]) if len(pr) > 4 else (None, None)
        Xs, Ys = cloud2data(X), cloud2data(Y)
        Rh, th = _pose_in(R0, t0)
        rt = np.concatenate([Rh, th]).astype(np.float32)
        keep.append((Xs, Ys, rt))
        arr[i].algorithm = int(algo)
        arr[i].N = len(X)
        arr[i].M = len(Y)
        arr[i].X = Xs.ctypes.data
        arr[i].Y = Ys.ctypes.data
        arr[i].Rt = rt.ctypes.data
        arr[i].params = prm if prm is not None else Params.default()
    rep = Report()
    _check(lib().cesa_register_batch(ctypes.cast(arr, ctypes.c_void_p), n, ctypes.byref(rep)), "register_batch")
    out = [(k[2][:9].reshape(3, 3).astype(np.float64), k[2][9:].astype(np.float64)) for k in keep]
    return (out, rep) if report else out


def register_batch_device(pairs, d_status=None, stream=None):
    """Batched registration on device tensors: pairs of (algorithm, dX, dY,
    dRt, params) with SoA float32 dX (3N), dY (3M) and dRt (12, in/out).
    Enqueues on `stream` (default: torch's current stream)."""
    n = len(pairs)
    arr = (Pair * n)()
    for i, (algo, dX, dY, dRt, prm) in enumerate(pairs):
        arr[i].algorithm = int(algo)
        arr[i].N = dX.numel() // 3
        arr[i].M = dY.numel() // 3
        arr[i].X = dX.data_ptr()
        arr[i].Y = dY.data_ptr()
        arr[i].Rt = dRt.data_ptr()
        arr[i].params = prm if prm is not None else Params.default()
    rc = lib().cesa_register_batch_device(ctypes.cast(arr, ctypes.c_void_p), n,
                                          _dptr(d_status) if d_status is not None else None,
                                          ctypes.c_void_p(_stream_handle(stream)))
    _check(rc, "register_batch_device")


def stream_status(stream=None):
    return lib().cesa_stream_status(ctypes.c_void_p(_stream_handle(stream)))


def emicp_step(dX, dY, R, t, sigma_p2, d_02, row_out=None, stream=None):
    """One fused E-step from (R, t). Returns moments[16] = sum(lambda), Xc, Yc, S."""
    Rh, th = _pose_in(R, t)
    mom = np.zeros(16)
    rc = lib().cesa_emicp_step_device(_dptr(dX), dX.numel() // 3, _dptr(dY), dY.numel() // 3,
                                      _ptr(Rh), _ptr(th), sigma_p2, d_02,
                                      _dptr(row_out) if row_out is not None else None, _ptr(mom),
                                      ctypes.c_void_p(_stream_handle(stream)))
    _check(rc, "emicp_step")
    return mom


def softassign_step(dX, dY, R, t, T, alpha, I1, s, u, rs=None, cs=None, w=None,
                    form=SINKHORN_MATRIX_FREE, stream=None):
    """One Softassign inner iteration; s, u (device) are updated in place."""
    Rh, th = _pose_in(R, t)
    mom = np.zeros(16)
    opt = lambda x: _dptr(x) if x is not None else None  # noqa: E731
    rc = lib().cesa_softassign_step_device(_dptr(dX), dX.numel() // 3, _dptr(dY), dY.numel() // 3,
                                           _ptr(Rh), _ptr(th), T, alpha, I1, form, _dptr(s), _dptr(u),
                                           opt(rs), opt(cs), opt(w), _ptr(mom),
                                           ctypes.c_void_p(_stream_handle(stream)))
    _check(rc, "softassign_step")
    return mom


def tune_sinkhorn(N, M, param=None):
    """Times both Sinkhorn forms for N x M on the current device and records
    the faster one for CESA_SINKHORN_AUTO. Returns (form, ms per pose update
    matrix-free, ms per pose update materialised or -1)."""
    f = ctypes.c_int(0)
    a = ctypes.c_float(0)
    b = ctypes.c_float(0)
    _check(lib().cesa_tune_sinkhorn(int(N), int(M), ctypes.byref(param) if param is not None else None,
                                    ctypes.byref(f), ctypes.byref(a), ctypes.byref(b)), "tune_sinkhorn")
    return f.value, a.value, b.value


def release_workspaces():
    lib().cesa_release_workspaces()


def self_test_waits(which, timeout_us=1000):
    """Runs the grid barrier (which=0) or the mbarrier wait (which=1) of the
    kernels on a barrier that nothing completes. Returns (rc, status, where):
    rc is CESA_OK when the probe ran and the device still works afterwards;
    status is the code the expired wait recorded (CESA_ERR_TIMEOUT)."""
    st = ctypes.c_int(-1)
    wh = ctypes.c_int(-1)
    rc = lib().cesa_self_test_waits(int(which), int(timeout_us), ctypes.byref(st), ctypes.byref(wh))
    return rc, st.value, wh.value


def version():
    return lib().cesa_version()
