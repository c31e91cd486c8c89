"""ctypes binding of libops_fft.so (the GB300 aclfft C API).

This is the Python face of the same C ABI a C/C++ caller links against:
every call goes through ``libops_fft.so``; nothing here computes a
transform.  Loading fails loudly when the library has not been built.

    import aclfft
    p = aclfft.Plan.plan1d(4096, aclfft.C2C, batch=256)
    p.exec_c2c(x.data_ptr(), y.data_ptr(), aclfft.FORWARD)   # device tensors
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libops_fft.so")

# include/cann_ops_fft.h
SUCCESS = 0
INVALID_PLAN = 1
ALLOC_FAILED = 2
INVALID_TYPE = 3
INVALID_VALUE = 4
INTERNAL_ERROR = 5
EXEC_FAILED = 6
SETUP_FAILED = 7
INVALID_SIZE = 8
UNALIGNED_DATA = 9
INCOMPLETE_PARAMETER_LIST = 10
INVALID_DEVICE = 11
PARSE_ERROR = 12
NO_WORKSPACE = 13
NOT_IMPLEMENTED = 14
NOT_SUPPORTED = 16

R2C = 0x2A
C2R = 0x2C
C2C = 0x29
D2Z = 0x6A
Z2D = 0x6C
Z2Z = 0x69

FORWARD = -1
BACKWARD = 1
HORIZONTAL = 0
VERTICAL = 1

# include/aclfft_ext.h
NORM_NONE = 0
NORM_BACKWARD = 1
NORM_ORTHO = 2
NORM_FORWARD = 3

# aclfftPrecisionMode (C2C DFT-stage arithmetic)
PREC_FP32 = 0
PREC_TF32X3 = 1
PREC_BF16X3 = 2


class PlanInfo(ctypes.Structure):
    _fields_ = [
        ("supported", ctypes.c_int),
        ("nsteps", ctypes.c_int),
        ("nradix", ctypes.c_int),
        ("radix", ctypes.c_int * 12),
        ("onchip_length", ctypes.c_int),
        ("threads_per_transform", ctypes.c_int),
        ("transforms_per_cta", ctypes.c_int),
        ("twiddle_entries", ctypes.c_longlong),
        ("workspace_bytes", ctypes.c_size_t),
        ("kernel", ctypes.c_int),
        ("groups_per_cta", ctypes.c_int),
        ("stages", ctypes.c_int),
        ("smem_bytes", ctypes.c_int),
        ("tc_stages", ctypes.c_int),
        ("cluster_ctas", ctypes.c_int),
        ("cluster_count", ctypes.c_int),
        ("tuned", ctypes.c_int),
        ("tune_candidates", ctypes.c_int),
    ]


class AclfftError(RuntimeError):
    def __init__(self, code: int, what: str):
        self.code = code
        super().__init__(f"{what} failed with {code} ({error_string(code)}) {last_error_detail()}")


_lib = None

class RaggedInfo(ctypes.Structure):
    _fields_ = [
        ("transforms", ctypes.c_int),
        ("classes", ctypes.c_int),
        ("long_transforms", ctypes.c_int),
        ("items", ctypes.c_int),
        ("tuned_classes", ctypes.c_int),
        ("graph", ctypes.c_int),
        ("smem_bytes", ctypes.c_int),
        ("twiddle_entries", ctypes.c_longlong),
        ("workspace_bytes", ctypes.c_size_t),
        ("in_bytes_min", ctypes.c_size_t),
        ("out_bytes_min", ctypes.c_size_t),
    ]


_H = ctypes.c_void_p
_HP = ctypes.POINTER(ctypes.c_void_p)
_I = ctypes.c_int
_VP = ctypes.c_void_p
_SZP = ctypes.POINTER(ctypes.c_size_t)

_SIGNATURES = {
    "aclfftPlan1d": [_HP, _I, _I, _I, _I],
    "aclfftPlan2d": [_HP, _I, _I, _I, _I],
    "aclfftPlan3d": [_HP, _I, _I, _I, _I],
    "aclfftCreate": [_HP],
    "aclfftMakePlan1d": [_H, _I, _I, _I, _I, _SZP],
    "aclfftMakePlan2d": [_H, _I, _I, _I, _I, _SZP],
    "aclfftMakePlan3d": [_H, _I, _I, _I, _I, _SZP],
    "aclfftGetSize1d": [_H, _I, _I, _I, _SZP],
    "aclfftGetSize2d": [_H, _I, _I, _I, _SZP],
    "aclfftGetSize3d": [_H, _I, _I, _I, _I, _SZP],
    "aclfftGetSize": [_H, _SZP],
    "aclfftSetAutoAllocation": [_H, _I],
    "aclfftSetWorkArea": [_H, _VP],
    "aclfftExecC2C": [_H, _VP, _VP, _I],
    "aclfftExecR2C": [_H, _VP, _VP],
    "aclfftExecC2R": [_H, _VP, _VP],
    "aclfftExecZ2Z": [_H, _VP, _VP, _I],
    "aclfftExecD2Z": [_H, _VP, _VP],
    "aclfftExecZ2D": [_H, _VP, _VP],
    "aclfftSetStream": [_H, _VP],
    "aclfftSetStride": [_H, ctypes.c_int32],
    "aclfftDestroy": [_H],
    "aclfftGetVersion": [ctypes.POINTER(_I)],
    "aclfftGetProperty": [_I, ctypes.POINTER(_I)],
    "aclfftSetNormMode": [_H, _I],
    "aclfftGetNormMode": [_H, ctypes.POINTER(_I)],
    "aclfftSetPrecisionMode": [_H, _I],
    "aclfftGetPrecisionMode": [_H, ctypes.POINTER(_I)],
    "aclfftExecC2CAdjoint": [_H, _VP, _VP, _I],
    "aclfftExecR2CAdjoint": [_H, _VP, _VP],
    "aclfftExecC2RAdjoint": [_H, _VP, _VP],
    "aclfftExecR2CAdjointWeighted": [_H, _VP, _VP, _VP],
    "aclfftGetPlanInfo": [_H, ctypes.POINTER(PlanInfo)],
    "aclfftSetAutotune": [_H, _I],
    "aclfftGetTwiddles": [_H, _VP, ctypes.c_longlong, ctypes.POINTER(ctypes.c_longlong)],
    "aclfftDebugCheckPlan": [_H, ctypes.c_char_p, _I],
    "aclfftExecC2CNoAlloc": [_VP, _VP, _I, _I, _I, _VP],
    "aclfftRaggedPlanCreate": [_HP, _I, _VP, _VP, _VP, _VP],
    "aclfftRaggedSetStream": [_H, _VP],
    "aclfftRaggedSetOptions": [_H, _I, _I],
    "aclfftRaggedAutotune": [_H],
    "aclfftRaggedExec": [_H, _VP, _VP, _I],
    "aclfftRaggedGetInfo": [_H, ctypes.POINTER(RaggedInfo)],
    "aclfftRaggedGetError": [_H, ctypes.POINTER(_I)],
    "aclfftRaggedDestroy": [_H],
    "aclfftRaggedDebugCheck": [_H, ctypes.c_char_p, _I],
    "aclfftRaggedSetWaitLimit": [_H, ctypes.c_longlong],
    "aclfftRaggedDebugHoldDependencies": [_H, _I],
    "aclfftGetExecError": [_H, ctypes.POINTER(_I)],
    "aclfftDebugSetExecError": [_H, _I],
    "aclfftDebugFailAllocations": [_I],
    "aclfftDebugButterfly": [_I, ctypes.c_void_p, ctypes.c_void_p],
    "aclfftDebugGetTwiddleSegments": [_H, _VP, _I, ctypes.POINTER(_I)],
}


# include/aclfft_ops.h: the per-operator direct entries (aclError results)
ACL_SUCCESS = 0
ACL_ERROR_INVALID_PARAM = 100000
ACL_ERROR_BAD_ALLOC = 200000
ACL_ERROR_INTERNAL_ERROR = 500000
_U = ctypes.c_uint32
_OPS_STD = ["aclfftFft1DDft", "aclfftFft1DN", "aclfftFft1DB", "aclfftFft1DMix", "aclfftFft1DC2C", "aclfftFft1DC2CMix",
            "aclfftRfft1DR2CFft", "aclfftRfft1DFft", "aclfftRfft1DDft", "aclfftIrfft1DFft", "aclfftIrfft1DDft",
            "aclfftIrfft1DC2RFft"]
_OPS_POW2 = ["aclfftRfft1DR2CFft1", "aclfftRfft1DR2CFft2", "aclfftRfft1DR2CFft31", "aclfftRfft1DR2CFft32",
             "aclfftRfft1DR2CFft4", "aclfftRfft1DR2CFft5"]
for _n in _OPS_STD:
    _SIGNATURES[_n] = [_VP, _VP, _U, ctypes.c_int32, _U, _I, _VP]
for _n in _OPS_POW2:
    _SIGNATURES[_n] = [_VP, _VP, _U, _U, _I, _VP]
_SIGNATURES["aclfftFft1DStride"] = [_VP, _VP, _U, ctypes.c_int32, _U, _U, _I, _VP]
_SIGNATURES["aclfftRfft1D"] = [_VP, _VP, _U, ctypes.c_int32, _U, _VP]
_SIGNATURES["aclfftFft2DDd"] = [_VP, _VP, _U, _U, _U, _I, _VP]


def lib():
    """Load libops_fft.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise FileNotFoundError(f"{LIB_PATH} is missing: build it with ops-fft_gb300/build.py")
        L = ctypes.CDLL(LIB_PATH)
        for name, args in _SIGNATURES.items():
            fn = getattr(L, name, None)
            if fn is None:
                continue
            fn.argtypes = args
            fn.restype = ctypes.c_int
        L.aclfftGetErrorString.argtypes = [_I]
        L.aclfftGetErrorString.restype = ctypes.c_char_p
        L.aclfftGetLastErrorDetail.argtypes = []
        L.aclfftGetLastErrorDetail.restype = ctypes.c_char_p
        _lib = L
    return _lib


def error_string(code: int) -> str:
    return lib().aclfftGetErrorString(int(code)).decode()


def last_error_detail() -> str:
    return lib().aclfftGetLastErrorDetail().decode()


def ptr(x) -> int:
    """Address of a torch tensor, numpy array or raw integer pointer."""
    if x is None:
        return 0
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return int(x.data_ptr())
    if hasattr(x, "ctypes"):
        return int(x.ctypes.data)
    raise TypeError(f"cannot take the address of {type(x)}")


def _check(code: int, what: str):
    if code != SUCCESS:
        raise AclfftError(code, what)


class Plan:
    """Owning wrapper of an aclfftHandle."""

    def __init__(self, handle: int):
        self.handle = ctypes.c_void_p(handle)

    @classmethod
    def plan1d(cls, nx: int, type_: int, batch: int = 1, dim: int = HORIZONTAL) -> "Plan":
        h = ctypes.c_void_p()
        _check(lib().aclfftPlan1d(ctypes.byref(h), nx, type_, batch, dim), "aclfftPlan1d")
        return cls(h.value)

    @classmethod
    def plan2d(cls, batch: int, nx: int, ny: int, type_: int = C2C) -> "Plan":
        h = ctypes.c_void_p()
        _check(lib().aclfftPlan2d(ctypes.byref(h), batch, nx, ny, type_), "aclfftPlan2d")
        return cls(h.value)

    @classmethod
    def plan3d(cls, nx: int, ny: int, nz: int, type_: int = C2C) -> "Plan":
        h = ctypes.c_void_p()
        _check(lib().aclfftPlan3d(ctypes.byref(h), nx, ny, nz, type_), "aclfftPlan3d")
        return cls(h.value)

    def set_stream(self, stream) -> None:
        s = getattr(stream, "cuda_stream", stream)
        _check(lib().aclfftSetStream(self.handle, ctypes.c_void_p(int(s) if s else None)), "aclfftSetStream")

    def set_norm(self, mode: int) -> None:
        _check(lib().aclfftSetNormMode(self.handle, mode), "aclfftSetNormMode")

    def set_precision(self, mode: int) -> None:
        """PREC_FP32 (Stockham), PREC_TF32X3 or PREC_BF16X3 (tensor-core DFT stages)."""
        _check(lib().aclfftSetPrecisionMode(self.handle, mode), "aclfftSetPrecisionMode")

    def set_autotune(self, on: bool = True) -> None:
        """Time the planner's candidate choices for this plan and keep the fastest."""
        _check(lib().aclfftSetAutotune(self.handle, int(bool(on))), "aclfftSetAutotune")

    def precision(self) -> int:
        m = _I()
        _check(lib().aclfftGetPrecisionMode(self.handle, ctypes.byref(m)), "aclfftGetPrecisionMode")
        return m.value

    def exec_c2c(self, x, y, direction: int = FORWARD) -> None:
        _check(lib().aclfftExecC2C(self.handle, ptr(x), ptr(y), direction), "aclfftExecC2C")

    def exec_r2c(self, x, y) -> None:
        _check(lib().aclfftExecR2C(self.handle, ptr(x), ptr(y)), "aclfftExecR2C")

    def exec_c2r(self, x, y) -> None:
        _check(lib().aclfftExecC2R(self.handle, ptr(x), ptr(y)), "aclfftExecC2R")

    def exec_z2z(self, x, y, direction: int = FORWARD) -> None:
        _check(lib().aclfftExecZ2Z(self.handle, ptr(x), ptr(y), direction), "aclfftExecZ2Z")

    def exec_d2z(self, x, y) -> None:
        _check(lib().aclfftExecD2Z(self.handle, ptr(x), ptr(y)), "aclfftExecD2Z")

    def exec_z2d(self, x, y) -> None:
        _check(lib().aclfftExecZ2D(self.handle, ptr(x), ptr(y)), "aclfftExecZ2D")

    def exec_c2c_adjoint(self, g_out, g_in, direction: int = FORWARD) -> None:
        _check(lib().aclfftExecC2CAdjoint(self.handle, ptr(g_out), ptr(g_in), direction), "aclfftExecC2CAdjoint")

    def exec_r2c_adjoint(self, g_out, g_in) -> None:
        _check(lib().aclfftExecR2CAdjoint(self.handle, ptr(g_out), ptr(g_in)), "aclfftExecR2CAdjoint")

    def exec_r2c_adjoint_weighted(self, g_out, weights, g_in) -> None:
        """g_in = R2C adjoint of (weights * g_out), the weights applied as the
        bins are loaded (device tensors)."""
        _check(lib().aclfftExecR2CAdjointWeighted(self.handle, ptr(g_out), ptr(weights), ptr(g_in)),
               "aclfftExecR2CAdjointWeighted")

    def exec_c2r_adjoint(self, g_out, g_in) -> None:
        _check(lib().aclfftExecC2RAdjoint(self.handle, ptr(g_out), ptr(g_in)), "aclfftExecC2RAdjoint")

    def exec_error(self) -> int:
        """Synchronises the plan's stream and returns (and clears) the device
        error flags of its execs (0: every bounded wait completed)."""
        f = _I()
        rc = lib().aclfftGetExecError(self.handle, ctypes.byref(f))
        if rc not in (SUCCESS, EXEC_FAILED):
            _check(rc, "aclfftGetExecError")
        return f.value

    def work_size(self) -> int:
        sz = ctypes.c_size_t()
        _check(lib().aclfftGetSize(self.handle, ctypes.byref(sz)), "aclfftGetSize")
        return sz.value

    def set_auto_allocation(self, on: bool) -> None:
        _check(lib().aclfftSetAutoAllocation(self.handle, int(bool(on))), "aclfftSetAutoAllocation")

    def set_work_area(self, area) -> None:
        _check(lib().aclfftSetWorkArea(self.handle, ptr(area) or None), "aclfftSetWorkArea")

    def info(self) -> PlanInfo:
        inf = PlanInfo()
        _check(lib().aclfftGetPlanInfo(self.handle, ctypes.byref(inf)), "aclfftGetPlanInfo")
        return inf

    def twiddles(self):
        import numpy as np

        n = ctypes.c_longlong()
        _check(lib().aclfftGetTwiddles(self.handle, None, 0, ctypes.byref(n)), "aclfftGetTwiddles")
        out = np.zeros(n.value, dtype=np.complex64)
        _check(lib().aclfftGetTwiddles(self.handle, out.ctypes.data, n.value, ctypes.byref(n)), "aclfftGetTwiddles")
        return out

    def twiddle_segments(self):
        """(offset, count, M, param, kind) of every segment of the twiddle blob."""
        import numpy as np

        n = _I()
        _check(lib().aclfftDebugGetTwiddleSegments(self.handle, None, 0, ctypes.byref(n)), "aclfftDebugGetTwiddleSegments")
        out = np.zeros((max(n.value, 1), 5), dtype=np.int64)
        _check(lib().aclfftDebugGetTwiddleSegments(self.handle, out.ctypes.data, n.value, ctypes.byref(n)),
               "aclfftDebugGetTwiddleSegments")
        return [tuple(int(v) for v in row) for row in out[: n.value]]

    def check(self) -> str:
        """Host-side bounds check of every launch of the plan ('ok' or why)."""
        buf = ctypes.create_string_buffer(256)
        rc = lib().aclfftDebugCheckPlan(self.handle, buf, 256)
        msg = buf.value.decode()
        if rc != 0:
            raise AssertionError(msg)
        return msg

    def destroy(self) -> None:
        if self.handle and self.handle.value:
            lib().aclfftDestroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.destroy()


class RaggedPlan:
    """Owning wrapper of an aclfftRaggedPlan: many 1D C2C / R2C transforms of
    different lengths executed by one persistent launch.

    lengths, types (C2C or R2C per transform) and byte offsets of each
    transform's input and output relative to the exec pointers."""

    def __init__(self, lengths, types, in_offsets, out_offsets):
        import numpy as np

        n = len(lengths)
        self._len = np.ascontiguousarray(lengths, dtype=np.int32)
        self._typ = np.ascontiguousarray(types, dtype=np.int32)
        self._ino = np.ascontiguousarray(in_offsets, dtype=np.int64)
        self._outo = np.ascontiguousarray(out_offsets, dtype=np.int64)
        self.handle = ctypes.c_void_p()
        _check(lib().aclfftRaggedPlanCreate(ctypes.byref(self.handle), n, self._len.ctypes.data,
                                            self._typ.ctypes.data, self._ino.ctypes.data, self._outo.ctypes.data),
               "aclfftRaggedPlanCreate")

    def set_stream(self, stream) -> None:
        s = stream.cuda_stream if hasattr(stream, "cuda_stream") else stream
        _check(lib().aclfftRaggedSetStream(self.handle, s), "aclfftRaggedSetStream")

    def set_options(self, autotune: bool = True, graph: bool = True) -> None:
        _check(lib().aclfftRaggedSetOptions(self.handle, int(autotune), int(graph)), "aclfftRaggedSetOptions")

    def autotune(self) -> None:
        _check(lib().aclfftRaggedAutotune(self.handle), "aclfftRaggedAutotune")

    def exec(self, x, y, direction: int = FORWARD) -> None:
        _check(lib().aclfftRaggedExec(self.handle, ptr(x), ptr(y), direction), "aclfftRaggedExec")

    def info(self) -> RaggedInfo:
        inf = RaggedInfo()
        _check(lib().aclfftRaggedGetInfo(self.handle, ctypes.byref(inf)), "aclfftRaggedGetInfo")
        return inf

    def error_flags(self) -> int:
        """Synchronises the plan's stream and returns (and clears) the device
        error flags (bit 2: a dependency wait ran out of time)."""
        f = _I()
        rc = lib().aclfftRaggedGetError(self.handle, ctypes.byref(f))
        if rc not in (SUCCESS, EXEC_FAILED):
            _check(rc, "aclfftRaggedGetError")
        return f.value

    def set_wait_limit(self, cycles: int) -> None:
        _check(lib().aclfftRaggedSetWaitLimit(self.handle, int(cycles)), "aclfftRaggedSetWaitLimit")

    def debug_hold_dependencies(self, extra: int) -> None:
        _check(lib().aclfftRaggedDebugHoldDependencies(self.handle, int(extra)),
               "aclfftRaggedDebugHoldDependencies")

    def check(self) -> str:
        buf = ctypes.create_string_buffer(256)
        rc = lib().aclfftRaggedDebugCheck(self.handle, buf, 256)
        msg = buf.value.decode()
        if rc != 0:
            raise AssertionError(msg)
        return msg

    def destroy(self) -> None:
        if self.handle and self.handle.value:
            lib().aclfftRaggedDestroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.destroy()


def ragged_lengths(count: int, lo: int = 16, hi: int = 32768, c2c_frac: float = 0.7, seed: int = 12345,
                   primes=(2, 3, 5, 7)):
    """Seeded ragged workload: lengths log-uniform over the integers in
    [lo, hi] whose prime factors are in `primes` (a log-uniform draw snapped
    to the nearest such length), kinds C2C with probability c2c_frac else
    R2C.  Returns (lengths, types) as numpy int arrays."""
    import numpy as np

    smooth = [1]
    for p in primes:
        nxt = []
        for v in smooth:
            x = v
            while x <= hi:
                nxt.append(x)
                x *= p
        smooth = sorted(set(nxt))
    smooth = np.array([v for v in smooth if lo <= v <= hi], dtype=np.int64)
    logs = np.log(smooth.astype(np.float64))
    rng = np.random.default_rng(seed)
    u = rng.uniform(np.log(lo), np.log(hi), size=count)
    idx = np.clip(np.searchsorted(logs, u), 1, len(smooth) - 1)
    pick = np.where(np.abs(logs[idx - 1] - u) <= np.abs(logs[idx] - u), idx - 1, idx)
    lengths = smooth[pick].astype(np.int32)
    types = np.where(rng.uniform(size=count) < c2c_frac, C2C, R2C).astype(np.int32)
    return lengths, types


def ragged_layout(lengths, types, align: int = 256):
    """Packed byte offsets of each transform's input and output (each start
    rounded up to `align` bytes) and the total input / output bytes."""
    import numpy as np

    ino = np.zeros(len(lengths), dtype=np.int64)
    outo = np.zeros(len(lengths), dtype=np.int64)
    ci = co = 0
    for i, (n, t) in enumerate(zip(lengths, types)):
        n = int(n)
        ino[i], outo[i] = ci, co
        inb = 8 * n if t == C2C else 4 * n
        outb = 8 * n if t == C2C else 8 * (n // 2 + 1)
        ci += -(-inb // align) * align
        co += -(-outb // align) * align
    return ino, outo, ci, co
