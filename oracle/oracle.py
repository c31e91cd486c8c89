"""CPU oracle for the aclfft transform path (test infrastructure only).

Only tests/, __graft_entry__.smoke() (as the checker) and bench.py's
CPU-baseline leg import this module.  The shipped library never does.

Contents
--------
* numpy wrappers over ``oracle_fft.c`` (FP64 checker ``orc_*`` and the FP32
  port of the reference's arch35 Stockham path ``port_*``);
* ``comparison_details`` - the reference's pass/fail metric, restated from
  src/common/host/test_helper.py:41-71 (max-abs error, rel-L2 error and the
  count of elements above atol, all in float64 over the interleaved floats);
* ``ordered_factorize`` / ``choose_radix`` - the reference's plan-time
  factorisation, restated from src/common/host/fft_exec_helper.h:79-139;
* ``stockham_index_maps`` - the autosort Stockham read/write index maps of
  src/fft1_d/arch35/mix/fft1_d_c2c_mix_kernel.h:29-120 (``len/prev/part``
  indexing), used to prove index permutations bit-exactly on integers.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_REF_LIB_PATH = os.path.join(_HERE, "_ref", "libref_aclfft.so")
_lock = threading.Lock()
_lib = None


def build(quiet: bool = True) -> str:
    """Compile oracle_fft.c into _build/liboracle.so (gcc, seconds)."""
    out = subprocess.run(["make", "-C", _HERE, "all"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)
    return _LIB_PATH


def reference_root() -> str:
    """Where the reference tree is mounted: $OPS_FFT_REFERENCE, by default
    /root/reference (only this container has it; nothing on a GPU machine
    reads it)."""
    return os.environ.get("OPS_FFT_REFERENCE", "/root/reference")


def build_ref(ref_root: str | None = None) -> str | None:
    """Compile the reference's API layer into _ref/ when its sources exist."""
    ref_root = ref_root or reference_root()
    if not os.path.isdir(os.path.join(ref_root, "lib")):
        return None
    out = subprocess.run(["make", "-C", _HERE, "ref", f"REF={ref_root}"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("reference API build failed:\n" + out.stdout + out.stderr)
    return _REF_LIB_PATH


def ref_lib_path() -> str | None:
    return _REF_LIB_PATH if os.path.exists(_REF_LIB_PATH) else None


def _load():
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(_LIB_PATH):
                build()
            lib = ctypes.CDLL(_LIB_PATH)
            dp = ctypes.POINTER(ctypes.c_double)
            fp = ctypes.POINTER(ctypes.c_float)
            i64 = ctypes.c_int64
            lib.orc_c2c.argtypes = [dp, dp, i64, i64, ctypes.c_int]
            lib.orc_c2c_vertical.argtypes = [dp, dp, i64, i64, ctypes.c_int]
            lib.orc_c2c_2d.argtypes = [dp, dp, i64, i64, i64, ctypes.c_int]
            lib.orc_r2c.argtypes = [dp, dp, i64, i64]
            lib.orc_c2r.argtypes = [dp, dp, i64, i64]
            lib.orc_dft_bins.argtypes = [dp, i64, ctypes.POINTER(i64), i64, ctypes.c_int, dp]
            lib.port_c2c.argtypes = [fp, fp, i64, i64, ctypes.c_int, ctypes.c_int]
            lib.port_r2c.argtypes = [fp, fp, i64, i64, ctypes.c_int]
            lib.port_c2r.argtypes = [fp, fp, i64, i64, ctypes.c_int]
            lib.orc_num_threads.restype = ctypes.c_int
            _lib = lib
    return _lib


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"oracle {what} failed with {rc}")


# ---------------------------------------------------------------- FP64 checker
def c2c(x, sign: int = -1) -> np.ndarray:
    """Unscaled batched C2C over the last axis of a complex array."""
    x = np.ascontiguousarray(x, dtype=np.complex128)
    n = x.shape[-1]
    batch = x.size // n if n else 0
    out = np.empty_like(x)
    _check(_load().orc_c2c(_dptr(x), _dptr(out), n, batch, int(sign)), "c2c")
    return out


def c2c_vertical(x, sign: int = -1) -> np.ndarray:
    """Transforms down the columns of an [n, batch] complex array."""
    x = np.ascontiguousarray(x, dtype=np.complex128)
    n, batch = x.shape
    out = np.empty_like(x)
    _check(_load().orc_c2c_vertical(_dptr(x), _dptr(out), n, batch, int(sign)), "c2c_vertical")
    return out


def c2c_2d(x, sign: int = -1) -> np.ndarray:
    """Unscaled 2D C2C over the last two axes of [..., nx, ny]."""
    x = np.ascontiguousarray(x, dtype=np.complex128)
    nx, ny = x.shape[-2], x.shape[-1]
    batch = x.size // (nx * ny)
    out = np.empty_like(x)
    _check(_load().orc_c2c_2d(_dptr(x), _dptr(out), nx, ny, batch, int(sign)), "c2c_2d")
    return out


def r2c(x) -> np.ndarray:
    """Real-to-complex over the last axis; output has n//2+1 bins."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    n = x.shape[-1]
    batch = x.size // n
    out = np.empty(x.shape[:-1] + (n // 2 + 1,), dtype=np.complex128)
    _check(_load().orc_r2c(_dptr(x), _dptr(out), n, batch), "r2c")
    return out


def r2c_long_rows(x) -> np.ndarray:
    """FP64 R2C of very long rows (n in the millions) through numpy's pocketfft
    in double precision, about ten times faster than ``r2c`` at n = 2^24; an
    independent FP64 FFT, cross-checked against ``r2c`` in the oracle tests."""
    return np.fft.rfft(np.asarray(x, dtype=np.float64), axis=-1)


def c2r(X, n: int) -> np.ndarray:
    """Unscaled complex-to-real (N * irfft) of n//2+1 bins to n samples."""
    X = np.ascontiguousarray(X, dtype=np.complex128)
    if X.shape[-1] != n // 2 + 1:
        raise ValueError("c2r expects n//2+1 bins")
    batch = X.size // (n // 2 + 1)
    out = np.empty(X.shape[:-1] + (n,), dtype=np.float64)
    _check(_load().orc_c2r(_dptr(X), _dptr(out), n, batch), "c2r")
    return out


def _c2c_axis(x, axis: int, sign: int) -> np.ndarray:
    """Unscaled C2C along one axis through the C oracle (moved last, back)."""
    y = np.moveaxis(np.asarray(x, dtype=np.complex128), axis, -1)
    return np.moveaxis(c2c(y, sign), -1, axis)


def r2c_2d(x) -> np.ndarray:
    """2D real-to-complex over the last two axes of [..., nx, ny]: rows of
    length ny to ny//2+1 bins, then forward C2C down the columns (length nx).
    Composed from the pinned 1D oracles; the reference has no 2D real path
    (lib/fft_plan_init_api.cpp:200-209 rejects it), numpy's rfft2 is the
    independent cross-check in the oracle tests."""
    return _c2c_axis(r2c(x), -2, -1)


def c2r_2d(X, ny: int) -> np.ndarray:
    """Unscaled 2D complex-to-real (nx * ny * irfft2): backward C2C down the
    columns of the half spectrum, then rows of ny//2+1 bins to ny samples."""
    return c2r(_c2c_axis(X, -2, +1), ny)


def r2c_3d(x) -> np.ndarray:
    """3D real-to-complex over the last three axes: rows to nz//2+1 bins,
    then forward C2C along y and x (composed from the pinned 1D oracles)."""
    return _c2c_axis(_c2c_axis(r2c(x), -2, -1), -3, -1)


def c2r_3d(X, nz: int) -> np.ndarray:
    """Unscaled 3D complex-to-real: backward C2C along x and y of the half
    spectrum, then rows of nz//2+1 bins to nz samples."""
    return c2r(_c2c_axis(_c2c_axis(X, -3, +1), -2, +1), nz)


def c2c_3d(x, sign: int = -1) -> np.ndarray:
    """Unscaled 3D C2C over the last three axes (fastest first)."""
    y = c2c(np.asarray(x, dtype=np.complex128), sign)
    return _c2c_axis(_c2c_axis(y, -2, sign), -3, sign)


def dft_bins(x, bins, sign: int = -1) -> np.ndarray:
    """Direct O(n) evaluation of a few bins of one transform (cross-check)."""
    x = np.ascontiguousarray(x, dtype=np.complex128).reshape(-1)
    bins = np.ascontiguousarray(bins, dtype=np.int64)
    out = np.empty(bins.shape[0], dtype=np.complex128)
    _check(_load().orc_dft_bins(_dptr(x), x.shape[0], bins.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                bins.shape[0], int(sign), _dptr(out)), "dft_bins")
    return out


# ------------------------------------------------------- FP32 reference port
def port_c2c(x, sign: int = -1, nthreads: int = 0) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.complex64)
    n = x.shape[-1]
    out = np.empty_like(x)
    _check(_load().port_c2c(_fptr(x.view(np.float32)), _fptr(out.view(np.float32)), n, x.size // n,
                            int(sign), int(nthreads)), "port_c2c")
    return out


def port_r2c(x, nthreads: int = 0) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    n = x.shape[-1]
    out = np.empty(x.shape[:-1] + (n // 2 + 1,), dtype=np.complex64)
    _check(_load().port_r2c(_fptr(x), _fptr(out.view(np.float32)), n, x.size // n, int(nthreads)), "port_r2c")
    return out


def port_c2r(X, n: int, nthreads: int = 0) -> np.ndarray:
    X = np.ascontiguousarray(X, dtype=np.complex64)
    out = np.empty(X.shape[:-1] + (n,), dtype=np.float32)
    _check(_load().port_c2r(_fptr(X.view(np.float32)), _fptr(out), n, X.size // (n // 2 + 1), int(nthreads)),
           "port_c2r")
    return out


def num_threads() -> int:
    return int(_load().orc_num_threads())


# ------------------------------------------------------------------- metrics
def comparison_details(output, golden, atol: float, rtol: float):
    """The reference's compare rule over interleaved float arrays.

    Restates src/common/host/test_helper.py:41-71: float64 arithmetic,
    ``max_abs``, ``rel_l2 = |out - gold| / |gold|`` (absolute norm when the
    golden is all zero) and ``mismatch = #(|diff| > atol)``; a case passes
    when there is no mismatch and rel_l2 <= rtol.  Non-finite values and
    size mismatches fail.
    """
    o = np.asarray(output).reshape(-1)
    g = np.asarray(golden).reshape(-1)
    if np.iscomplexobj(o):
        o = o.astype(np.complex128).view(np.float64)
    if np.iscomplexobj(g):
        g = g.astype(np.complex128).view(np.float64)
    o = o.astype(np.float64)
    g = g.astype(np.float64)
    if o.size == 0 or g.size == 0 or o.size != g.size:
        return False, {"detail": f"size mismatch or empty ({o.size} vs {g.size})"}
    if not (np.all(np.isfinite(o)) and np.all(np.isfinite(g))):
        return False, {"detail": "non-finite values"}
    diff = np.abs(o - g)
    max_abs = float(diff.max())
    gn = float(np.linalg.norm(g))
    dn = float(np.linalg.norm(o - g))
    rel = dn / gn if gn > 0 else dn
    mismatch = int(np.count_nonzero(diff > atol))
    passed = mismatch == 0 and rel <= rtol
    return passed, {"max_abs": max_abs, "rel_l2": rel, "mismatch": mismatch, "atol": atol, "rtol": rtol}


def errors(output, exact):
    """rel-L2 and max-abs error of ``output`` against an FP64 ``exact``."""
    o = np.asarray(output).astype(np.complex128 if np.iscomplexobj(output) else np.float64).reshape(-1)
    e = np.asarray(exact).astype(np.complex128 if np.iscomplexobj(exact) else np.float64).reshape(-1)
    d = o - e
    en = float(np.linalg.norm(e))
    return {"rel_l2": float(np.linalg.norm(d)) / en if en > 0 else float(np.linalg.norm(d)),
            "max_abs": float(np.abs(d).max()) if d.size else 0.0}


# ------------------------------------------------------ plan-time arithmetic
def ordered_factorize(n: int) -> list[int]:
    """Trial-division prime factors in ascending order.

    Restates orderedFactorize, src/common/host/fft_exec_helper.h:79-100.
    """
    factors = []
    if n <= 0:
        return factors
    bound = int(math.isqrt(n))
    f = 2
    while f <= bound:
        if n % f == 0:
            factors.append(f)
            n //= f
            bound = int(math.isqrt(n))
        else:
            f += 1
    if n != 1:
        factors.append(n)
    return factors


RADIX_MIX = (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47)


def choose_radix(is_c2c: bool, n: int) -> int:
    """2 for powers of two (C2C only), -2 for primes <= 47, -1 otherwise.

    Restates deDuplicates/Support/ChooseRadix, fft_exec_helper.h:102-139.
    """
    uniq = sorted(set(ordered_factorize(n)))
    if is_c2c and all(f == 2 for f in uniq):
        return 2
    if all(f in RADIX_MIX for f in uniq):
        return -2
    return -1


def stockham_index_maps(radices):
    """Per-pass (read, write) index arrays of the autosort Stockham form.

    Pass with radix r after a product ``prev`` of earlier radices, over a
    length-L sequence with ``part = L // r``: butterfly ``idx`` reads
    ``x[idx + k*part]`` (k < r) and writes ``y[block*len + q*prev + j]``
    with ``block = idx // prev``, ``j = idx % prev``, ``len = prev*r``
    (src/fft1_d/arch35/mix/fft1_d_c2c_mix_kernel.h:29-120).
    Returns a list of (read[part, r], write[part, r]) int64 arrays.
    """
    L = int(np.prod(radices))
    maps = []
    prev = 1
    for r in radices:
        part = L // r
        idx = np.arange(part, dtype=np.int64)[:, None]
        k = np.arange(r, dtype=np.int64)[None, :]
        read = idx + k * part
        block, j = idx // prev, idx % prev
        write = block * (prev * r) + k * prev + j
        maps.append((read, write))
        prev *= r
    return maps


def stockham_simulate_exact(x, radices, sign: int = -1):
    """Run the Stockham passes in exact rational-free FP64 using the maps.

    Twiddle of butterfly j and input k in a pass is W_{prev*r}^{j*k}.  Used
    to check that the index maps compose to a natural-order DFT.
    """
    a = np.asarray(x, dtype=np.complex128).copy()
    prev = 1
    for (read, write), r in zip(stockham_index_maps(radices), radices):
        part = read.shape[0]
        j = (np.arange(part) % prev)[:, None]
        k = np.arange(r)[None, :]
        tw = np.exp(sign * 2j * np.pi * ((j * k) % (prev * r)) / (prev * r))
        v = a[read] * tw
        q = np.arange(r)
        D = np.exp(sign * 2j * np.pi * ((q[:, None] * q[None, :]) % r) / r)
        y = v @ D.T
        b = np.empty_like(a)
        b[write] = y
        a = b
        prev *= r
    return a
