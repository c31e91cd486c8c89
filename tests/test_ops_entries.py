"""The reference's per-operator direct entries (include/aclfft_ops.h).

CPU: argument validation, rule by rule, with the reference's codes (every
rejection is ACL_ERROR_INVALID_PARAM before any device work).  GPU: each
entry on host buffers (the reference's calling convention) against the
FP64 oracle at the plain-FP32 bound rel-L2 <= 1e-5, in place and out of
place, plus the reference's tolerances on its golden cases where one fits.
"""
import numpy as np
import pytest

import aclfft as A
import oracle as O

INV = A.ACL_ERROR_INVALID_PARAM
REL = 1e-5
STD_C2C = ["aclfftFft1DDft", "aclfftFft1DN", "aclfftFft1DB", "aclfftFft1DMix", "aclfftFft1DC2C", "aclfftFft1DC2CMix"]


def _buf(n=64):
    return np.zeros(4 * n, dtype=np.float32)


# ------------------------------------------------------------------- CPU
@pytest.mark.parametrize("name", STD_C2C)
def test_c2c_entries_reject_like_the_reference(name):
    f = getattr(A.lib(), name)
    b = _buf()
    p = b.ctypes.data
    assert f(None, p, 64, 0, 1, 1, None) == INV
    assert f(p, None, 64, 0, 1, 1, None) == INV
    assert f(p, p, 64, 1, 1, 1, None) == INV       # norm != 0
    assert f(p, p, 64, 0, 1, 2, None) == INV       # isForward not 0/1
    assert f(p, p, 64, 0, 1, -1, None) == INV
    assert f(p, p, 0, 0, 1, 1, None) == INV        # n = 0
    assert f(p, p, 256, 0, 0, 1, None) == INV      # batches = 0
    assert f(p, p, (1 << 27) + 1, 0, 1, 1, None) == INV


def test_family_domains():
    L = A.lib()
    b = _buf()
    p = b.ctypes.data
    assert L.aclfftFft1DDft(p, p, 1025, 0, 1, 1, None) == INV
    assert L.aclfftFft1DN(p, p, 32, 0, 1, 1, None) == INV          # below 64
    assert L.aclfftFft1DN(p, p, 96, 0, 1, 1, None) == INV          # not a power of two
    assert L.aclfftFft1DB(p, p, 128, 0, 1, 1, None) == INV
    assert L.aclfftFft1DB(p, p, 32768, 0, 1, 1, None) == INV
    assert L.aclfftFft1DB(p, p, 3000, 0, 1, 1, None) == INV
    # VERTICAL: one matrix, stride a multiple of 4, n a power of two in [2^8, 2^18]
    assert L.aclfftFft1DStride(p, p, 256, 0, 8, 2, 1, None) == INV
    assert L.aclfftFft1DStride(p, p, 256, 0, 0, 1, 1, None) == INV
    assert L.aclfftFft1DStride(p, p, 256, 0, 6, 1, 1, None) == INV
    assert L.aclfftFft1DStride(p, p, 128, 0, 8, 1, 1, None) == INV
    assert L.aclfftFft1DStride(p, p, 1 << 18, 0, 1 << 13, 1, 1, None) == INV   # n*stride > 2^30
    assert L.aclfftFft1DStride(p, p, 256, 1, 8, 1, 1, None) == INV
    # R2C: isForward must be 1, C2R: 0
    for name in ("aclfftRfft1DR2CFft", "aclfftRfft1DFft", "aclfftRfft1DDft"):
        assert getattr(L, name)(p, p, 64, 0, 1, 0, None) == INV
        assert getattr(L, name)(p, p, 64, 1, 1, 1, None) == INV
        assert getattr(L, name)(p, p, 0, 0, 1, 1, None) == INV
        assert getattr(L, name)(p, p, 64, 0, 0, 1, None) == INV
    assert L.aclfftRfft1DDft(p, p, 2048, 0, 1, 1, None) == INV
    for name in ("aclfftIrfft1DFft", "aclfftIrfft1DDft", "aclfftIrfft1DC2RFft"):
        assert getattr(L, name)(p, p, 64, 0, 1, 1, None) == INV
        assert getattr(L, name)(p, p, 64, 1, 1, 0, None) == INV
        assert getattr(L, name)(None, p, 64, 0, 1, 0, None) == INV
    assert L.aclfftIrfft1DDft(p, p, 1025, 0, 1, 0, None) == INV
    # FastDFT R2C: n <= 4096, norm 0..2, no isForward
    assert L.aclfftRfft1D(p, p, 4097, 0, 1, None) == INV
    assert L.aclfftRfft1D(p, p, 64, 3, 1, None) == INV
    assert L.aclfftRfft1D(p, p, 64, -1, 1, None) == INV
    assert L.aclfftRfft1D(p, p, 0, 0, 1, None) == INV
    # power-of-two R2C families
    for name in ("aclfftRfft1DR2CFft1", "aclfftRfft1DR2CFft2", "aclfftRfft1DR2CFft31", "aclfftRfft1DR2CFft32",
                 "aclfftRfft1DR2CFft4", "aclfftRfft1DR2CFft5"):
        f = getattr(L, name)
        assert f(p, p, 256, 1, 0, None) == INV         # isForward must be 1
        assert f(p, p, 3000, 1, 1, None) == INV        # not a power of two
        assert f(p, p, 0, 1, 1, None) == INV
        assert f(p, p, 256, 0, 1, None) == INV         # batches = 0
        assert f(p, p, 1 << 20, 4096, 1, None) == INV  # batches*(n+2) > 2^31
    assert L.aclfftRfft1DR2CFft2(p, p, 128, 1, 1, None) == INV
    assert L.aclfftRfft1DR2CFft2(p, p, 32768, 1, 1, None) == INV
    assert L.aclfftRfft1DR2CFft1(p, p, 1, 1, 1, None) == INV
    assert L.aclfftRfft1DR2CFft5(p, p, 2, 1, 1, None) == INV
    # 2D
    assert L.aclfftFft2DDd(p, p, 32, 32, 1, 2, None) == INV
    assert L.aclfftFft2DDd(p, p, 0, 32, 1, 1, None) == INV
    assert L.aclfftFft2DDd(p, p, 32, 32, 0, 1, None) == INV
    assert L.aclfftFft2DDd(None, p, 32, 32, 1, 1, None) == INV


# ------------------------------------------------------------------- GPU
def _cplx(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


def _ok(out, exact, what):
    e = O.errors(out, exact)
    assert e["rel_l2"] <= REL, (what, e)


@pytest.mark.gpu
@pytest.mark.parametrize("name,n,b", [("aclfftFft1DDft", 1000, 6), ("aclfftFft1DN", 1 << 16, 3), ("aclfftFft1DB", 4096, 9),
                                      ("aclfftFft1DMix", 3000, 5), ("aclfftFft1DC2C", 46200, 2),
                                      ("aclfftFft1DC2CMix", 2310, 7)])
def test_c2c_entries_vs_fp64(name, n, b):
    f = getattr(A.lib(), name)
    rng = np.random.default_rng(n)
    x = _cplx(rng, (b, n))
    for isf, sign in ((1, -1), (0, +1)):
        y = np.empty_like(x)
        assert f(x.ctypes.data, y.ctypes.data, n, 0, b, isf, None) == A.ACL_SUCCESS, A.last_error_detail()
        _ok(y, O.c2c(x, sign), (name, isf))
    z = x.copy()
    assert f(z.ctypes.data, z.ctypes.data, n, 0, b, 1, None) == A.ACL_SUCCESS
    _ok(z, O.c2c(x, -1), (name, "in place"))


@pytest.mark.gpu
def test_stride_entry_vs_fp64_and_reference_case():
    n, stride = 4096, 128   # the reference's stride_forward_n4096 shape
    rng = np.random.default_rng(3)
    x = _cplx(rng, (n, stride))
    y = np.empty_like(x)
    assert A.lib().aclfftFft1DStride(x.ctypes.data, y.ctypes.data, n, 0, stride, 1, 1, None) == A.ACL_SUCCESS
    _ok(y, O.c2c_vertical(x, -1), "stride forward")
    ok, det = O.comparison_details(y, O.c2c_vertical(x, -1), 1e-2, 1e-3)
    assert ok, det
    assert A.lib().aclfftFft1DStride(y.ctypes.data, y.ctypes.data, n, 0, stride, 1, 0, None) == A.ACL_SUCCESS
    _ok(y, n * x.astype(np.complex128), "stride round trip in place")


@pytest.mark.gpu
@pytest.mark.parametrize("name,n,b", [("aclfftRfft1DR2CFft", 3000, 8), ("aclfftRfft1DFft", 1025, 4),
                                      ("aclfftRfft1DDft", 1000, 16)])
def test_r2c_entries_vs_fp64(name, n, b):
    f = getattr(A.lib(), name)
    rng = np.random.default_rng(n + b)
    x = rng.standard_normal((b, n)).astype(np.float32)
    y = np.empty((b, n // 2 + 1), dtype=np.complex64)
    assert f(x.ctypes.data, y.ctypes.data, n, 0, b, 1, None) == A.ACL_SUCCESS, A.last_error_detail()
    _ok(y, O.r2c(x), name)
    buf = np.zeros(b * 2 * (n // 2 + 1), dtype=np.float32)
    buf[: b * n] = x.reshape(-1)
    assert f(buf.ctypes.data, buf.ctypes.data, n, 0, b, 1, None) == A.ACL_SUCCESS
    _ok(buf.view(np.complex64).reshape(b, n // 2 + 1), O.r2c(x), (name, "in place"))


@pytest.mark.gpu
@pytest.mark.parametrize("norm,scale", [(0, 1.0), (1, None), (2, None)])
def test_fastdft_r2c_norm_modes(norm, scale):
    n, b = 4096, 4
    rng = np.random.default_rng(norm)
    x = rng.standard_normal((b, n)).astype(np.float32)
    y = np.empty((b, n // 2 + 1), dtype=np.complex64)
    assert A.lib().aclfftRfft1D(x.ctypes.data, y.ctypes.data, n, norm, b, None) == A.ACL_SUCCESS
    s = {0: 1.0, 1: n ** -0.5, 2: 1.0 / n}[norm]
    _ok(y, s * O.r2c(x), ("Rfft1D", norm))


@pytest.mark.gpu
@pytest.mark.parametrize("name,n", [("aclfftRfft1DR2CFft1", 128), ("aclfftRfft1DR2CFft2", 16384),
                                    ("aclfftRfft1DR2CFft31", 65536), ("aclfftRfft1DR2CFft32", 1 << 21),
                                    ("aclfftRfft1DR2CFft4", 1 << 23), ("aclfftRfft1DR2CFft5", 1 << 26)])
def test_pow2_r2c_families_vs_fp64(name, n):
    b = max(1, min(16, (1 << 24) // n))
    rng = np.random.default_rng(n)
    x = rng.standard_normal((b, n)).astype(np.float32)
    y = np.empty((b, n // 2 + 1), dtype=np.complex64)
    assert getattr(A.lib(), name)(x.ctypes.data, y.ctypes.data, n, b, 1, None) == A.ACL_SUCCESS
    r = b - 1
    exact = O.r2c(x[r:r + 1])[0] if n <= (1 << 22) else O.r2c_long_rows(x[r])
    _ok(y[r], exact, name)


@pytest.mark.gpu
@pytest.mark.parametrize("name,n,b", [("aclfftIrfft1DFft", 3000, 6), ("aclfftIrfft1DDft", 999, 5),
                                      ("aclfftIrfft1DC2RFft", 1 << 16, 2)])
def test_c2r_entries_vs_fp64(name, n, b):
    f = getattr(A.lib(), name)
    rng = np.random.default_rng(n)
    X = _cplx(rng, (b, n // 2 + 1))
    y = np.empty((b, n), dtype=np.float32)
    assert f(X.ctypes.data, y.ctypes.data, n, 0, b, 0, None) == A.ACL_SUCCESS, A.last_error_detail()
    _ok(y, O.c2r(X, n), name)


@pytest.mark.gpu
@pytest.mark.parametrize("nx,ny,b", [(64, 128, 3), (32, 32, 2), (2048, 1000, 1)])
def test_fft2d_entry_vs_fp64(nx, ny, b):
    rng = np.random.default_rng(nx + ny)
    x = _cplx(rng, (b, nx, ny))
    for isf, sign in ((1, -1), (0, +1)):
        y = np.empty_like(x)
        assert A.lib().aclfftFft2DDd(x.ctypes.data, y.ctypes.data, nx, ny, b, isf, None) == A.ACL_SUCCESS
        for i in range(b):
            _ok(y[i], O.c2c_2d(x[i], sign), ("Fft2DDd", nx, ny, isf))
