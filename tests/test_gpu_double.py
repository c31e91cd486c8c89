"""GPU parity of the double-precision transforms (Z2Z, D2Z and Z2D of rank
1-3) through the C ABI against the FP64 oracle.  The reference declares
these entries and leaves them as stubs, so parity is against the oracle
only.  Tolerance: rel-L2 <= 1e-12 (FP64 arithmetic and FP64 twiddles; the
errors seen are ~1e-15)."""
import numpy as np
import pytest

import aclfft as A
import oracle as O

pytestmark = pytest.mark.gpu

REL_FP64 = 1e-12

torch = pytest.importorskip("torch")


def _dev():
    return torch.device("cuda:0")


def _ok(out, exact, what):
    e = O.errors(out, exact)
    assert e["rel_l2"] <= REL_FP64, (what, e)


LENGTHS = [1, 2, 3, 7, 16, 47, 64, 210, 1000, 1536, 2021, 3000, 4096, 46200, 47 * 43, 1 << 20]


@pytest.mark.parametrize("n", LENGTHS)
def test_z2z_lengths_both_directions(n):
    b = max(1, min(16, (1 << 21) // n))
    rng = np.random.default_rng(n)
    x = rng.standard_normal((b, n)) + 1j * rng.standard_normal((b, n))
    xd = torch.from_numpy(x).to(_dev())
    yd = torch.empty_like(xd)
    with A.Plan.plan1d(n, A.Z2Z, b) as p:
        assert p.info().supported
        p.set_stream(torch.cuda.current_stream())
        for d in (A.FORWARD, A.BACKWARD):
            p.exec_z2z(xd, yd, d)
            torch.cuda.synchronize()
            _ok(yd.cpu().numpy(), O.c2c(x, d), ("z2z", n, d))
        zd = xd.clone()
        p.exec_z2z(zd, zd, A.FORWARD)  # in place
        p.set_norm(A.NORM_BACKWARD)
        p.exec_z2z(zd, zd, A.BACKWARD)  # and back, scaled by 1/n in FP64
        torch.cuda.synchronize()
        _ok(zd.cpu().numpy(), x, ("z2z round trip", n))
        h = np.empty_like(x)
        p.set_norm(A.NORM_NONE)
        p.exec_z2z(x, h, A.FORWARD)  # host buffers
        _ok(h, O.c2c(x, -1), ("z2z host", n))


@pytest.mark.parametrize("n", [1, 2, 3, 4, 7, 8, 999, 1000, 3000, 4096, 65536, 26624])
def test_d2z_z2d_lengths(n):
    b = max(1, min(16, (1 << 20) // n))
    nb = n // 2 + 1
    rng = np.random.default_rng(n + 1)
    x = rng.standard_normal((b, n))
    X = np.empty((b, nb), dtype=np.complex128)
    with A.Plan.plan1d(n, A.D2Z, b) as p:
        p.exec_d2z(x, X)
    _ok(X, O.r2c(x), ("d2z", n))
    assert np.all(X[:, 0].imag == 0)
    # a general half spectrum: the imaginary parts of DC / Nyquist are ignored
    Y = rng.standard_normal((b, nb)) + 1j * rng.standard_normal((b, nb))
    y = np.empty((b, n))
    with A.Plan.plan1d(n, A.Z2D, b) as p:
        p.exec_z2d(Y, y)
    _ok(y, O.c2r(Y, n), ("z2d", n))


@pytest.mark.parametrize("n,b", [(3000, 64), (1024, 33), (7, 5)])
def test_d2z_z2d_device_and_inplace(n, b):
    """Device buffers, and in-place calls (real rows at the start of a buffer
    large enough for the half spectrum) equal to out-of-place ones."""
    nb = n // 2 + 1
    g = torch.Generator().manual_seed(n)
    x = torch.randn((b, n), generator=g, dtype=torch.float64).to(_dev())
    X = torch.empty((b, nb), dtype=torch.complex128, device=_dev())
    buf = torch.zeros(b * nb * 2, dtype=torch.float64, device=_dev())
    buf[: b * n] = x.reshape(-1)
    with A.Plan.plan1d(n, A.D2Z, b) as p:
        p.set_stream(torch.cuda.current_stream())
        p.exec_d2z(x, X)
        p.exec_d2z(buf, buf)
        torch.cuda.synchronize()
    assert torch.equal(torch.view_as_complex(buf.view(b, nb, 2)), X)
    _ok(X.cpu().numpy(), O.r2c(x.cpu().numpy()), ("d2z device", n))
    with A.Plan.plan1d(n, A.Z2D, b) as p:
        p.set_norm(A.NORM_BACKWARD)
        p.set_stream(torch.cuda.current_stream())
        y = torch.empty((b, n), dtype=torch.float64, device=_dev())
        p.exec_z2d(X, y)
        p.exec_z2d(buf, buf)
        torch.cuda.synchronize()
    assert torch.equal(buf[: b * n].view(b, n), y)
    _ok(y.cpu().numpy(), x.cpu().numpy(), ("d2z/z2d round trip", n))


def test_z2z_vertical_and_multidim():
    rng = np.random.default_rng(3)
    # VERTICAL: 512-point transforms down the columns of [512][263]
    x = rng.standard_normal((512, 263)) + 1j * rng.standard_normal((512, 263))
    y = np.empty_like(x)
    with A.Plan.plan1d(512, A.Z2Z, 263, A.VERTICAL) as p:
        p.exec_z2z(x, y, A.FORWARD)
    _ok(y, O.c2c_vertical(x, -1), "z2z vertical")
    for b, nx, ny in ((3, 64, 100), (1, 1, 7), (2, 48, 1)):
        x = rng.standard_normal((b, nx, ny)) + 1j * rng.standard_normal((b, nx, ny))
        y = np.empty_like(x)
        with A.Plan.plan2d(b, nx, ny, A.Z2Z) as p:
            for d in (A.FORWARD, A.BACKWARD):
                p.exec_z2z(x, y, d)
                _ok(y, O.c2c_2d(x, d), ("z2z 2d", b, nx, ny, d))
    for dims in ((16, 24, 30), (5, 1, 8), (1, 1, 1)):
        x = rng.standard_normal(dims) + 1j * rng.standard_normal(dims)
        y = np.empty_like(x)
        with A.Plan.plan3d(*dims, A.Z2Z) as p:
            for d in (A.FORWARD, A.BACKWARD):
                p.exec_z2z(x, y, d)
                _ok(y, O.c2c_3d(x, d), ("z2z 3d", dims, d))


def test_unaligned_device_pointers_are_rejected():
    """Device pointers must be aligned to the complex element the kernels
    load (8 bytes FP32, 16 bytes FP64; real FP64 rows 8): otherwise the exec
    returns ACLFFT_UNALIGNED_DATA before any launch."""
    buf = torch.zeros(4096 + 4, dtype=torch.float64, device=_dev())
    base = buf.data_ptr()
    lib = A.lib()
    with A.Plan.plan1d(256, A.Z2Z, 2) as p:
        assert lib.aclfftExecZ2Z(p.handle, base + 8, base + 4096, A.FORWARD) == A.UNALIGNED_DATA
        assert lib.aclfftExecZ2Z(p.handle, base, base + 4096 + 8, A.FORWARD) == A.UNALIGNED_DATA
    with A.Plan.plan1d(256, A.D2Z, 2) as p:
        # real rows need 8 bytes only; the half spectrum 16
        assert lib.aclfftExecD2Z(p.handle, base + 8, base + 8192 - 8) == A.UNALIGNED_DATA
        torch.cuda.synchronize()
        assert lib.aclfftExecD2Z(p.handle, base + 8, base + 8192) == A.SUCCESS
        torch.cuda.synchronize()
    with A.Plan.plan1d(256, A.C2C, 2) as p:
        assert lib.aclfftExecC2C(p.handle, base + 4, base + 8192, A.FORWARD) == A.UNALIGNED_DATA


@pytest.mark.parametrize("b,nx,ny", [(3, 64, 100), (2, 7, 3000), (1, 30, 999), (2, 1, 64), (3, 5, 1), (2, 9, 4),
                                     (1, 256, 2048)])
def test_2d_d2z_z2d_vs_fp64(b, nx, ny):
    """2D double-precision real transforms: rows through the 1D real path,
    columns as Z2Z passes over the half spectrum (Z2D: columns first), host
    and device buffers, in place, against the FP64 oracle."""
    nb = ny // 2 + 1
    rng = np.random.default_rng(nx * 11 + ny)
    x = rng.standard_normal((b, nx, ny))
    X = np.empty((b, nx, nb), dtype=np.complex128)
    with A.Plan.plan2d(b, nx, ny, A.D2Z) as p:
        p.exec_d2z(x, X)
    _ok(X, O.r2c_2d(x), ("2d d2z", b, nx, ny))
    Y = rng.standard_normal((b, nx, nb)) + 1j * rng.standard_normal((b, nx, nb))
    y = np.empty((b, nx, ny))
    with A.Plan.plan2d(b, nx, ny, A.Z2D) as p:
        p.exec_z2d(Y, y)
        Yd = torch.from_numpy(Y).to(_dev())
        buf = torch.zeros(b * nx * nb * 2, dtype=torch.float64, device=_dev())
        torch.view_as_complex(buf.view(b, nx, nb, 2)).copy_(Yd)
        p.set_stream(torch.cuda.current_stream())
        p.exec_z2d(buf, buf)  # in place
        torch.cuda.synchronize()
        assert np.array_equal(buf[: b * nx * ny].view(b, nx, ny).cpu().numpy(), y)
    _ok(y, O.c2r_2d(Y, ny), ("2d z2d", b, nx, ny))


@pytest.mark.parametrize("dims", [(8, 12, 20), (5, 7, 9), (1, 6, 31)])
def test_3d_d2z_z2d_vs_fp64(dims):
    nz = dims[-1]
    half = dims[:-1] + (nz // 2 + 1,)
    rng = np.random.default_rng(sum(dims) + 9)
    x = rng.standard_normal(dims)
    X = np.empty(half, dtype=np.complex128)
    with A.Plan.plan3d(*dims, A.D2Z) as p:
        p.exec_d2z(x, X)
    _ok(X, O.r2c_3d(x), ("3d d2z", dims))
    Y = rng.standard_normal(half) + 1j * rng.standard_normal(half)
    y = np.empty(dims)
    with A.Plan.plan3d(*dims, A.Z2D) as p:
        p.exec_z2d(Y, y)
    _ok(y, O.c2r_3d(Y, nz), ("3d z2d", dims))
