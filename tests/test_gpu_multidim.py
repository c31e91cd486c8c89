"""GPU parity of the multi-dimensional transforms beyond the reference's 2D
C2C: 2D R2C/C2R (batched, rows through the 1D real kernels, columns over the
half spectrum) and 3D C2C, all through the C ABI, against the FP64 oracle at
the FP32 bound (rel-L2 <= 1e-5), with their adjoints against torch's FP64
autograd and in-place calls against out-of-place ones."""
import numpy as np
import pytest

import aclfft as A
import oracle as O

pytestmark = pytest.mark.gpu

REL_FP32 = 1e-5

torch = pytest.importorskip("torch")


def _dev():
    return torch.device("cuda:0")


def _ok(out, exact, what, bound=REL_FP32):
    e = O.errors(out, exact)
    assert e["rel_l2"] <= bound, (what, e)


REAL_2D = [(2, 64, 128), (3, 7, 3000), (1, 30, 999), (2, 256, 1000), (1, 5, 1), (4, 1, 64), (1, 2048, 2048),
           (2, 3, 1 << 17), (1, 4, 1 << 20), (5, 9, 8192), (3, 128, 33), (1, 1000, 26624),
           (3, 512, 300), (2, 1024, 130)]


@pytest.mark.parametrize("b,nx,ny", REAL_2D)
def test_2d_r2c_c2r_vs_fp64(b, nx, ny):
    rng = np.random.default_rng(nx * 7 + ny)
    x = rng.standard_normal((b, nx, ny)).astype(np.float32)
    nb = ny // 2 + 1
    with A.Plan.plan2d(b, nx, ny, A.R2C) as p:
        assert p.info().supported
        X = np.empty((b, nx, nb), dtype=np.complex64)
        p.exec_r2c(x, X)  # host buffers
    _ok(X, O.r2c_2d(x), ("2d r2c", b, nx, ny))
    # a general half spectrum (not Hermitian in its DC / Nyquist columns)
    Y = (rng.standard_normal((b, nx, nb)) + 1j * rng.standard_normal((b, nx, nb))).astype(np.complex64)
    with A.Plan.plan2d(b, nx, ny, A.C2R) as p:
        assert p.info().supported
        y = np.empty((b, nx, ny), dtype=np.float32)
        p.exec_c2r(Y, y)
        Yd = torch.from_numpy(Y).to(_dev())
        yd = torch.empty((b, nx, ny), dtype=torch.float32, device=_dev())
        p.set_stream(torch.cuda.current_stream())
        p.exec_c2r(Yd, yd)
        torch.cuda.synchronize()
        assert np.array_equal(yd.cpu().numpy(), y)
        assert torch.equal(Yd.cpu(), torch.from_numpy(Y))  # the input stays intact
    _ok(y, O.c2r_2d(Y, ny), ("2d c2r", b, nx, ny))


@pytest.mark.parametrize("b,nx,ny", [(2, 64, 128), (1, 30, 999), (3, 256, 1000), (1, 4, 1 << 20)])
def test_2d_real_inplace_matches_out_of_place(b, nx, ny):
    """In-place calls: R2C reads packed real rows from the start of the
    buffer, C2R reads the half spectrum; both equal the out-of-place result."""
    nb = ny // 2 + 1
    g = torch.Generator().manual_seed(nx + ny)
    x = torch.randn((b, nx, ny), generator=g).to(_dev())
    X = torch.empty((b, nx, nb), dtype=torch.complex64, device=_dev())
    buf = torch.zeros(b * nx * nb * 2, dtype=torch.float32, device=_dev())
    buf[: b * nx * ny] = x.reshape(-1)
    with A.Plan.plan2d(b, nx, ny, A.R2C) as p:
        p.set_stream(torch.cuda.current_stream())
        p.exec_r2c(x, X)
        p.exec_r2c(buf, buf)
        torch.cuda.synchronize()
    assert torch.equal(torch.view_as_complex(buf.view(b, nx, nb, 2)), X)
    with A.Plan.plan2d(b, nx, ny, A.C2R) as p:
        p.set_norm(A.NORM_BACKWARD)
        p.set_stream(torch.cuda.current_stream())
        y = torch.empty((b, nx, ny), dtype=torch.float32, device=_dev())
        p.exec_c2r(X, y)
        p.exec_c2r(buf, buf)
        torch.cuda.synchronize()
    assert torch.equal(buf[: b * nx * ny].view(b, nx, ny), y)
    _ok(y.cpu().numpy(), x.cpu().numpy(), ("2d real round trip", b, nx, ny))


@pytest.mark.parametrize("nx,ny", [(8, 16), (5, 9), (6, 7)])
def test_2d_real_adjoints_against_torch(nx, ny):
    """dL/dx of L = sum w |rfft2(x)|^2 and dL/dX of L = sum v * irfft2(X) * nx ny
    from torch's FP64 autograd, against ExecR2CAdjoint / ExecC2RAdjoint."""
    b = 3
    nb = ny // 2 + 1
    rng = np.random.default_rng(nx * ny)
    x = rng.standard_normal((b, nx, ny))
    w = rng.uniform(0, 1, (b, nx, nb))
    xt = torch.tensor(x, requires_grad=True)
    (torch.tensor(w) * torch.fft.rfft2(xt).abs() ** 2).sum().backward()
    Xbar = (2 * w * np.fft.rfft2(x)).astype(np.complex64)
    out = np.empty((b, nx, ny), dtype=np.float32)
    with A.Plan.plan2d(b, nx, ny, A.R2C) as p:
        p.exec_r2c_adjoint(Xbar, out)
    _ok(out, xt.grad.numpy(), ("2d r2c adjoint", nx, ny))

    X = rng.standard_normal((b, nx, nb)) + 1j * rng.standard_normal((b, nx, nb))
    v = rng.standard_normal((b, nx, ny))
    Xt = torch.tensor(X, requires_grad=True)
    (torch.tensor(v) * torch.fft.irfft2(Xt, s=(nx, ny)) * (nx * ny)).sum().backward()
    gout = np.empty((b, nx, nb), dtype=np.complex64)
    with A.Plan.plan2d(b, nx, ny, A.C2R) as p:
        p.exec_c2r_adjoint(v.astype(np.float32), gout)
    _ok(gout, Xt.grad.numpy(), ("2d c2r adjoint", nx, ny))


DIMS_3D = [(64, 64, 64), (7, 5, 3000), (3000, 7, 5), (5, 3000, 7), (2, 2, 2), (1, 1, 1), (5, 30, 64), (16, 1, 65536),
           (128, 128, 128), (1, 64, 1), (32, 48, 1000)]


@pytest.mark.parametrize("dims", DIMS_3D)
def test_3d_c2c_vs_fp64(dims):
    rng = np.random.default_rng(sum(dims))
    x = (rng.standard_normal(dims) + 1j * rng.standard_normal(dims)).astype(np.complex64)
    xd = torch.from_numpy(x).to(_dev())
    yd = torch.empty_like(xd)
    with A.Plan.plan3d(*dims) as p:
        assert p.info().supported
        p.set_stream(torch.cuda.current_stream())
        for d in (A.FORWARD, A.BACKWARD):
            p.exec_c2c(xd, yd, d)
            torch.cuda.synchronize()
            _ok(yd.cpu().numpy(), O.c2c_3d(x, d), ("3d", dims, d))
        zd = xd.clone()
        p.exec_c2c(zd, zd, A.FORWARD)
        p.exec_c2c(xd, yd, A.FORWARD)
        torch.cuda.synchronize()
        assert torch.equal(zd, yd)
        h = np.empty_like(x)
        p.exec_c2c(x, h, A.FORWARD)  # host buffers
        assert np.array_equal(h, yd.cpu().numpy())


def test_3d_512_cube_round_trip_and_norms():
    """A 1 GiB volume: forward then normalised inverse returns the input, and
    one 2D slice of the forward output matches the oracle's transform of the
    x-summed volume (the kx = 0 plane)."""
    n = 512
    g = torch.Generator(device=_dev()).manual_seed(5)
    x = torch.complex(torch.rand((n, n, n), generator=g, device=_dev()) * 2 - 1,
                      torch.rand((n, n, n), generator=g, device=_dev()) * 2 - 1)
    y = torch.empty_like(x)
    with A.Plan.plan3d(n, n, n) as p:
        p.set_stream(torch.cuda.current_stream())
        p.exec_c2c(x, y, A.FORWARD)
        torch.cuda.synchronize()
        plane = y[0].cpu().numpy()
        xs = x.to(torch.complex128).sum(dim=0).cpu().numpy()
        _ok(plane, O.c2c_2d(xs, -1), "3d kx=0 plane")
        p.set_norm(A.NORM_BACKWARD)
        p.exec_c2c(y, y, A.BACKWARD)
        torch.cuda.synchronize()
    e = (y - x).abs().pow(2).sum().sqrt() / x.abs().pow(2).sum().sqrt()
    assert float(e) <= REL_FP32, float(e)


@pytest.mark.parametrize("mode", [A.NORM_ORTHO, A.NORM_FORWARD])
def test_3d_norm_and_adjoint(mode):
    dims = (6, 10, 12)
    n = int(np.prod(dims))
    rng = np.random.default_rng(mode)
    x = (rng.standard_normal(dims) + 1j * rng.standard_normal(dims)).astype(np.complex64)
    y = np.empty_like(x)
    scale = 1 / np.sqrt(n) if mode == A.NORM_ORTHO else 1 / n
    with A.Plan.plan3d(*dims) as p:
        p.set_norm(mode)
        p.exec_c2c(x, y, A.FORWARD)
        _ok(y, O.c2c_3d(x, -1) * scale, ("3d norm", mode))
        # <F x, G> = <x, F^H G>
        G = (rng.standard_normal(dims) + 1j * rng.standard_normal(dims)).astype(np.complex64)
        a = np.empty_like(x)
        p.exec_c2c_adjoint(G, a, A.FORWARD)
    lhs = np.vdot(G.astype(np.complex128), O.c2c_3d(x, -1) * scale)
    rhs = np.vdot(a.astype(np.complex128), x.astype(np.complex128))
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs), (lhs, rhs)


@pytest.mark.parametrize("dims", [(8, 12, 20), (5, 7, 9), (16, 1, 64), (1, 6, 31), (64, 64, 64), (3, 5, 4096),
                                  (4, 512, 96), (512, 8, 30), (256, 256, 256)])
def test_3d_r2c_c2r_vs_fp64(dims):
    """3D real transforms: rows through the 1D real path, then the y and x
    axes as column passes over the half spectrum (C2R: columns first, into
    the second work area), against the FP64 oracle, host buffers and in
    place on the device."""
    nz = dims[-1]
    nb = nz // 2 + 1
    half = dims[:-1] + (nb,)
    rng = np.random.default_rng(sum(dims) + 5)
    x = rng.standard_normal(dims).astype(np.float32)
    X = np.empty(half, dtype=np.complex64)
    with A.Plan.plan3d(*dims, A.R2C) as p:
        p.exec_r2c(x, X)
    _ok(X, O.r2c_3d(x), ("3d r2c", dims))
    Y = (rng.standard_normal(half) + 1j * rng.standard_normal(half)).astype(np.complex64)
    y = np.empty(dims, dtype=np.float32)
    with A.Plan.plan3d(*dims, A.C2R) as p:
        p.exec_c2r(Y, y)
        buf = torch.zeros(int(np.prod(half)) * 2, dtype=torch.float32, device=_dev())
        torch.view_as_complex(buf.view(*half, 2)).copy_(torch.from_numpy(Y).to(_dev()))
        p.set_stream(torch.cuda.current_stream())
        p.exec_c2r(buf, buf)  # in place
        torch.cuda.synchronize()
        assert np.array_equal(buf[: x.size].view(*dims).cpu().numpy(), y)
    _ok(y, O.c2r_3d(Y, nz), ("3d c2r", dims))
