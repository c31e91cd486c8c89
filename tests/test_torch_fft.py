"""GPU tests of the torch.autograd wrappers (ops-fft_gb300/torch_fft.py) over
the C ABI: forward values against torch.fft, and gradients of real losses
through loss.backward() against torch.fft's own autograd in FP64 and
against FP64 central finite differences of the oracle.  Tolerances: the
plain-FP32 bound, rel-L2 <= 1e-5."""
import threading

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

REL = 1e-5


def _rel(a, b):
    a = np.asarray(a, dtype=np.complex128).reshape(-1)
    b = np.asarray(b, dtype=np.complex128).reshape(-1)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _fd(f, x, h=1e-6):
    g = np.zeros_like(x)
    for i in range(x.size):
        e = np.zeros_like(x)
        e.flat[i] = h
        g.flat[i] = (f(x + e) - f(x - e)) / (2 * h)
    return g


@pytest.fixture(scope="module")
def F():
    import torch_fft

    yield torch_fft
    torch_fft.clear_cache()


@pytest.mark.parametrize("n", [64, 63])
def test_rfft_forward_and_gradient(F, n):
    b = 4
    rng = np.random.default_rng(n)
    x = rng.standard_normal((b, n))
    w = rng.uniform(0, 1, (b, n // 2 + 1))
    xd = torch.tensor(x, dtype=torch.float32, device="cuda", requires_grad=True)
    X = F.rfft(xd)
    loss = (torch.tensor(w, dtype=torch.float32, device="cuda") * X.abs() ** 2).sum()
    loss.backward()
    assert _rel(X.detach().cpu().numpy(), O.r2c(x)) <= REL
    xt = torch.tensor(x, dtype=torch.float64, requires_grad=True)
    (torch.tensor(w) * torch.fft.rfft(xt).abs() ** 2).sum().backward()
    g = xd.grad.cpu().numpy()
    assert _rel(g, xt.grad.numpy()) <= REL
    gfd = _fd(lambda v: float(np.sum(w * np.abs(O.r2c(v.reshape(b, n))) ** 2)), x.reshape(-1)).reshape(b, n)
    assert _rel(g, gfd) <= REL


@pytest.mark.parametrize("n", [64, 63])
def test_irfft_forward_and_gradient(F, n):
    b = 4
    nb = n // 2 + 1
    rng = np.random.default_rng(n + 1)
    X = rng.standard_normal((b, nb)) + 1j * rng.standard_normal((b, nb))
    v = rng.standard_normal((b, n))
    Xd = torch.tensor(X, dtype=torch.complex64, device="cuda", requires_grad=True)
    y = F.irfft(Xd, n)
    loss = (torch.tensor(v, dtype=torch.float32, device="cuda") * y).sum()
    loss.backward()
    assert _rel(y.detach().cpu().numpy(), O.c2r(X, n)) <= REL
    Xt = torch.tensor(X, dtype=torch.complex128, requires_grad=True)
    (torch.tensor(v) * torch.fft.irfft(Xt, n=n) * n).sum().backward()
    g = Xd.grad.cpu().numpy()
    assert _rel(g, Xt.grad.numpy()) <= REL

    def L(u):
        Z = u[: u.size // 2] + 1j * u[u.size // 2:]
        return float(np.sum(v * O.c2r(Z.reshape(b, nb), n)))

    u0 = np.concatenate([X.real.reshape(-1), X.imag.reshape(-1)])
    gg = _fd(L, u0)
    assert _rel(g, (gg[: u0.size // 2] + 1j * gg[u0.size // 2:]).reshape(b, nb)) <= REL


@pytest.mark.parametrize("n,inverse", [(64, False), (63, True)])
def test_fft_forward_and_gradient(F, n, inverse):
    b = 4
    rng = np.random.default_rng(n + 2)
    z = rng.standard_normal((b, n)) + 1j * rng.standard_normal((b, n))
    G = rng.standard_normal((b, n)) + 1j * rng.standard_normal((b, n))
    zd = torch.tensor(z, dtype=torch.complex64, device="cuda", requires_grad=True)
    Z = F.fft(zd, inverse=inverse)
    loss = torch.real(torch.conj(torch.tensor(G, dtype=torch.complex64, device="cuda")) * Z).sum()
    loss.backward()
    sign = 1 if inverse else -1
    assert _rel(Z.detach().cpu().numpy(), O.c2c(z, sign)) <= REL
    zt = torch.tensor(z, dtype=torch.complex128, requires_grad=True)
    Zt = torch.fft.ifft(zt) * n if inverse else torch.fft.fft(zt)
    torch.real(torch.conj(torch.tensor(G)) * Zt).sum().backward()
    assert _rel(zd.grad.cpu().numpy(), zt.grad.numpy()) <= REL


def test_plans_are_per_stream_and_threads_do_not_race(F):
    """Two threads, each on its own stream, transform the same shape
    concurrently many times: each stream has its own cached plan (stream and
    workspace), so every result is right."""
    n, b = 1 << 20, 2       # a long length: its plan uses a workspace between passes
    rng = np.random.default_rng(7)
    xs = [(rng.standard_normal((b, n)) + 1j * rng.standard_normal((b, n))).astype(np.complex64) for _ in range(2)]
    exact = [O.c2c(x, -1) for x in xs]
    results = [None, None]
    errors = []

    def work(i):
        try:
            s = torch.cuda.Stream()
            with torch.cuda.stream(s):
                xd = torch.from_numpy(xs[i]).cuda()
                for _ in range(20):
                    y = F.fft(xd)
                s.synchronize()
                results[i] = y.cpu().numpy()
        except Exception as e:  # pragma: no cover - reported below
            errors.append(e)

    ts = [threading.Thread(target=work, args=(i,)) for i in range(2)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errors, errors
    for i in range(2):
        assert _rel(results[i], exact[i]) <= REL


@pytest.mark.parametrize("shape", [(3, 16, 12), (2, 9, 7), (1, 64, 1000)])
def test_rfft2_irfft2_forward_and_gradient(F, shape):
    """2D real wrappers: values against torch.fft.rfft2 / irfft2 and
    gradients of L = sum w|rfft2(x)|^2 + sum v * irfft2(X) against FP64
    autograd."""
    nx, ny = shape[-2:]
    rng = np.random.default_rng(nx + ny)
    x = rng.standard_normal(shape)
    w = rng.uniform(0, 1, shape[:-1] + (ny // 2 + 1,))
    v = rng.standard_normal(shape)
    xd = torch.tensor(x, dtype=torch.float32, device="cuda", requires_grad=True)
    X = F.rfft2(xd)
    y = F.irfft2(X, (nx, ny))
    loss = (torch.tensor(w, dtype=torch.float32, device="cuda") * X.abs() ** 2).sum() + \
        (torch.tensor(v, dtype=torch.float32, device="cuda") * y).sum()
    loss.backward()
    assert _rel(X.detach().cpu().numpy(), np.fft.rfft2(x)) <= REL
    assert _rel(y.detach().cpu().numpy(), x * nx * ny) <= REL
    xt = torch.tensor(x, requires_grad=True)
    Xt = torch.fft.rfft2(xt)
    yt = torch.fft.irfft2(Xt, s=(nx, ny)) * (nx * ny)
    ((torch.tensor(w) * Xt.abs() ** 2).sum() + (torch.tensor(v) * yt).sum()).backward()
    assert _rel(xd.grad.cpu().numpy(), xt.grad.numpy()) <= REL
    with pytest.raises(ValueError):
        F.irfft2(X, (nx, ny + 2))


@pytest.mark.parametrize("inverse", [False, True])
def test_fft2_fftn_forward_and_gradient(F, inverse):
    rng = np.random.default_rng(int(inverse))
    for shape, fn, tfn, axes in (((2, 12, 20), F.fft2, torch.fft.fft2, (-2, -1)),
                                 ((3, 6, 10, 14), F.fftn, torch.fft.fftn, (-3, -2, -1))):
        z = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
        G = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
        zd = torch.tensor(z, dtype=torch.complex64, device="cuda", requires_grad=True)
        Z = fn(zd, inverse=inverse)
        torch.real(torch.conj(torch.tensor(G, dtype=torch.complex64, device="cuda")) * Z).sum().backward()
        npts = int(np.prod([shape[a] for a in axes]))
        zt = torch.tensor(z, requires_grad=True)
        Zt = (torch.fft.ifftn(zt, dim=axes) * npts) if inverse else tfn(zt, dim=axes)
        torch.real(torch.conj(torch.tensor(G)) * Zt).sum().backward()
        assert _rel(Z.detach().cpu().numpy(), Zt.detach().numpy()) <= REL, shape
        assert _rel(zd.grad.cpu().numpy(), zt.grad.numpy()) <= REL, shape


@pytest.mark.parametrize("n", [64, 63])
def test_double_precision_wrappers_and_gradients(F, n):
    """complex128 / float64 tensors go through the double-precision entries:
    values against torch.fft in FP64 at 1e-12, and gradients of real losses
    through fft, rfft and irfft against torch's FP64 autograd."""
    rng = np.random.default_rng(n)
    b = 4
    z = rng.standard_normal((b, n)) + 1j * rng.standard_normal((b, n))
    x = rng.standard_normal((b, n))
    G = rng.standard_normal((b, n)) + 1j * rng.standard_normal((b, n))
    w = rng.uniform(0, 1, (b, n // 2 + 1))
    v = rng.standard_normal((b, n))
    zd = torch.tensor(z, device="cuda", requires_grad=True)
    xd = torch.tensor(x, device="cuda", requires_grad=True)
    Z = F.fft(zd)
    X = F.rfft(xd)
    y = F.irfft(X, n)
    assert Z.dtype == torch.complex128 and X.dtype == torch.complex128 and y.dtype == torch.float64
    loss = torch.real(torch.conj(torch.tensor(G, device="cuda")) * Z).sum() + \
        (torch.tensor(w, device="cuda") * X.abs() ** 2).sum() + (torch.tensor(v, device="cuda") * y).sum()
    loss.backward()
    zt = torch.tensor(z, requires_grad=True)
    xt = torch.tensor(x, requires_grad=True)
    Zt = torch.fft.fft(zt)
    Xt = torch.fft.rfft(xt)
    yt = torch.fft.irfft(Xt, n=n) * n
    (torch.real(torch.conj(torch.tensor(G)) * Zt).sum() + (torch.tensor(w) * Xt.abs() ** 2).sum() +
     (torch.tensor(v) * yt).sum()).backward()
    assert _rel(Z.detach().cpu().numpy(), Zt.detach().numpy()) <= 1e-12
    assert _rel(X.detach().cpu().numpy(), Xt.detach().numpy()) <= 1e-12
    assert _rel(y.detach().cpu().numpy(), yt.detach().numpy()) <= 1e-12
    assert _rel(zd.grad.cpu().numpy(), zt.grad.numpy()) <= 1e-12
    assert _rel(xd.grad.cpu().numpy(), xt.grad.numpy()) <= 1e-12


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_rfftn_irfftn_forward_and_gradient(F, dtype):
    """3D real wrappers in both precisions (batched volumes): values against
    numpy and gradients of L = sum w|rfftn(x)|^2 + sum v * irfftn(X) against
    torch's FP64 autograd."""
    shape = (2, 6, 10, 12)
    nx, ny, nz = shape[1:]
    tol = REL if dtype == torch.float32 else 1e-12
    rng = np.random.default_rng(17)
    x = rng.standard_normal(shape)
    w = rng.uniform(0, 1, shape[:-1] + (nz // 2 + 1,))
    v = rng.standard_normal(shape)
    xd = torch.tensor(x, dtype=dtype, device="cuda", requires_grad=True)
    X = F.rfftn(xd)
    y = F.irfftn(X, (nx, ny, nz))
    loss = (torch.tensor(w, dtype=dtype, device="cuda") * X.abs() ** 2).sum() + \
        (torch.tensor(v, dtype=dtype, device="cuda") * y).sum()
    loss.backward()
    axes = (-3, -2, -1)
    assert _rel(X.detach().cpu().numpy(), np.fft.rfftn(x, axes=axes)) <= tol
    assert _rel(y.detach().cpu().numpy(), x * nx * ny * nz) <= tol
    xt = torch.tensor(x, requires_grad=True)
    Xt = torch.fft.rfftn(xt, dim=axes)
    yt = torch.fft.irfftn(Xt, s=(nx, ny, nz), dim=axes) * (nx * ny * nz)
    ((torch.tensor(w) * Xt.abs() ** 2).sum() + (torch.tensor(v) * yt).sum()).backward()
    assert _rel(xd.grad.cpu().numpy(), xt.grad.numpy()) <= tol
