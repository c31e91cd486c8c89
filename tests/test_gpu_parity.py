"""GPU parity tests: every transform goes through the C ABI of libops_fft.so
and is compared with the reference's golden vectors (its own compare rule
and tolerances) and with the FP64 oracle at the tight FP32 bound.

Tolerances (stated here, used below):
  * plain FP32 Stockham vs FP64 oracle: rel-L2 <= 1e-5 (the plain-FP32 target);
  * reference golden vectors: the reference's per-case atol/rtol
    (compare_data.py), which are looser.
"""
import numpy as np
import pytest

import aclfft as A
import oracle as O
from helpers import as_complex, cases, read_bin, regenerate

pytestmark = pytest.mark.gpu

REL_FP32 = 1e-5
MAX_REGEN_ELEMS = 1 << 26

torch = pytest.importorskip("torch")


def _dev():
    return torch.device("cuda:0")


# ------------------------------------------------------------ host harness
def c2c_host(n, b, x, direction, dim=A.HORIZONTAL):
    """The reference harness flow: Plan1d -> Exec on host buffers -> Destroy."""
    out = np.empty_like(x)
    with A.Plan.plan1d(n, A.C2C, b, dim) as p:
        p.exec_c2c(x, out, direction)
    return out


def _gold_ok(out, gold, c):
    ok, det = O.comparison_details(out, gold, c["atol"], c["rtol"])
    assert ok, (c["name"], det)


def _fp64_ok(out, exact, bound=REL_FP32, what=""):
    e = O.errors(out, exact)
    assert e["rel_l2"] <= bound, (what, e)
    return e


def _fft1_case_io(c):
    n, b = c["n"], c["batch"]
    if "files" in c:
        x = as_complex(read_bin("fft1_d", c["files"]["input"]).copy())
        gold = read_bin("fft1_d", c["files"]["golden"])
    else:
        x = regenerate("fft1_d", c).astype(np.complex64)
        gold = None
    return n, b, x, gold


def _small(op):
    return [c for c in cases(op, include_skipped=True) if c["n"] * c["batch"] <= MAX_REGEN_ELEMS]


def _large(op):
    return [c for c in cases(op, include_skipped=True) if c["n"] * c["batch"] > MAX_REGEN_ELEMS]


@pytest.mark.parametrize("c", _small("fft1_d"), ids=lambda c: c["name"])
def test_fft1_d_reference_cases(c):
    n, b, x, gold = _fft1_case_io(c)
    if c.get("roundtrip"):
        mid = c2c_host(n, b, x, A.FORWARD)
        out = c2c_host(n, b, mid, A.BACKWARD)
        exact = n * x.astype(np.complex128)
        _fp64_ok(mid, O.c2c(x.reshape(b, n), -1), what="forward half")
    elif c.get("vertical"):
        d = A.FORWARD if c["forward"] else A.BACKWARD
        out = c2c_host(n, b, x, d, A.VERTICAL)
        exact = O.c2c_vertical(x.reshape(n, b), d)
    else:
        d = A.FORWARD if c["forward"] else A.BACKWARD
        out = c2c_host(n, b, x, d)
        exact = O.c2c(x.reshape(b, n), d)
    if gold is not None:
        _gold_ok(out, gold, c)
    _fp64_ok(out, exact, what=c["name"])


@pytest.mark.parametrize("c", _small("rfft1_d"), ids=lambda c: c["name"])
def test_rfft1_d_reference_cases(c):
    n, b = c["n"], c["batch"]
    if "files" in c:
        x = read_bin("rfft1_d", c["files"]["input"]).copy()
        gold = read_bin("rfft1_d", c["files"]["golden"])
    else:
        x = regenerate("rfft1_d", c)
        gold = None
    out = np.empty(b * (n // 2 + 1), dtype=np.complex64)
    with A.Plan.plan1d(n, A.R2C, b) as p:
        p.exec_r2c(x, out)
    if gold is not None:
        _gold_ok(out, gold, c)
    _fp64_ok(out, O.r2c(x.reshape(b, n)), what=c["name"])
    # DC (and Nyquist for even n) imaginary parts are exactly zero, as in the reference
    o = out.reshape(b, n // 2 + 1)
    assert np.all(o[:, 0].imag == 0)
    if n % 2 == 0:
        assert np.all(o[:, -1].imag == 0)


@pytest.mark.parametrize("c", cases("irfft1_d", include_skipped=True), ids=lambda c: c["name"])
def test_irfft1_d_reference_cases(c):
    n, b = c["n"], c["batch"]
    X = as_complex(read_bin("irfft1_d", c["files"]["input"]).copy())
    gold = read_bin("irfft1_d", c["files"]["golden"])
    out = np.empty(b * n, dtype=np.float32)
    with A.Plan.plan1d(n, A.C2R, b) as p:
        p.exec_c2r(X, out)
    _gold_ok(out, gold, c)
    _fp64_ok(out, O.c2r(X.reshape(b, n // 2 + 1), n), what=c["name"])


@pytest.mark.parametrize("c", cases("fft2_d"), ids=lambda c: c["name"])
def test_fft2_d_reference_cases(c):
    nx, ny, b = c["fft_x"], c["fft_y"], c["batch"]
    x = as_complex(read_bin("fft2_d", c["files"]["input"]).copy())
    gold = read_bin("fft2_d", c["files"]["golden"])
    d = A.FORWARD if c["forward"] else A.BACKWARD
    out = np.empty_like(x)
    with A.Plan.plan2d(b, nx, ny, A.C2C) as p:
        p.exec_c2c(x, out, d)
    _gold_ok(out, gold, c)
    _fp64_ok(out, O.c2c_2d(x.reshape(b, nx, ny), d), what=c["name"])


# ----------------------------------------- the reference's largest cases
# Cases above 2^26 elements (R2C up to N = 2^27, the 263168-column VERTICAL
# case) run at the reference's full shape on device buffers.  Inputs follow
# the reference recipe's distribution (randn, seeded) but are drawn on the
# GPU; the FP64 oracle checks sampled transforms with the reference's own
# atol/rtol and the FP32 bound, and a size-independent property covers every
# transform: the unnormalised round trip returns n * x.
def _rel_diff_chunked(a, b, scale, rows_per_chunk):
    """||a - scale*b|| / ||scale*b|| over rows, in float64, chunked."""
    num = den = 0.0
    for r0 in range(0, a.shape[0], rows_per_chunk):
        ad = a[r0: r0 + rows_per_chunk].double()
        bd = b[r0: r0 + rows_per_chunk].double() * scale
        num += float(torch.sum((ad - bd) ** 2))
        den += float(torch.sum(bd ** 2))
    return (num / den) ** 0.5


@pytest.mark.parametrize("c", _large("rfft1_d"), ids=lambda c: c["name"])
def test_rfft1_d_large_reference_cases_full_shape(c):
    n, b = c["n"], c["batch"]
    dev = _dev()
    g = torch.Generator(device=dev).manual_seed(12345)
    x = torch.randn((b, n), generator=g, device=dev)
    X = torch.empty((b, n // 2 + 1), dtype=torch.complex64, device=dev)
    with A.Plan.plan1d(n, A.R2C, b) as p:
        p.set_stream(torch.cuda.current_stream())
        p.exec_r2c(x, X)
        torch.cuda.synchronize()
        assert p.exec_error() == 0
    rows = sorted({0, b - 1}) if n <= (1 << 22) else [b - 1]
    for r in rows:
        xr = x[r].cpu().numpy()
        exact = O.r2c(xr[None, :])[0] if n <= (1 << 22) else O.r2c_long_rows(xr)
        out = X[r].cpu().numpy()
        ok, det = O.comparison_details(out, exact, c["atol"], c["rtol"])
        assert ok, (c["name"], r, det)
        _fp64_ok(out, exact, what=(c["name"], r))
        assert out[0].imag == 0 and out[-1].imag == 0
    y = torch.empty_like(x)
    with A.Plan.plan1d(n, A.C2R, b) as p:
        p.set_stream(torch.cuda.current_stream())
        p.exec_c2r(X, y)
        torch.cuda.synchronize()
        assert p.exec_error() == 0
    rel = _rel_diff_chunked(y, x, float(n), max(1, (1 << 24) // n))
    assert rel <= REL_FP32, (c["name"], "round trip", rel)


@pytest.mark.parametrize("c", _large("fft1_d"), ids=lambda c: c["name"])
def test_fft1_d_large_reference_cases_full_shape(c):
    n, b = c["n"], c["batch"]
    assert c.get("vertical")
    dev = _dev()
    g = torch.Generator(device=dev).manual_seed(12345)
    x = torch.complex(torch.randn((n, b), generator=g, device=dev), torch.randn((n, b), generator=g, device=dev))
    y = torch.empty_like(x)
    d = A.FORWARD if c["forward"] else A.BACKWARD
    with A.Plan.plan1d(n, A.C2C, b, A.VERTICAL) as p:
        p.set_stream(torch.cuda.current_stream())
        p.exec_c2c(x, y, d)
        torch.cuda.synchronize()
        cols = np.unique(np.concatenate([np.arange(8), np.linspace(0, b - 1, 56).astype(np.int64)]))
        xs = x[:, cols].cpu().numpy()
        exact = O.c2c_vertical(xs, d)
        out = y[:, cols].cpu().numpy()
        ok, det = O.comparison_details(out, exact, c["atol"], c["rtol"])
        assert ok, (c["name"], det)
        _fp64_ok(out, exact, what=c["name"])
        z = torch.empty_like(x)
        p.exec_c2c(y, z, -d)
        torch.cuda.synchronize()
        assert p.exec_error() == 0
    rel = _rel_diff_chunked(torch.view_as_real(z), torch.view_as_real(x), float(n), 16)
    assert rel <= REL_FP32, (c["name"], "round trip", rel)


# ------------------------------------------------ benchmark configurations
def _uniform_c64(gen, shape):
    re = torch.rand(shape, generator=gen) * 2 - 1
    im = torch.rand(shape, generator=gen) * 2 - 1
    return torch.complex(re, im)


def _normal_c64(gen, shape):
    return torch.complex(torch.randn(shape, generator=gen), torch.randn(shape, generator=gen))


def test_config1_c2c_4096x256_device():
    g = torch.Generator().manual_seed(12345)
    x = _uniform_c64(g, (256, 4096))
    xd = x.to(_dev())
    yd = torch.empty_like(xd)
    with A.Plan.plan1d(4096, A.C2C, 256) as p:
        p.set_stream(torch.cuda.current_stream())
        p.exec_c2c(xd, yd, A.FORWARD)
        torch.cuda.synchronize()
        y = yd.cpu().numpy()
        _fp64_ok(y, O.c2c(x.numpy(), -1), what="C2C 4096 x 256")
        # same result through host buffers (staging path) and in place
        yh = c2c_host(4096, 256, x.numpy().reshape(-1).copy(), A.FORWARD).reshape(256, 4096)
        assert np.array_equal(yh, y)
        p.exec_c2c(xd, xd, A.FORWARD)
        torch.cuda.synchronize()
        assert np.array_equal(xd.cpu().numpy(), y)


@pytest.mark.parametrize("n,variant", [(3000, None), (1024, None), (3000, "1"), (1024, "1")])
def test_config2_r2c_c2r_batch4096_device(n, variant, monkeypatch):
    # variant "1": the second codelet of the length (a 64-register build of
    # the same radix sequence), selected by OPS_FFT_CODELET_VARIANT
    if variant is not None:
        monkeypatch.setenv("OPS_FFT_CODELET_VARIANT", variant)
    g = torch.Generator().manual_seed(12345)
    b = 4096
    x = torch.randn((b, n), generator=g)
    xd = x.to(_dev())
    Xd = torch.empty((b, n // 2 + 1), dtype=torch.complex64, device=_dev())
    yd = torch.empty((b, n), device=_dev())
    with A.Plan.plan1d(n, A.R2C, b) as pr, A.Plan.plan1d(n, A.C2R, b) as pc:
        pr.set_stream(torch.cuda.current_stream())
        pc.set_stream(torch.cuda.current_stream())
        pr.exec_r2c(xd, Xd)
        pc.exec_c2r(Xd, yd)
        torch.cuda.synchronize()
        X = Xd.cpu().numpy()
        _fp64_ok(X, O.r2c(x.numpy()), what=f"r2c {n}")
        _fp64_ok(yd.cpu().numpy(), O.c2r(X, n), what=f"c2r {n}")
        _fp64_ok(yd.cpu().numpy(), n * x.numpy().astype(np.float64), what=f"round trip {n}")


@pytest.mark.parametrize("n", [65536, 16384])
def test_config3_c2c_batch64_device(n):
    g = torch.Generator().manual_seed(12345)
    x = _normal_c64(g, (64, n))
    xd = x.to(_dev())
    yd = torch.empty_like(xd)
    with A.Plan.plan1d(n, A.C2C, 64) as p:
        p.set_stream(torch.cuda.current_stream())
        p.exec_c2c(xd, yd, A.FORWARD)
        torch.cuda.synchronize()
        e = _fp64_ok(yd.cpu().numpy(), O.c2c(x.numpy(), -1), what=f"C2C {n} x 64")
        assert e["rel_l2"] < 2e-6
        # in place (uses the plan's workspace routing)
        zd = xd.clone()
        p.exec_c2c(zd, zd, A.FORWARD)
        torch.cuda.synchronize()
        assert torch.equal(zd, yd)


def test_config4_2d_2048_batch8_forward_inverse():
    g = torch.Generator().manual_seed(12345)
    x = _uniform_c64(g, (8, 2048, 2048))
    xd = x.to(_dev())
    yd = torch.empty_like(xd)
    zd = torch.empty_like(xd)
    with A.Plan.plan2d(8, 2048, 2048, A.C2C) as p:
        p.set_stream(torch.cuda.current_stream())
        p.exec_c2c(xd, yd, A.FORWARD)
        p.set_norm(A.NORM_BACKWARD)  # inverse scaled by 1/(2048*2048)
        p.exec_c2c(yd, zd, A.BACKWARD)
        torch.cuda.synchronize()
        _fp64_ok(yd[0].cpu().numpy(), O.c2c_2d(x[0].numpy(), -1), what="2d fwd image 0")
        _fp64_ok(zd.cpu().numpy(), x.numpy(), what="2d round trip")


@pytest.mark.parametrize("b,nx,ny", [(2, 256, 1000), (3, 128, 3000), (1, 256, 64), (2, 2048, 1000), (1, 4096, 48)])
def test_2d_column_tiles_vs_fp64(b, nx, ny):
    """2D transforms whose column length has a codelet that fits 8 columns
    per tile (128, 256) run their column pass as column tiles; the row length
    is chosen so the column pass's tables sit after the row pass's in the
    twiddle blob (a non-zero table window).  The other shapes cover the
    column kernel next to row codelets."""
    rng = np.random.default_rng(nx + ny)
    x = (rng.uniform(-1, 1, (b, nx, ny)) + 1j * rng.uniform(-1, 1, (b, nx, ny))).astype(np.complex64)
    xd = torch.from_numpy(x).to(_dev())
    yd = torch.empty_like(xd)
    with A.Plan.plan2d(b, nx, ny, A.C2C) as p:
        p.set_stream(torch.cuda.current_stream())
        for d in (A.FORWARD, A.BACKWARD):
            p.exec_c2c(xd, yd, d)
            torch.cuda.synchronize()
            y = yd.cpu().numpy()
            for i in range(b):
                _fp64_ok(y[i], O.c2c_2d(x[i], d), what=("2d tiles", b, nx, ny, d))
        # in place
        zd = xd.clone()
        p.exec_c2c(zd, zd, A.FORWARD)
        p.exec_c2c(xd, yd, A.FORWARD)
        torch.cuda.synchronize()
        assert torch.equal(zd, yd)


# ------------------------------------------------------------- edge cases
@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 7, 8, 11, 13, 16, 17, 30, 47, 64, 100, 121, 143, 210, 256, 420, 1000,
                               1536, 2048, 2310, 4096, 6561, 8192, 12288, 13312, 16384, 32768, 46200, 100000])
def test_c2c_lengths_both_directions(n):
    b = max(1, min(64, (1 << 20) // n))
    rng = np.random.default_rng(n)
    x = (rng.standard_normal((b, n)) + 1j * rng.standard_normal((b, n))).astype(np.complex64)
    for d in (A.FORWARD, A.BACKWARD):
        out = c2c_host(n, b, x.reshape(-1).copy(), d).reshape(b, n)
        _fp64_ok(out, O.c2c(x, d), what=(n, d))


@pytest.mark.parametrize("n", [1, 2, 3, 4, 6, 7, 8, 9, 15, 16, 30, 33, 64, 100, 255, 256, 999, 1023, 1024, 1025, 2048,
                               3000, 5040, 8190, 12288, 25200, 26624, 32768, 65536, 100000])
def test_r2c_c2r_lengths(n):
    b = max(1, min(32, (1 << 20) // n))
    rng = np.random.default_rng(n)
    x = rng.standard_normal((b, n)).astype(np.float32)
    X = np.empty((b, n // 2 + 1), dtype=np.complex64)
    with A.Plan.plan1d(n, A.R2C, b) as p:
        p.exec_r2c(x, X)
    _fp64_ok(X, O.r2c(x), what=("r2c", n))
    y = np.empty((b, n), dtype=np.float32)
    with A.Plan.plan1d(n, A.C2R, b) as p:
        p.exec_c2r(X, y)
    _fp64_ok(y, O.c2r(X, n), what=("c2r", n))


def test_delta_inputs_pin_index_maps():
    """x = e_m gives X[k] = W^{mk}: any index-permutation error in any pass
    shows up as an O(1) error, so this pins the index maps exactly."""
    for n in (4096, 1500, 65536, 46200):
        ms = [0, 1, 7, n // 2, n - 1]
        x = np.zeros((len(ms), n), dtype=np.complex64)
        for r, m in enumerate(ms):
            x[r, m] = 1.0
        out = c2c_host(n, len(ms), x.reshape(-1).copy(), A.FORWARD).reshape(len(ms), n)
        k = np.arange(n)
        for r, m in enumerate(ms):
            exact = np.exp(-2j * np.pi * ((m * k) % n) / n)
            assert np.abs(out[r] - exact).max() < 2e-6, (n, m)


def test_vertical_large_and_inplace_device():
    for n, b in ((256, 128), (4096, 128), (262144, 4)):
        rng = np.random.default_rng(n)
        x = (rng.standard_normal((n, b)) + 1j * rng.standard_normal((n, b))).astype(np.complex64)
        xd = torch.from_numpy(x).to(_dev())
        with A.Plan.plan1d(n, A.C2C, b, A.VERTICAL) as p:
            p.set_stream(torch.cuda.current_stream())
            p.exec_c2c(xd, xd, A.BACKWARD)
            torch.cuda.synchronize()
        _fp64_ok(xd.cpu().numpy(), O.c2c_vertical(x, +1), what=("vertical", n))


@pytest.mark.parametrize("n,b", [(1024, 8), (3000, 8), (7, 8), (65536, 8), (2048, 600), (4096, 300)])
def test_r2c_c2r_inplace_device(n, b):
    rng = np.random.default_rng(n)
    x = rng.standard_normal((b, n)).astype(np.float32)
    buf = torch.zeros(b * (n // 2 + 1) * 2, device=_dev())
    buf[: b * n] = torch.from_numpy(x.reshape(-1)).to(_dev())
    with A.Plan.plan1d(n, A.R2C, b) as p:
        p.set_stream(torch.cuda.current_stream())
        p.exec_r2c(buf, buf)
    torch.cuda.synchronize()
    X = buf.cpu().numpy().view(np.complex64).reshape(b, n // 2 + 1)
    _fp64_ok(X, O.r2c(x), what=("r2c in place", n))
    with A.Plan.plan1d(n, A.C2R, b) as p:
        p.set_stream(torch.cuda.current_stream())
        p.exec_c2r(buf, buf)
    torch.cuda.synchronize()
    y = buf.cpu().numpy()[: b * n].reshape(b, n)
    _fp64_ok(y, n * x.astype(np.float64), what=("c2r in place", n))


@pytest.mark.parametrize("n,b", [(1024, 4096), (3000, 4096), (1025, 64), (1 << 20, 2), (4096, 2048)])
def test_host_inplace_r2c_c2r_c2c(n, b):
    """In-place calls on HOST buffers (the reference's documented layout,
    docs/zh/API_Reference/FFT_1D.md:201: one buffer of batch*2*(n/2+1)
    floats, the input rows packed at its start).  The batch-4096 shapes are
    large enough to take the chunked host pipeline, where an R2C chunk's
    output rows cover later chunks' input rows."""
    rng = np.random.default_rng(n + b)
    x = rng.standard_normal((b, n)).astype(np.float32)
    buf = np.zeros(b * 2 * (n // 2 + 1), dtype=np.float32)
    buf[: b * n] = x.reshape(-1)
    with A.Plan.plan1d(n, A.R2C, b) as p:
        p.exec_r2c(buf, buf)
    X = buf.view(np.complex64).reshape(b, n // 2 + 1).copy()
    _fp64_ok(X, O.r2c(x), what=("host r2c in place", n, b))
    with A.Plan.plan1d(n, A.C2R, b) as p:
        p.exec_c2r(buf, buf)
    y = buf[: b * n].reshape(b, n)
    _fp64_ok(y, O.c2r(X, n), what=("host c2r in place", n, b))
    _fp64_ok(y, n * x.astype(np.float64), what=("host round trip in place", n, b))
    z = (rng.standard_normal((b, n)) + 1j * rng.standard_normal((b, n))).astype(np.complex64)
    zb = z.reshape(-1).copy()
    with A.Plan.plan1d(n, A.C2C, b) as p:
        p.exec_c2c(zb, zb, A.FORWARD)
    _fp64_ok(zb.reshape(b, n), O.c2c(z, -1), what=("host c2c in place", n, b))


@pytest.mark.parametrize("mode", [A.NORM_NONE, A.NORM_BACKWARD, A.NORM_ORTHO, A.NORM_FORWARD])
def test_norm_modes(mode):
    n, b = 1000, 3
    rng = np.random.default_rng(mode)
    x = (rng.standard_normal((b, n)) + 1j * rng.standard_normal((b, n))).astype(np.complex64)
    sf = {A.NORM_NONE: 1, A.NORM_BACKWARD: 1, A.NORM_ORTHO: n ** -0.5, A.NORM_FORWARD: 1 / n}[mode]
    sb = {A.NORM_NONE: 1, A.NORM_BACKWARD: 1 / n, A.NORM_ORTHO: n ** -0.5, A.NORM_FORWARD: 1}[mode]
    with A.Plan.plan1d(n, A.C2C, b) as p:
        p.set_norm(mode)
        f = np.empty_like(x)
        p.exec_c2c(x, f, A.FORWARD)
        bk = np.empty_like(x)
        p.exec_c2c(x, bk, A.BACKWARD)
    _fp64_ok(f, sf * O.c2c(x, -1), what="fwd")
    _fp64_ok(bk, sb * O.c2c(x, +1), what="bwd")


def test_unsupported_length_is_not_implemented_on_gpu():
    n = 53 * 7
    x = np.zeros(n, dtype=np.complex64)
    with A.Plan.plan1d(n, A.C2C, 1) as p:
        assert A.lib().aclfftExecC2C(p.handle, x.ctypes.data, x.ctypes.data, -1) == A.NOT_IMPLEMENTED


# -------------------------------------------------------------- adjoints
def _fd_grad(f, x, h=1e-6):
    """Central finite differences of a real scalar f over a real vector x."""
    g = np.zeros_like(x)
    for i in range(x.size):
        e = np.zeros_like(x)
        e.flat[i] = h
        g.flat[i] = (f(x + e) - f(x - e)) / (2 * h)
    return g


def test_adjoint_c2c_against_fd():
    n, b = 64, 4
    rng = np.random.default_rng(1)
    x = rng.standard_normal((b, n)) + 1j * rng.standard_normal((b, n))
    G = rng.standard_normal((b, n)) + 1j * rng.standard_normal((b, n))
    for d in (A.FORWARD, A.BACKWARD):
        # L(x) = sum Re(conj(G) * F_d(x)); complex gradient dL/dRe + i dL/dIm
        def L(v):
            z = v[: v.size // 2] + 1j * v[v.size // 2:]
            return float(np.sum(np.real(np.conj(G) * O.c2c(z.reshape(b, n), d))))
        v0 = np.concatenate([x.real.reshape(-1), x.imag.reshape(-1)])
        gfd = _fd_grad(L, v0)
        gfd = gfd[: v0.size // 2] + 1j * gfd[v0.size // 2:]
        out = np.empty((b, n), dtype=np.complex64)
        with A.Plan.plan1d(n, A.C2C, b) as p:
            p.exec_c2c_adjoint(G.astype(np.complex64), out, d)
        _fp64_ok(out.reshape(-1), gfd, bound=1e-5, what=("c2c adjoint", d))


def test_adjoint_2d_against_fd_32x32():
    """2D C2C backward pass through L = sum Re(conj(G) * F2(x)) on a 32x32
    instance (and the normalised inverse), against FP64 central differences."""
    nx = ny = 32
    rng = np.random.default_rng(4)
    x = rng.uniform(-1, 1, (nx, ny)) + 1j * rng.uniform(-1, 1, (nx, ny))
    G = rng.standard_normal((nx, ny)) + 1j * rng.standard_normal((nx, ny))
    for d, norm, scale in ((A.FORWARD, A.NORM_NONE, 1.0), (A.BACKWARD, A.NORM_BACKWARD, 1.0 / (nx * ny))):
        def L(v):
            z = (v[: v.size // 2] + 1j * v[v.size // 2:]).reshape(nx, ny)
            return float(np.sum(np.real(np.conj(G) * O.c2c_2d(z, d) * scale)))
        v0 = np.concatenate([x.real.reshape(-1), x.imag.reshape(-1)])
        gfd = _fd_grad(L, v0)
        gfd = gfd[: v0.size // 2] + 1j * gfd[v0.size // 2:]
        out = np.empty((nx, ny), dtype=np.complex64)
        with A.Plan.plan2d(1, nx, ny, A.C2C) as p:
            p.set_norm(norm)
            p.exec_c2c_adjoint(G.astype(np.complex64), out, d)
        _fp64_ok(out.reshape(-1), gfd, bound=1e-5, what=("2d adjoint", d))


@pytest.mark.parametrize("n", [64, 63])
def test_adjoint_r2c_against_fd_and_torch(n):
    b = 4
    rng = np.random.default_rng(2)
    x = rng.standard_normal((b, n))
    w = rng.uniform(0, 1, (b, n // 2 + 1))

    def L(v):
        X = O.r2c(v.reshape(b, n))
        return float(np.sum(w * np.abs(X) ** 2))

    gfd = _fd_grad(L, x.reshape(-1)).reshape(b, n)
    Xbar = (2 * w * O.r2c(x)).astype(np.complex64)  # dL/dX in the complex-gradient convention
    out = np.empty((b, n), dtype=np.float32)
    with A.Plan.plan1d(n, A.R2C, b) as p:
        p.exec_r2c_adjoint(Xbar, out)
    _fp64_ok(out, gfd, bound=1e-5, what="r2c adjoint vs FD")
    xt = torch.tensor(x, dtype=torch.float64, requires_grad=True)
    Lt = (torch.tensor(w) * torch.fft.rfft(xt).abs() ** 2).sum()
    Lt.backward()
    _fp64_ok(out, xt.grad.numpy(), bound=1e-5, what="r2c adjoint vs torch")


@pytest.mark.parametrize("n", [64, 63])
def test_adjoint_c2r_against_fd_and_torch(n):
    b = 4
    nb = n // 2 + 1
    rng = np.random.default_rng(3)
    X = rng.standard_normal((b, nb)) + 1j * rng.standard_normal((b, nb))
    v = rng.standard_normal((b, n))

    def L(u):
        Z = u[: u.size // 2] + 1j * u[u.size // 2:]
        return float(np.sum(v * O.c2r(Z.reshape(b, nb), n)))

    u0 = np.concatenate([X.real.reshape(-1), X.imag.reshape(-1)])
    g = _fd_grad(L, u0)
    gfd = (g[: u0.size // 2] + 1j * g[u0.size // 2:]).reshape(b, nb)
    out = np.empty((b, nb), dtype=np.complex64)
    with A.Plan.plan1d(n, A.C2R, b) as p:
        p.exec_c2r_adjoint(v.astype(np.float32), out)
    _fp64_ok(out, gfd, bound=1e-5, what="c2r adjoint vs FD")
    Xt = torch.tensor(X, dtype=torch.complex128, requires_grad=True)
    Lt = (torch.tensor(v) * torch.fft.irfft(Xt, n=n) * n).sum()
    Lt.backward()
    # torch's irfft gradient follows the same Hermitian convention
    _fp64_ok(out, Xt.grad.numpy(), bound=1e-5, what="c2r adjoint vs torch")


def _unit_root_fp32(m, M):
    """exp(-2 pi i m / M) in FP64 rounded to complex64, with the angle reduced
    exactly: 2m/M = q/2 + y with integer q and |y| <= 1/4 (y from an exact
    integer numerator), so quarter-turn values come out exact (cos(pi/2) = 0,
    not 6e-17)."""
    m = np.asarray(m, dtype=np.int64) % M
    q = (4 * m + M // 2) // M                      # nearest multiple of 1/2 of 2m/M
    y = (4 * m - q * M).astype(np.float64) / (2.0 * M)
    c, s = np.cos(np.pi * y), np.sin(np.pi * y)
    q = q % 4
    cr = np.select([q == 0, q == 1, q == 2, q == 3], [c, -s, -c, s])
    sr = np.select([q == 0, q == 1, q == 2, q == 3], [s, c, -s, -c])
    return (cr - 1j * sr).astype(np.complex64)


@pytest.mark.parametrize("n,b", [(3000, 64), (1024, 37), (2048, 5), (8192, 3), (8192, 1100)])
def test_weighted_r2c_adjoint(n, b):
    """aclfftExecR2CAdjointWeighted(X, 2w) = dL/dx of L = sum(w*|X|^2),
    X = R2C(x): bit-identical to scaling X by 2w first and calling the plain
    adjoint, and equal to the FP64 gradient (torch autograd in complex128)."""
    dev = _dev()
    rng = np.random.default_rng(n)
    x = rng.standard_normal((b, n))
    w = rng.uniform(0, 1, (b, n // 2 + 1))
    xd = torch.tensor(x, dtype=torch.float32, device=dev)
    w2 = torch.tensor(2 * w, dtype=torch.float32, device=dev)
    X = torch.empty((b, n // 2 + 1), dtype=torch.complex64, device=dev)
    g1 = torch.empty((b, n), dtype=torch.float32, device=dev)
    g2 = torch.empty_like(g1)
    with A.Plan.plan1d(n, A.R2C, b) as p:
        p.set_stream(torch.cuda.current_stream())
        p.exec_r2c(xd, X)
        p.exec_r2c_adjoint_weighted(X, w2, g1)
        G = X * w2
        p.exec_r2c_adjoint(G, g2)
        torch.cuda.synchronize()
        assert p.exec_error() == 0
    assert torch.equal(g1, g2)
    xt = torch.tensor(xd.cpu().numpy(), dtype=torch.float64, requires_grad=True)
    (torch.tensor(w2.cpu().numpy(), dtype=torch.float64) / 2 * torch.fft.rfft(xt).abs() ** 2).sum().backward()
    _fp64_ok(g1.cpu().numpy(), xt.grad.numpy(), what=("weighted adjoint", n))


def test_weighted_r2c_adjoint_domain():
    dev = _dev()
    for n, b in ((65536, 2), (999, 3), (1 << 20, 1), (16384, 4)):   # cluster, odd, column passes, cluster
        X = torch.zeros((b, n // 2 + 1), dtype=torch.complex64, device=dev)
        w = torch.ones((b, n // 2 + 1), dtype=torch.float32, device=dev)
        g = torch.empty((b, n), dtype=torch.float32, device=dev)
        with A.Plan.plan1d(n, A.R2C, b) as p:
            rc = A.lib().aclfftExecR2CAdjointWeighted(p.handle, X.data_ptr(), w.data_ptr(), g.data_ptr())
            assert rc == A.NOT_IMPLEMENTED, (n, rc)
    with A.Plan.plan1d(3000, A.R2C, 2) as p:
        X = torch.zeros((2, 1501), dtype=torch.complex64, device=dev)
        hw = np.ones((2, 1501), dtype=np.float32)
        g = torch.empty((2, 3000), dtype=torch.float32, device=dev)
        assert A.lib().aclfftExecR2CAdjointWeighted(p.handle, X.data_ptr(), hw.ctypes.data, g.data_ptr()) == \
            A.INVALID_VALUE
        assert A.lib().aclfftExecR2CAdjointWeighted(p.handle, X.data_ptr(), None, g.data_ptr()) == A.INVALID_VALUE


@pytest.mark.parametrize("plan_args", [("1d", 4096, A.C2C, 1), ("1d", 3000, A.R2C, 4), ("1d", 1 << 20, A.C2C, 2),
                                       ("1d", 46200, A.C2C, 1), ("2d", 2048, 1000, 1), ("1d", 1 << 25, A.R2C, 1)])
def test_twiddles_are_correctly_rounded_fp64_values(plan_args):
    """Every pass-table and linear-table entry of the GPU-generated blob
    equals exp(-2 pi i m / M) for its documented index m, evaluated in FP64
    and rounded to FP32: bit-exact except where FP64 rounding of the angle
    lands next to an FP32 rounding tie (then within 1 ulp)."""
    kind, a, bb, c = plan_args
    p = A.Plan.plan1d(a, bb, c) if kind == "1d" else A.Plan.plan2d(c, a, bb, A.C2C)
    with p:
        tw = p.twiddles()
        segs = p.twiddle_segments()
    checked = exact_bits = 0
    for off, cnt, M, param, k in segs:
        if k not in (1, 2):
            continue
        i = np.arange(cnt, dtype=np.int64)
        m = ((i // param) * (i % param)) % M if k == 2 else (i * param) % M
        want = _unit_root_fp32(m, M)
        got = tw[off: off + cnt]
        gf, wf = got.view(np.float32), want.view(np.float32)
        ulp = np.spacing(np.maximum(np.abs(wf), np.float32(1e-30)))
        assert np.all(np.abs(gf - wf) <= ulp), (plan_args, off, M, param, k)
        checked += gf.size
        exact_bits += int(np.count_nonzero(gf == wf))
    assert checked > 0
    assert exact_bits >= 0.999 * checked, (exact_bits, checked)


@pytest.mark.parametrize("kind,n,b", [("c2c", 4096, 64), ("c2c", 4096, 2048), ("c2c", 65536, 3), ("r2c", 3000, 37),
                                      ("c2r", 3000, 37), ("r2c", 32768, 5), ("c2r", 1024, 9), ("2d", 2048, 1)])
def test_device_execs_replay_from_a_cuda_graph(kind, n, b):
    # exec with device pointers only enqueues precomputed launches on the
    # plan's stream, so it can be captured: one graph of two execs on two
    # input sets, replayed after the inputs change, matches the FP64 oracle
    # (cluster, codelet, column-tile and real-data kernels)
    dev = _dev()
    s = torch.cuda.Stream(dev)
    rng = np.random.default_rng(n + b)
    if kind == "2d":
        shape_in = shape_out = (b, n, n)
        plan = A.Plan.plan2d(b, n, n, A.C2C)
    else:
        plan = A.Plan.plan1d(n, {"c2c": A.C2C, "r2c": A.R2C, "c2r": A.C2R}[kind], b)
        shape_in = (b, n) if kind != "c2r" else (b, n // 2 + 1)
        shape_out = (b, n) if kind != "r2c" else (b, n // 2 + 1)
    real_in, real_out = kind == "r2c", kind == "c2r"
    xs = [torch.empty(shape_in, dtype=torch.float32 if real_in else torch.complex64, device=dev) for _ in range(2)]
    ys = [torch.empty(shape_out, dtype=torch.float32 if real_out else torch.complex64, device=dev) for _ in range(2)]

    def run(i):
        if kind == "r2c":
            plan.exec_r2c(xs[i], ys[i])
        elif kind == "c2r":
            plan.exec_c2r(xs[i], ys[i])
        else:
            plan.exec_c2c(xs[i], ys[i], A.FORWARD)

    with plan:
        plan.set_stream(s)
        for x in xs:
            x.copy_(torch.from_numpy(rng.standard_normal(shape_in).astype(np.float32)) if real_in else
                    torch.from_numpy((rng.standard_normal(shape_in) + 1j * rng.standard_normal(shape_in))
                                     .astype(np.complex64)))
        torch.cuda.synchronize()
        run(0)  # first exec outside the capture (lazy per-device set-up)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            run(0)
            run(1)
        for i, x in enumerate(xs):  # new inputs after the capture
            x.mul_(-0.5 - i)
        g.replay()
        torch.cuda.synchronize()
        for i in range(2):
            x = xs[i].cpu().numpy()
            if kind == "r2c":
                exact = O.r2c(x)
            elif kind == "c2r":
                exact = O.c2r(x, n)
            elif kind == "2d":
                exact = np.fft.fft2(x.astype(np.complex128))
            else:
                exact = O.c2c(x, -1)
            _fp64_ok(ys[i].cpu().numpy(), exact, what=f"{kind} {n} graph replay {i}")
