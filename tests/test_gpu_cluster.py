"""GPU parity of the thread-block-cluster C2C path (one cluster of 4-16 CTAs
per transform, distributed shared memory between the column and the row
phase) against the FP64 oracle.

Tolerance: rel-L2 <= 1e-6 vs FP64 (plain FP32 Stockham with table
twiddles; the contract bound for FP32 is 1e-5).  Every case checks that the
plan really runs a cluster step (aclfftGetPlanInfo.cluster_ctas), and the
batches exceed the number of co-resident clusters so each cluster runs
several transforms through the same receive buffers.
"""
import numpy as np
import pytest

import aclfft as A
import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

BOUND = 1e-6
# (length, cluster size, batch)
CASES = [(4096, 4, 301), (4096, 8, 203), (8192, 4, 301), (16384, 4, 150), (16384, 8, 77), (32768, 8, 60), (65536, 16, 40), (65536, 8, 37)]


def _data(n, b, seed):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal((b, n)) + 1j * rng.standard_normal((b, n))).astype(np.complex64)


def _run(x, n, b, direction=A.FORWARD, inplace=False, norm=None):
    dev = torch.device("cuda:0")
    xt = torch.from_numpy(x).to(dev)
    yt = xt if inplace else torch.empty_like(xt)
    with A.Plan.plan1d(n, A.C2C, b) as p:
        if norm is not None:
            p.set_norm(norm)
        info = p.info()
        assert p.check() == "ok"
        p.set_stream(torch.cuda.current_stream(dev))
        p.exec_c2c(xt, yt, direction)
        torch.cuda.synchronize()
    return yt.cpu().numpy(), info


@pytest.fixture(autouse=True)
def _clusters_for_short_lengths(monkeypatch):
    # 4096-point C2C (8192-point R2C/C2R) transforms run on the row codelet
    # by default; the knob keeps their cluster configurations under test
    monkeypatch.setenv("OPS_FFT_CLUSTER_MAXBATCH", "1000000")


@pytest.mark.parametrize("n,c,b", CASES)
def test_cluster_forward_vs_fp64(n, c, b, monkeypatch):
    monkeypatch.setenv("OPS_FFT_CLUSTER_C", str(c))
    x = _data(n, b, 1000 + n + c)
    y, info = _run(x, n, b)
    assert info.cluster_ctas == c and info.nsteps == 1
    e = O.errors(y, O.c2c(x, -1))
    assert e["rel_l2"] <= BOUND, e


@pytest.mark.parametrize("n,c", [(8192, 4), (16384, 8), (65536, 16)])
def test_cluster_backward_inplace_scaled(n, c, monkeypatch):
    monkeypatch.setenv("OPS_FFT_CLUSTER_C", str(c))
    b = 5
    x = _data(n, b, 7 + n)
    y, info = _run(x, n, b, direction=A.BACKWARD, inplace=True, norm=A.NORM_BACKWARD)
    assert info.cluster_ctas == c
    e = O.errors(y, O.c2c(x, +1) / n)
    assert e["rel_l2"] <= BOUND, e


def test_cluster_single_transform_and_impulses():
    # batch 1 (one cluster) and impulse inputs: exact spectra pin the index
    # maps of the column loads, the exchange and the row stores
    n = 32768
    x = np.zeros((3, n), np.complex64)
    x[0, 1] = 1.0
    x[1, n - 1] = 1.0 - 2.0j
    x[2, 12345] = 0.5j
    y, info = _run(x, n, 3)
    assert info.cluster_ctas > 0
    exact = O.c2c(x, -1)
    assert np.abs(y - exact).max() <= 1e-5
    y1, _ = _run(x[:1].copy(), n, 1)
    assert np.array_equal(y1, y[:1])


def test_cluster_adjoint_matches_backward():
    n, b = 16384, 3
    x = _data(n, b, 3)
    dev = torch.device("cuda:0")
    xt = torch.from_numpy(x).to(dev)
    gt = torch.empty_like(xt)
    with A.Plan.plan1d(n, A.C2C, b) as p:
        assert p.info().cluster_ctas > 0
        p.exec_c2c_adjoint(xt, gt, A.FORWARD)
        torch.cuda.synchronize()
    e = O.errors(gt.cpu().numpy(), O.c2c(x, +1))
    assert e["rel_l2"] <= BOUND, e


@pytest.mark.parametrize("n,c", [(8192, 4), (8192, 8), (16384, 4), (32768, 4), (32768, 8), (65536, 8), (131072, 16),
                                 (131072, 8)])
def test_cluster_real_transforms_vs_fp64(n, c, monkeypatch):
    # even real lengths beyond one CTA (and N = 8192 in a small batch): the
    # half-length complex transform runs on a cluster with the even/odd
    # packing fused (one launch); the batch exceeds the co-resident clusters
    monkeypatch.setenv("OPS_FFT_CLUSTER_C", str(c))
    b = max(9, (1 << 24) // n) if n > 8192 else 700
    rng = np.random.default_rng(n + c)
    x = rng.standard_normal((b, n)).astype(np.float32)
    X = np.empty((b, n // 2 + 1), np.complex64)
    with A.Plan.plan1d(n, A.R2C, b) as p:
        assert p.info().cluster_ctas == c and p.info().nsteps == 1
        p.exec_r2c(x, X)
    e = O.errors(X, O.r2c(x))
    assert e["rel_l2"] <= BOUND, e
    Xc = (rng.standard_normal((b, n // 2 + 1)) + 1j * rng.standard_normal((b, n // 2 + 1))).astype(np.complex64)
    y = np.empty((b, n), np.float32)
    with A.Plan.plan1d(n, A.C2R, b) as p:
        assert p.info().cluster_ctas == c and p.info().nsteps == 1
        p.exec_c2r(Xc, y)
    e = O.errors(y, O.c2r(Xc, n))
    assert e["rel_l2"] <= BOUND, e


def test_cluster_real_inplace_scaled_and_impulses():
    # in place (a copy step first), backward normalisation, and impulses
    # whose exact spectra pin the post-process pairing of rows 0, Q/2 and
    # the mirrored rows
    n, b = 65536, 4
    dev = torch.device("cuda:0")
    x = np.zeros((b, n), np.float32)
    x[0, 1] = 1.0
    x[1, 3] = -2.0
    x[2, n - 1] = 0.5
    x[3] = np.random.default_rng(9).standard_normal(n)
    nb = n // 2 + 1
    buf = torch.zeros(b * nb * 2, dtype=torch.float32, device=dev)
    buf[: b * n] = torch.from_numpy(x.reshape(-1)).to(dev)
    with A.Plan.plan1d(n, A.R2C, b) as p:
        assert p.info().cluster_ctas > 0
        p.set_stream(torch.cuda.current_stream(dev))
        p.exec_r2c(buf, buf)
        torch.cuda.synchronize()
    X = buf.cpu().numpy().view(np.complex64).reshape(b, nb)
    exact = O.r2c(x)
    assert np.abs(X[:3] - exact[:3]).max() <= 1e-5
    e = O.errors(X, exact)
    assert e["rel_l2"] <= BOUND, e
    y = np.empty((b, n), np.float32)
    with A.Plan.plan1d(n, A.C2R, b) as p:
        p.set_norm(A.NORM_BACKWARD)
        p.exec_c2r(X, y)
    e = O.errors(y, x)
    assert e["rel_l2"] <= BOUND, e


def test_cluster_real_adjoints_vs_torch():
    n, b = 32768, 2
    nb = n // 2 + 1
    rng = np.random.default_rng(5)
    x = rng.standard_normal((b, n))
    w = rng.uniform(0, 1, (b, nb))
    xt = torch.tensor(x, dtype=torch.float64, requires_grad=True)
    (torch.tensor(w) * torch.fft.rfft(xt).abs() ** 2).sum().backward()
    Xbar = (2 * w * O.r2c(x)).astype(np.complex64)
    out = np.empty((b, n), np.float32)
    with A.Plan.plan1d(n, A.R2C, b) as p:
        assert p.info().cluster_ctas > 0
        p.exec_r2c_adjoint(Xbar, out)
    e = O.errors(out, xt.grad.numpy())
    assert e["rel_l2"] <= 1e-5, e
    X = rng.standard_normal((b, nb)) + 1j * rng.standard_normal((b, nb))
    v = rng.standard_normal((b, n))
    Xt = torch.tensor(X, dtype=torch.complex128, requires_grad=True)
    (torch.tensor(v) * torch.fft.irfft(Xt, n=n) * n).sum().backward()
    g = np.empty((b, nb), np.complex64)
    with A.Plan.plan1d(n, A.C2R, b) as p:
        p.exec_c2r_adjoint(v.astype(np.float32), g)
    e = O.errors(g, Xt.grad.numpy())
    assert e["rel_l2"] <= 1e-5, e


def test_short_lengths_use_clusters_only_in_small_batches(monkeypatch):
    # N = 4096 C2C and N = 8192 R2C: the row codelet by default; a cluster
    # per transform at or below OPS_FFT_CLUSTER_MAXBATCH; both give the FP64
    # result
    for kind, n, b, lim, want in [(A.C2C, 4096, 256, None, False), (A.C2C, 4096, 256, "256", True),
                                  (A.C2C, 4096, 256, "100", False), (A.R2C, 8192, 64, None, False),
                                  (A.R2C, 8192, 64, "64", True), (A.R2C, 8192, 64, "32", False)]:
        if lim is None:
            monkeypatch.delenv("OPS_FFT_CLUSTER_MAXBATCH", raising=False)
        else:
            monkeypatch.setenv("OPS_FFT_CLUSTER_MAXBATCH", lim)
        rng = np.random.default_rng(n + b)
        if kind == A.C2C:
            x = _data(n, b, n + b)
            y, info = _run(x, n, b)
            ref = O.c2c(x, -1)
        else:
            x = rng.standard_normal((b, n)).astype(np.float32)
            y = np.empty((b, n // 2 + 1), np.complex64)
            with A.Plan.plan1d(n, A.R2C, b) as p:
                info = p.info()
                p.exec_r2c(x, y)
            ref = O.r2c(x)
        assert (info.cluster_ctas > 0) == want
        e = O.errors(y, ref)
        assert e["rel_l2"] <= BOUND, e
