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
CASES = [(8192, 4, 301), (16384, 4, 150), (16384, 8, 77), (32768, 8, 60), (65536, 16, 40), (65536, 8, 37)]


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
