"""Pinned host buffers on one-launch codelet plans: the kernel fills its
input slots from host memory with per-thread asynchronous copies and writes
its results to host memory directly (no staging copies).  By default only
small calls run that way; the tests force it (OPS_FFT_HOST_DIRECT=1) at every
size.  The same kernel runs as on device buffers, so results equal the staged
path (OPS_FFT_HOST_DIRECT=0) bit for bit, and the FP64 oracle within the FP32
tolerance (rel-L2 <= 1e-5)."""
import os

import numpy as np
import pytest

import aclfft as A
import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

REL = 1e-5


def _pinned(a: np.ndarray):
    t = torch.empty(a.shape, dtype=torch.from_numpy(a).dtype, pin_memory=True)
    t.copy_(torch.from_numpy(a))
    return t


def _with_mode(mode, fn):
    old = os.environ.get("OPS_FFT_HOST_DIRECT")
    if mode is None:
        os.environ.pop("OPS_FFT_HOST_DIRECT", None)
    else:
        os.environ["OPS_FFT_HOST_DIRECT"] = mode
    try:
        fn()
    finally:
        if old is None:
            os.environ.pop("OPS_FFT_HOST_DIRECT", None)
        else:
            os.environ["OPS_FFT_HOST_DIRECT"] = old


def _staged(fn):
    _with_mode("0", fn)


@pytest.fixture(autouse=True)
def _force_direct():
    old = os.environ.get("OPS_FFT_HOST_DIRECT")
    os.environ["OPS_FFT_HOST_DIRECT"] = "1"
    yield
    if old is None:
        os.environ.pop("OPS_FFT_HOST_DIRECT", None)
    else:
        os.environ["OPS_FFT_HOST_DIRECT"] = old


def _direct_plan(p):
    info = p.info()
    assert info.nsteps == 1 and info.kernel >= 0, "expected a one-launch codelet plan"


@pytest.mark.parametrize("n,b", [(3000, 64), (3000, 63), (1024, 33), (8192, 5), (3000, 4096)])
def test_r2c_c2r_pinned_direct(n, b):
    nb = n // 2 + 1
    rng = np.random.default_rng(n + b)
    x = rng.standard_normal((b, n)).astype(np.float32)
    Y = (rng.standard_normal((b, nb)) + 1j * rng.standard_normal((b, nb))).astype(np.complex64)
    xh, Yh = _pinned(x), _pinned(Y)
    X1 = torch.empty((b, nb), dtype=torch.complex64, pin_memory=True)
    X2 = torch.empty_like(X1).pin_memory()
    y1 = torch.empty((b, n), dtype=torch.float32, pin_memory=True)
    y2 = torch.empty_like(y1).pin_memory()
    with A.Plan.plan1d(n, A.R2C, b) as pr, A.Plan.plan1d(n, A.C2R, b) as pc:
        _direct_plan(pr)
        _direct_plan(pc)
        pr.exec_r2c(xh, X1)
        pc.exec_c2r(Yh, y1)
        _staged(lambda: (pr.exec_r2c(xh, X2), pc.exec_c2r(Yh, y2)))
    assert torch.equal(X1, X2) and torch.equal(y1, y2)
    assert O.errors(X1.numpy(), O.r2c(x.astype(np.float64)))["rel_l2"] <= REL
    assert O.errors(y1.numpy(), O.c2r(Y.astype(np.complex128), n))["rel_l2"] <= REL


@pytest.mark.parametrize("n,b", [(4096, 16), (512, 101), (1500, 7)])
def test_c2c_pinned_direct_both_directions_and_norm(n, b):
    rng = np.random.default_rng(n)
    x = (rng.standard_normal((b, n)) + 1j * rng.standard_normal((b, n))).astype(np.complex64)
    xh = _pinned(x)
    y1 = torch.empty((b, n), dtype=torch.complex64, pin_memory=True)
    y2 = torch.empty_like(y1).pin_memory()
    with A.Plan.plan1d(n, A.C2C, b) as p:
        _direct_plan(p)
        for d in (A.FORWARD, A.BACKWARD):
            p.exec_c2c(xh, y1, d)
            _staged(lambda: p.exec_c2c(xh, y2, d))
            assert torch.equal(y1, y2)
            _with_mode(None, lambda: p.exec_c2c(xh, y2, d))  # the default (size-dependent) choice
            assert torch.equal(y1, y2)
            assert O.errors(y1.numpy(), O.c2c(x.astype(np.complex128), d))["rel_l2"] <= REL
        p.set_norm(A.NORM_ORTHO)
        p.exec_c2c(xh, y1, A.FORWARD)
        assert O.errors(y1.numpy(), O.c2c(x.astype(np.complex128), -1) / np.sqrt(n))["rel_l2"] <= REL


def test_adjoints_pinned_direct():
    n, b = 3000, 40
    nb = n // 2 + 1
    rng = np.random.default_rng(5)
    G = (rng.standard_normal((b, nb)) + 1j * rng.standard_normal((b, nb))).astype(np.complex64)
    g = rng.standard_normal((b, n)).astype(np.float32)
    Gh, gh = _pinned(G), _pinned(g)
    a1 = torch.empty((b, n), dtype=torch.float32, pin_memory=True)
    a2 = torch.empty_like(a1).pin_memory()
    c1 = torch.empty((b, nb), dtype=torch.complex64, pin_memory=True)
    c2 = torch.empty_like(c1).pin_memory()
    with A.Plan.plan1d(n, A.R2C, b) as pr, A.Plan.plan1d(n, A.C2R, b) as pc:
        pr.exec_r2c_adjoint(Gh, a1)
        pc.exec_c2r_adjoint(gh, c1)
        _staged(lambda: (pr.exec_r2c_adjoint(Gh, a2), pc.exec_c2r_adjoint(gh, c2)))
    assert torch.equal(a1, a2) and torch.equal(c1, c2)
    # R2C adjoint: C2R of the gradient with interior bins halved
    Gw = G.astype(np.complex128).copy()
    Gw[:, 1:(n + 1) // 2] *= 0.5
    assert O.errors(a1.numpy(), O.c2r(Gw, n))["rel_l2"] <= REL


def test_offsets_and_pageable_buffers():
    """A pinned buffer used at an 8-byte offset runs direct; at a 4-byte
    offset (not aligned to the complex element) and a pageable numpy array
    it is staged; all equal the oracle."""
    n, b = 4096, 8
    rng = np.random.default_rng(11)
    x = (rng.standard_normal((b, n)) + 1j * rng.standard_normal((b, n))).astype(np.complex64)
    exact = O.c2c(x.astype(np.complex128), -1)
    raw = torch.zeros(2 * b * n * 8 + 64, dtype=torch.uint8, pin_memory=True)
    with A.Plan.plan1d(n, A.C2C, b) as p:
        for off in (8, 4):
            xin = raw[off:off + b * n * 8]
            xin.copy_(torch.from_numpy(x.view(np.uint8).reshape(-1)))
            out = raw[b * n * 8 + 32 + off:b * n * 8 + 32 + off + b * n * 8]
            p.exec_c2c(xin.data_ptr(), out.data_ptr(), A.FORWARD)
            y = out.numpy().view(np.complex64).reshape(b, n)
            assert O.errors(y, exact)["rel_l2"] <= REL, off
        yp = np.empty_like(x)
        p.exec_c2c(x, yp, A.FORWARD)
        assert O.errors(yp, exact)["rel_l2"] <= REL
