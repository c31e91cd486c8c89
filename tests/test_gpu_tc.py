"""GPU parity of the split-precision tensor-core C2C forms (tcgen05 DFT-matrix
stages) against the FP64 oracle, next to the plain FP32 Stockham form.

Tolerances (stated here, used below):
  * TF32x3 (TF32 hi + lo operands, three products): rel-L2 <= 1e-6 vs FP64,
    the plain-FP32 accuracy target for the split form;
  * BF16x3 (BF16 hi + lo, three products, ~16 significant bits per
    operand): rel-L2 <= 5e-5 vs FP64;
  * plain FP32 Stockham: rel-L2 <= 1e-6 at these lengths.
Every case also checks that the plan really ran tensor-core launches
(aclfftGetPlanInfo.tc_stages) so a silent FP32 fallback cannot pass.
"""
import numpy as np
import pytest

import aclfft as A
import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

BOUND = {A.PREC_TF32X3: 1e-6, A.PREC_BF16X3: 5e-5, A.PREC_FP32: 1e-6}
TC_LENGTHS = [64, 256, 4096, 16384, 65536]


def _data(n, b, seed):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal((b, n)) + 1j * rng.standard_normal((b, n))).astype(np.complex64)


def _run(n, b, x, prec, direction=A.FORWARD, inplace=False, norm=None):
    dev = torch.device("cuda:0")
    xt = torch.from_numpy(x).to(dev)
    yt = xt if inplace else torch.empty_like(xt)
    with A.Plan.plan1d(n, A.C2C, b) as p:
        p.set_precision(prec)
        if norm is not None:
            p.set_norm(norm)
        info = p.info()
        p.set_stream(torch.cuda.current_stream(dev))
        p.exec_c2c(xt, yt, direction)
        torch.cuda.synchronize()
    return yt.cpu().numpy(), info


@pytest.mark.parametrize("prec", [A.PREC_TF32X3, A.PREC_BF16X3], ids=["tf32x3", "bf16x3"])
@pytest.mark.parametrize("n", TC_LENGTHS)
def test_tc_forward_vs_fp64(n, prec):
    b = 64 if n >= 16384 else 37
    x = _data(n, b, 12345 + n)
    y, info = _run(n, b, x, prec)
    assert info.tc_stages == (1 if n <= 256 else 2)
    e = O.errors(y, O.c2c(x, -1))
    assert e["rel_l2"] <= BOUND[prec], e


@pytest.mark.parametrize("prec", [A.PREC_TF32X3, A.PREC_BF16X3], ids=["tf32x3", "bf16x3"])
@pytest.mark.parametrize("n", [256, 16384])
def test_tc_backward_inplace_tail(n, prec):
    # batch 13: the last tile of the 256-point pass is partly empty
    b = 13
    x = _data(n, b, 7 + n)
    y, _ = _run(n, b, x, prec, direction=A.BACKWARD, inplace=True)
    e = O.errors(y, O.c2c(x, +1))
    assert e["rel_l2"] <= BOUND[prec], e


def test_tc_norm_and_fp32_comparison():
    n, b = 65536, 8
    x = _data(n, b, 99)
    exact = O.c2c(x, -1)
    errs = {}
    for prec in (A.PREC_FP32, A.PREC_TF32X3, A.PREC_BF16X3):
        y, info = _run(n, b, x, prec, norm=A.NORM_ORTHO)
        assert (info.tc_stages > 0) == (prec != A.PREC_FP32)
        errs[prec] = O.errors(y, exact / np.sqrt(n))
        assert errs[prec]["rel_l2"] <= BOUND[prec], (prec, errs[prec])
    # the TF32x3 form stays within a small factor of plain FP32 (measured on
    # GB300: 6.9e-7 vs 1.5e-7 at this size), the BF16x3 form well above it
    assert errs[A.PREC_TF32X3]["rel_l2"] <= 8 * max(errs[A.PREC_FP32]["rel_l2"], 1e-7)
    assert errs[A.PREC_BF16X3]["rel_l2"] > errs[A.PREC_TF32X3]["rel_l2"]


def test_tc_adjoint_matches_backward():
    n, b = 4096, 5
    x = _data(n, b, 3)
    dev = torch.device("cuda:0")
    xt = torch.from_numpy(x).to(dev)
    gt = torch.empty_like(xt)
    with A.Plan.plan1d(n, A.C2C, b) as p:
        p.set_precision(A.PREC_TF32X3)
        p.exec_c2c_adjoint(xt, gt, A.FORWARD)
        torch.cuda.synchronize()
    e = O.errors(gt.cpu().numpy(), O.c2c(x, +1))
    assert e["rel_l2"] <= BOUND[A.PREC_TF32X3], e


def test_tc_replan_switches_back():
    n, b = 256, 16
    x = _data(n, b, 5)
    dev = torch.device("cuda:0")
    xt = torch.from_numpy(x).to(dev)
    yt = torch.empty_like(xt)
    with A.Plan.plan1d(n, A.C2C, b) as p:
        p.set_precision(A.PREC_BF16X3)
        assert p.info().tc_stages == 1
        p.set_precision(A.PREC_FP32)
        assert p.info().tc_stages == 0 and p.precision() == A.PREC_FP32
        p.exec_c2c(xt, yt, A.FORWARD)
        torch.cuda.synchronize()
    e = O.errors(yt.cpu().numpy(), O.c2c(x, -1))
    assert e["rel_l2"] <= 1e-6, e


def test_tc_delta_and_constant_exact_shape():
    # impulse and constant inputs: exact spectra, so a wrong index map or a
    # wrong hi/lo recombination shows as a large error
    n, b = 16384, 2
    x = np.zeros((b, n), np.complex64)
    x[0, 1] = 1.0
    x[1, :] = 1.0 + 0.5j
    y, _ = _run(n, b, x, A.PREC_TF32X3)
    exact = O.c2c(x, -1)
    assert np.abs(y - exact).max() <= 2e-5 * n ** 0.5
