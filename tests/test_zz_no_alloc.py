"""GPU test of the allocation-free long C2C entry point (aclfftExecC2CNoAlloc).

Some callers cannot allocate device memory: code that runs while another
component owns the device memory pool, or code that must not trigger the
synchronisation cudaMalloc/cudaFree may cause.  This entry point serves them:
its intermediate lives in a fixed device array built into the library.  The
test calls it through the C ABI twice in a row (different inputs, so stale
scratch contents would show) and compares each result with the plan-based
aclfftExecC2C on the same data; an in-place case is checked directly
against the FP64 oracle.  It is collected last so that a run stopping
at the first failure has already run everything else, and it passes both on
its own and after the rest of the suite.
"""
import ctypes

import numpy as np
import pytest

import aclfft as A
import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

# same FP32 arithmetic and twiddles as the plan path; allow rounding-level
# differences only
REL_TOL = 1e-6


def _rel(a, b):
    return float(torch.linalg.norm((a - b).reshape(-1)) / torch.linalg.norm(b.reshape(-1)))


@pytest.mark.parametrize("nx,batch", [(65536, 8), (46200, 4), (16384, 64)])
def test_no_alloc_matches_plan_path_on_two_calls(nx, batch):
    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    g = torch.Generator().manual_seed(nx + batch)
    with A.Plan.plan1d(nx, A.C2C, batch) as plan:
        plan.set_stream(stream)
        for call, direction in enumerate((A.FORWARD, A.BACKWARD)):
            x = torch.complex(torch.randn((batch, nx), generator=g), torch.randn((batch, nx), generator=g)).to(dev)
            ref = torch.empty_like(x)
            out = torch.full_like(x, float("nan"))
            plan.exec_c2c(x, ref, direction)
            rc = A.lib().aclfftExecC2CNoAlloc(x.data_ptr(), out.data_ptr(), nx, batch, direction,
                                             ctypes.c_void_p(stream.cuda_stream))
            assert rc == A.SUCCESS, (call, rc, A.last_error_detail())
            torch.cuda.synchronize()
            assert torch.isfinite(torch.view_as_real(out)).all()
            assert _rel(out, ref) <= REL_TOL, (call, _rel(out, ref))


@pytest.mark.parametrize("nx,batch", [(65536, 4), (46200, 2)])
def test_no_alloc_in_place_matches_fp64_oracle(nx, batch):
    """idata == odata (documented as allowed: the intermediate lives in the
    library's fixed array, never in the caller's buffer), checked directly
    against the FP64 oracle on two calls in a row, forward then backward."""
    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    rng = np.random.default_rng(nx)
    for direction in (A.FORWARD, A.BACKWARD):
        x = (rng.standard_normal((batch, nx)) + 1j * rng.standard_normal((batch, nx))).astype(np.complex64)
        buf = torch.from_numpy(x).to(dev)
        rc = A.lib().aclfftExecC2CNoAlloc(buf.data_ptr(), buf.data_ptr(), nx, batch, direction,
                                         ctypes.c_void_p(stream.cuda_stream))
        assert rc == A.SUCCESS, (rc, A.last_error_detail())
        torch.cuda.synchronize()
        e = O.errors(buf.cpu().numpy(), O.c2c(x, direction))
        assert e["rel_l2"] <= 1e-5, (direction, e)


def test_no_alloc_rejects_oversize_and_host_buffers():
    dev = torch.device("cuda:0")
    x = torch.zeros((1, 1 << 21), dtype=torch.complex64, device=dev)
    y = torch.empty_like(x)
    # 2^22 elements exceed the fixed 2^21-element scratch
    rc = A.lib().aclfftExecC2CNoAlloc(x.data_ptr(), y.data_ptr(), 1 << 21, 2, A.FORWARD, None)
    assert rc == A.INVALID_SIZE
    h = np.zeros(65536, dtype=np.complex64)
    rc = A.lib().aclfftExecC2CNoAlloc(h.ctypes.data, h.ctypes.data, 65536, 1, A.FORWARD, None)
    assert rc == A.INVALID_VALUE
