"""GPU tests of the library's failure reporting, allocation failures and the
work-area API, all through the C ABI.

Failures are made without faulting the GPU:
  * a ragged plan whose dependency waits are told to wait for one more
    completed item than exists (a count nothing reaches) with a ~1 ms wait
    limit: the wait runs out, the kernel records bit 2 and returns, and the
    host reads the flag;
  * a plan's device error word set by a test hook, as a kernel whose wait
    ran out would set it, to check that execs report it;
  * device allocations failed by a host-side hook (no real out-of-memory).
"""
import ctypes

import numpy as np
import pytest

import aclfft as A
import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

REL_FP32 = 1e-5


def _dev():
    return torch.device("cuda:0")


def _ragged_case():
    lens = np.array([100, 8192, 3000, 16384, 512], np.int32)   # two long (two-step) transforms
    kinds = np.array([A.C2C, A.C2C, A.R2C, A.R2C, A.C2C], np.int32)
    ino, outo, ci, co = A.ragged_layout(lens, kinds)
    rng = np.random.default_rng(9)
    hin = rng.standard_normal(ci // 4).astype(np.float32)
    return lens, kinds, ino, outo, co, hin


def _ragged_check(lens, kinds, ino, outo, hin, hout):
    worst = 0.0
    for n, t, io, oo in zip(lens, kinds, ino, outo):
        n = int(n)
        if t == A.C2C:
            ref = O.c2c(hin[io // 4: io // 4 + 2 * n].view(np.complex64)[None, :], -1)[0]
            got = hout[oo // 4: oo // 4 + 2 * n].view(np.complex64)
        else:
            ref = O.r2c(hin[io // 4: io // 4 + n][None, :])[0]
            got = hout[oo // 4: oo // 4 + 2 * (n // 2 + 1)].view(np.complex64)
        worst = max(worst, O.errors(got, ref)["rel_l2"])
    return worst


def test_ragged_wait_that_runs_out_is_reported_on_a_nonblocking_stream():
    dev = _dev()
    torch.cuda.set_device(dev)
    s = torch.cuda.Stream(dev)  # torch streams are created non-blocking
    lens, kinds, ino, outo, co, hin = _ragged_case()
    din = torch.from_numpy(hin).to(dev)
    dout = torch.zeros(co // 4, dtype=torch.float32, device=dev)
    with A.RaggedPlan(lens, kinds, ino, outo) as rp:
        assert rp.info().long_transforms >= 2
        rp.set_options(autotune=False, graph=True)
        rp.set_stream(s)
        rp.set_wait_limit(1 << 21)          # ~1 ms at 2 GHz
        rp.debug_hold_dependencies(1)       # every dependency count is one short
        rp.exec(din, dout, A.FORWARD)
        flags = ctypes.c_int()
        rc = A.lib().aclfftRaggedGetError(rp.handle, ctypes.byref(flags))
        assert rc == A.EXEC_FAILED and flags.value & 4, (rc, flags.value)
        assert rp.error_flags() == 0         # read once, then cleared
        # the context is still usable: the same plan runs correctly again
        rp.debug_hold_dependencies(0)
        rp.set_wait_limit(1 << 31)
        rp.exec(din, dout, A.FORWARD)
        assert rp.error_flags() == 0
        s.synchronize()
    assert _ragged_check(lens, kinds, ino, outo, hin, dout.cpu().numpy()) <= REL_FP32


def test_plan_error_word_is_reported_and_cleared():
    n, b = 4096, 8
    rng = np.random.default_rng(1)
    x = (rng.standard_normal((b, n)) + 1j * rng.standard_normal((b, n))).astype(np.complex64)
    out = np.empty_like(x)
    with A.Plan.plan1d(n, A.C2C, b) as p:
        assert p.exec_error() == 0
        # device-pointer execs are asynchronous: the flags are read on demand
        assert A.lib().aclfftDebugSetExecError(p.handle, 8) == A.SUCCESS
        f = ctypes.c_int()
        assert A.lib().aclfftGetExecError(p.handle, ctypes.byref(f)) == A.EXEC_FAILED and f.value == 8
        assert A.lib().aclfftGetExecError(p.handle, ctypes.byref(f)) == A.SUCCESS and f.value == 0
        # host-buffer execs read the word before returning
        assert A.lib().aclfftDebugSetExecError(p.handle, 1) == A.SUCCESS
        rc = A.lib().aclfftExecC2C(p.handle, x.ctypes.data, out.ctypes.data, A.FORWARD)
        assert rc == A.EXEC_FAILED
        assert "ran out" in A.last_error_detail()
        rc = A.lib().aclfftExecC2C(p.handle, x.ctypes.data, out.ctypes.data, A.FORWARD)
        assert rc == A.SUCCESS
    e = O.errors(out, O.c2c(x, -1))
    assert e["rel_l2"] <= REL_FP32, e


def test_allocation_failures_return_alloc_failed():
    L = A.lib()
    try:
        # the twiddle table is a plan's first device allocation
        L.aclfftDebugFailAllocations(0)
        h = ctypes.c_void_p()
        assert L.aclfftPlan1d(ctypes.byref(h), 4096, A.C2C, 4, 0) == A.ALLOC_FAILED
        assert not h.value
        # the workspace of a long transform (second allocation) fails
        L.aclfftDebugFailAllocations(1)
        assert L.aclfftPlan1d(ctypes.byref(h), 1 << 20, A.C2C, 2, 0) == A.ALLOC_FAILED
        assert not h.value
        # a ragged plan's device tables (set up by its first autotune or exec;
        # autotune touches no caller buffer)
        L.aclfftDebugFailAllocations(0)
        lens, kinds, ino, outo, co, hin = _ragged_case()
        with A.RaggedPlan(lens, kinds, ino, outo) as rp:
            with pytest.raises(A.AclfftError) as ei:
                rp.autotune()
            assert ei.value.code == A.ALLOC_FAILED
        # host staging buffers of a made plan
        L.aclfftDebugFailAllocations(-1)
        x = np.ones((2, 1024), dtype=np.complex64)
        with A.Plan.plan1d(1024, A.C2C, 2) as p:
            L.aclfftDebugFailAllocations(0)
            assert L.aclfftExecC2C(p.handle, x.ctypes.data, x.ctypes.data, A.FORWARD) == A.ALLOC_FAILED
            L.aclfftDebugFailAllocations(-1)
            assert L.aclfftExecC2C(p.handle, x.ctypes.data, x.ctypes.data, A.FORWARD) == A.SUCCESS
        assert np.allclose(x[:, 0], 1024) and np.allclose(x[:, 1:], 0, atol=1e-3)
    finally:
        L.aclfftDebugFailAllocations(-1)
    # nothing leaked into later plans
    with A.Plan.plan1d(1 << 20, A.C2C, 2) as p:
        assert p.work_size() > 0


@pytest.mark.parametrize("n,b,typ", [(1 << 20, 2, A.C2C), (46200, 3, A.C2C), (1 << 18, 4, A.R2C), (3000, 16, A.R2C)])
def test_caller_work_area(n, b, typ):
    """Auto allocation off: an exec that needs the work area returns
    ACLFFT_NO_WORKSPACE until aclfftSetWorkArea binds one; with the caller's
    area bound the results match the FP64 oracle, out of place and in place,
    and match the auto-allocating plan bit for bit."""
    dev = _dev()
    L = A.lib()
    rng = np.random.default_rng(n)
    if typ == A.C2C:
        x = (rng.standard_normal((b, n)) + 1j * rng.standard_normal((b, n))).astype(np.complex64)
        exact = O.c2c(x, -1)
        xd = torch.from_numpy(x).to(dev)
        yd = torch.empty_like(xd)
        nbuf = x.size * 2
    else:
        x = rng.standard_normal((b, n)).astype(np.float32)
        exact = O.r2c(x)
        xd = torch.from_numpy(x).to(dev)
        yd = torch.empty((b, n // 2 + 1), dtype=torch.complex64, device=dev)
        nbuf = b * 2 * (n // 2 + 1)

    def run(p, a, out):
        if typ == A.C2C:
            return L.aclfftExecC2C(p.handle, a.data_ptr(), out.data_ptr(), A.FORWARD)
        return L.aclfftExecR2C(p.handle, a.data_ptr(), out.data_ptr())

    h = ctypes.c_void_p()
    assert L.aclfftCreate(ctypes.byref(h)) == 0
    p = A.Plan(h.value)
    with p:
        p.set_auto_allocation(False)
        ws = ctypes.c_size_t()
        assert L.aclfftMakePlan1d(p.handle, n, typ, b, 0, ctypes.byref(ws)) == 0
        p.set_stream(torch.cuda.current_stream())
        ibuf = torch.zeros(nbuf, dtype=torch.float32, device=dev)
        ibuf[: xd.numel() * (2 if typ == A.C2C else 1)] = torch.view_as_real(xd).reshape(-1) if typ == A.C2C else xd.reshape(-1)
        rc_oop, rc_ip = run(p, xd, yd), run(p, ibuf, ibuf)
        needs = ws.value > 0
        if needs:
            assert A.NO_WORKSPACE in (rc_oop, rc_ip), (rc_oop, rc_ip, ws.value)
        area = torch.empty(max(ws.value, 1) // 4 + 64, dtype=torch.float32, device=dev)
        p.set_work_area(area)
        ibuf.zero_()
        ibuf[: xd.numel() * (2 if typ == A.C2C else 1)] = torch.view_as_real(xd).reshape(-1) if typ == A.C2C else xd.reshape(-1)
        assert run(p, xd, yd) == A.SUCCESS
        assert run(p, ibuf, ibuf) == A.SUCCESS
        torch.cuda.synchronize()
        assert p.exec_error() == 0
        y = yd.cpu().numpy()
        e = O.errors(y, exact)
        assert e["rel_l2"] <= REL_FP32, e
        yi = ibuf.cpu().numpy().view(np.complex64)[: y.size].reshape(y.shape)
        assert np.array_equal(yi, y)
        # re-enabling auto allocation keeps the caller's area bound
        p.set_auto_allocation(True)
        assert run(p, xd, yd) == A.SUCCESS
        torch.cuda.synchronize()
        assert np.array_equal(yd.cpu().numpy(), y)
    with A.Plan.plan1d(n, typ, b) as q:
        q.set_stream(torch.cuda.current_stream())
        y2 = torch.empty_like(yd)
        assert run(q, xd, y2) == A.SUCCESS
        torch.cuda.synchronize()
        assert np.array_equal(y2.cpu().numpy(), y)


def test_work_area_must_be_device_memory_of_the_plan():
    with A.Plan.plan1d(1 << 20, A.C2C, 2) as p:
        host = np.zeros(p.work_size() // 4 + 128, dtype=np.float32)
        base = (host.ctypes.data + 255) // 256 * 256
        assert A.lib().aclfftSetWorkArea(p.handle, base) == A.INVALID_VALUE
        area = torch.empty(p.work_size() // 4 + 128, dtype=torch.float32, device=_dev())
        assert A.lib().aclfftSetWorkArea(p.handle, area.data_ptr() + 4) == A.UNALIGNED_DATA
        assert A.lib().aclfftSetWorkArea(p.handle, area.data_ptr()) == A.SUCCESS
        assert A.lib().aclfftSetWorkArea(p.handle, None) == A.SUCCESS   # back to the plan's own
