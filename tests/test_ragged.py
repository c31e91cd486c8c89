"""Ragged batches (aclfftRagged*): many transforms of different lengths and
kinds in one persistent launch.

CPU: argument validation, class/item construction and the host replay of
every work item's index ranges.  GPU: every transform of seeded ragged sets
against the FP64 oracle (rel-L2 <= 1e-5 per transform, the plain-FP32 bound),
both C2C directions, the graph replay path, the autotuner, and recording into
a caller's stream capture.
"""
import ctypes

import numpy as np
import pytest

import aclfft as A
import oracle as O

REL_FP32 = 1e-5


def _plan(lengths, types, align=256):
    ino, outo, ci, co = A.ragged_layout(lengths, types, align)
    return A.RaggedPlan(lengths, types, ino, outo), ino, outo, ci, co


# ------------------------------------------------------------------ CPU
def test_ragged_validation():
    L = ctypes.c_void_p()
    lens = np.array([64, 128], np.int32)
    typ = np.array([A.C2C, A.R2C], np.int32)
    off = np.array([0, 1024], np.int64)
    f = A.lib().aclfftRaggedPlanCreate
    assert f(None, 2, lens.ctypes.data, typ.ctypes.data, off.ctypes.data, off.ctypes.data) == A.INVALID_VALUE
    assert f(ctypes.byref(L), 0, lens.ctypes.data, typ.ctypes.data, off.ctypes.data, off.ctypes.data) == A.INVALID_SIZE
    bad_t = np.array([A.C2C, A.C2R], np.int32)
    assert f(ctypes.byref(L), 2, lens.ctypes.data, bad_t.ctypes.data, off.ctypes.data,
             off.ctypes.data) == A.INVALID_TYPE
    odd_off = np.array([0, 1020], np.int64)
    assert f(ctypes.byref(L), 2, lens.ctypes.data, typ.ctypes.data, odd_off.ctypes.data,
             off.ctypes.data) == A.INVALID_VALUE
    prime = np.array([64, 17 * 8], np.int32)
    assert f(ctypes.byref(L), 2, prime.ctypes.data, typ.ctypes.data, off.ctypes.data,
             off.ctypes.data) == A.NOT_SUPPORTED
    one = np.array([64, 1], np.int32)
    assert f(ctypes.byref(L), 2, one.ctypes.data, typ.ctypes.data, off.ctypes.data, off.ctypes.data) == A.INVALID_SIZE
    assert A.lib().aclfftRaggedExec(None, None, None, -1) == A.INVALID_PLAN
    with A.RaggedPlan(lens, typ, off, off) as p:
        assert A.lib().aclfftRaggedExec(p.handle, None, None, -1) == A.INVALID_VALUE
        host = np.zeros(4096, np.complex64)
        # host pointers are rejected (device pointers only)
        assert A.lib().aclfftRaggedExec(p.handle, host.ctypes.data, host.ctypes.data, -1) == A.INVALID_VALUE
        assert A.lib().aclfftRaggedExec(p.handle, host.ctypes.data, host.ctypes.data, 3) == A.INVALID_VALUE


def test_ragged_items_and_bounds():
    """Classes, long-transform splits, item order and index ranges of the
    config-5 workload (10000 transforms) and of edge sets, replayed on the
    host."""
    lengths, types = A.ragged_lengths(10000)
    p, ino, outo, ci, co = _plan(lengths, types)
    inf = p.info()
    assert inf.transforms == 10000
    cls = {(int(t), int(n)) for n, t in zip(lengths, types)}
    assert inf.classes == len(cls)
    r2c_half = np.where((types == A.R2C) & (lengths % 2 == 0), lengths // 2, lengths)
    assert inf.long_transforms == int(np.count_nonzero(r2c_half > 4096))
    assert inf.in_bytes_min <= ci and inf.out_bytes_min <= co
    assert p.check() == "ok"
    p.destroy()
    # edge sets: every kind of item, odd R2C, primes 11 and 13, lengths 2..3
    lens = np.array([2, 3, 5, 16, 11, 13 * 16, 4096, 4096, 8192, 8190, 15625, 16807, 32768,
                     2 * 3 * 5 * 7 * 11 * 13, 65536, 1 << 20, 3 ** 9], np.int32)
    for kinds in ([A.C2C] * len(lens), [A.R2C] * len(lens)):
        typ = np.array(kinds, np.int32)
        with _plan(lens, typ)[0] as q:
            assert q.check() == "ok"


def test_ragged_workload_generator():
    lengths, types = A.ragged_lengths(10000)
    assert lengths.min() >= 16 and lengths.max() <= 32768
    for n in np.unique(lengths):
        m = int(n)
        for pr in (2, 3, 5, 7):
            while m % pr == 0:
                m //= pr
        assert m == 1
    frac = float(np.mean(types == A.C2C))
    assert 0.67 < frac < 0.73
    # log-uniform: about half the draws fall below the geometric midpoint
    assert 0.4 < float(np.mean(lengths < np.sqrt(16 * 32768))) < 0.6


# ------------------------------------------------------------------ GPU
def _run(p, lengths, types, ino, outo, ci, co, seed, direction=A.FORWARD, graph=True, autotune=False):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(seed)
    hin = np.zeros(ci // 4, np.float32)
    xs = []
    for n, t, o in zip(lengths, types, ino):
        if t == A.C2C:
            x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
            hin[o // 4: o // 4 + 2 * n] = x.view(np.float32)
        else:
            x = rng.standard_normal(n).astype(np.float32)
            hin[o // 4: o // 4 + n] = x
        xs.append(x)
    din = torch.from_numpy(hin).to(dev)
    dout = torch.zeros(co // 4, dtype=torch.float32, device=dev)
    p.set_options(autotune=autotune, graph=graph)
    p.set_stream(torch.cuda.current_stream(dev))
    p.exec(din, dout, direction)
    torch.cuda.synchronize()
    assert p.error_flags() == 0
    hout = dout.cpu().numpy()
    errs = []
    for n, t, o, x in zip(lengths, types, outo, xs):
        if t == A.C2C:
            y = hout[o // 4: o // 4 + 2 * n].view(np.complex64)
            exact = O.c2c(x[None, :], direction)[0]
        else:
            y = hout[o // 4: o // 4 + 2 * (n // 2 + 1)].view(np.complex64)
            exact = O.r2c(x[None, :])[0]
        errs.append(O.errors(y, exact)["rel_l2"])
    return np.array(errs), din, dout


@pytest.mark.gpu
@pytest.mark.parametrize("direction", [A.FORWARD, A.BACKWARD])
def test_ragged_every_item_kind_vs_fp64(direction):
    # single groups (tiny to 4096), odd R2C, primes 11/13, and long C2C / even
    # and odd R2C (two dependent steps, post-process)
    lens = np.array([2, 3, 16, 16, 16, 11 * 13, 64, 100, 243, 1000, 2048, 4096, 5000, 8192, 8190, 9375, 16384,
                     16807, 32768, 3 ** 9, 30030, 65536], np.int32)
    lens = np.concatenate([lens, lens])
    types = np.array([A.C2C] * (len(lens) // 2) + [A.R2C] * (len(lens) // 2), np.int32)
    p, ino, outo, ci, co = _plan(lens, types)
    assert p.info().long_transforms > 0
    errs, _, _ = _run(p, lens, types, ino, outo, ci, co, seed=7, direction=direction)
    assert errs.max() <= REL_FP32, (lens[np.argmax(errs)], types[np.argmax(errs)], errs.max())
    p.destroy()


@pytest.mark.gpu
def test_ragged_config5_sample_graph_and_autotune():
    """A 600-transform slice of the config-5 distribution: graph replay (two
    execs, second from the captured graph), then the autotuned plan."""
    lengths, types = A.ragged_lengths(600, seed=3)
    p, ino, outo, ci, co = _plan(lengths, types)
    errs, din, dout = _run(p, lengths, types, ino, outo, ci, co, seed=11)
    assert errs.max() <= REL_FP32
    assert p.info().graph == 1
    # replay: same pointers, fresh output
    import torch

    dout.zero_()
    p.exec(din, dout, A.FORWARD)
    torch.cuda.synchronize()
    errs2, _, _ = _run(p, lengths, types, ino, outo, ci, co, seed=11, autotune=True)
    assert errs2.max() <= REL_FP32
    inf = p.info()
    assert inf.tuned_classes > 0
    assert p.check() == "ok"
    p.destroy()


@pytest.mark.gpu
def test_ragged_inside_caller_stream_capture():
    torch = pytest.importorskip("torch")
    lens = np.array([64, 3000, 4096, 8192, 20000], np.int32)
    types = np.array([A.C2C, A.R2C, A.C2C, A.R2C, A.C2C], np.int32)
    p, ino, outo, ci, co = _plan(lens, types)
    # warm-up exec (device setup) outside the capture
    errs, din, dout = _run(p, lens, types, ino, outo, ci, co, seed=5)
    assert errs.max() <= REL_FP32
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    p.set_stream(s)
    dout.zero_()
    torch.cuda.synchronize()
    with torch.cuda.graph(g, stream=s):
        p.exec(din, dout, A.FORWARD)
    g.replay()
    torch.cuda.synchronize()
    hout = dout.cpu().numpy()
    ref = np.zeros_like(hout)
    p2, *_ = _plan(lens, types)
    e2, _, d2 = _run(p2, lens, types, ino, outo, ci, co, seed=5)
    assert np.array_equal(hout, d2.cpu().numpy())
    p.destroy()
    p2.destroy()
