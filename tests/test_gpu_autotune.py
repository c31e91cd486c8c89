"""The plan autotuner (aclfftSetAutotune): CPU argument checks, and on the
GPU that tuned plans stay in bounds, match the FP64 oracle at the plain-FP32
bound (rel-L2 <= 1e-5), reuse cached choices, and survive a damaged cache
file."""
import ctypes
import json
import os
import subprocess
import sys

import numpy as np
import pytest

import aclfft as A
import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REL = 1e-5


def test_autotune_arguments():
    L = A.lib()
    assert L.aclfftSetAutotune(None, 1) == A.INVALID_PLAN
    h = ctypes.c_void_p()
    assert L.aclfftCreate(ctypes.byref(h)) == 0
    assert L.aclfftSetAutotune(h, 2) == A.INVALID_VALUE
    assert L.aclfftSetAutotune(h, 1) == A.SUCCESS      # recorded; MakePlan tunes when a device is present
    assert L.aclfftMakePlan1d(h, 3000, A.R2C, 16, 0, None) == A.SUCCESS
    assert L.aclfftDestroy(h) == 0


def _run(p, typ, n, b, torch, rng):
    dev = torch.device("cuda:0")
    if typ == A.C2C:
        x = (rng.standard_normal((b, n)) + 1j * rng.standard_normal((b, n))).astype(np.complex64)
        y = torch.empty((b, n), dtype=torch.complex64, device=dev)
        p.exec_c2c(torch.from_numpy(x).to(dev), y, A.FORWARD)
        exact = O.c2c(x, -1)
    elif typ == A.R2C:
        x = rng.standard_normal((b, n)).astype(np.float32)
        y = torch.empty((b, n // 2 + 1), dtype=torch.complex64, device=dev)
        p.exec_r2c(torch.from_numpy(x).to(dev), y)
        exact = O.r2c(x)
    else:
        x = (rng.standard_normal((b, n // 2 + 1)) + 1j * rng.standard_normal((b, n // 2 + 1))).astype(np.complex64)
        y = torch.empty((b, n), dtype=torch.float32, device=dev)
        p.exec_c2r(torch.from_numpy(x).to(dev), y)
        exact = O.c2r(x, n)
    torch.cuda.synchronize()
    return O.errors(y.cpu().numpy(), exact)


@pytest.mark.gpu
@pytest.mark.parametrize("n,typ,b", [(3000, A.R2C, 4096), (1024, A.C2R, 4096), (4096, A.C2C, 256),
                                     (4096, A.C2C, 2048), (16384, A.C2C, 64), (2048, A.C2C, 512)])
def test_tuned_plans_are_correct_and_cached(n, typ, b):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(n + b)
    with A.Plan.plan1d(n, typ, b) as p:
        p.set_autotune(True)
        inf = p.info()
        assert inf.tuned == 1 and inf.tune_candidates >= 1
        assert p.check() == "ok"
        e = _run(p, typ, n, b, torch, rng)
        assert e["rel_l2"] <= REL, e
        first = (inf.kernel, inf.groups_per_cta, inf.stages, inf.cluster_ctas, inf.nsteps)
    with A.Plan.plan1d(n, typ, b) as q:
        q.set_autotune(True)
        inf = q.info()
        assert inf.tuned == 1 and inf.tune_candidates == 0       # from the process cache
        assert (inf.kernel, inf.groups_per_cta, inf.stages, inf.cluster_ctas, inf.nsteps) == first


_CHILD = r"""
import json, sys
sys.path[:0] = [sys.argv[1] + "/ops-fft_gb300"]
import aclfft as A
with A.Plan.plan1d(1024, A.R2C, 512) as p:
    p.set_autotune(True)
    i = p.info()
    print(json.dumps({"tuned": i.tuned, "cand": i.tune_candidates, "kernel": i.kernel}))
"""


@pytest.mark.gpu
def test_cache_file_round_trip_and_damage(tmp_path):
    pytest.importorskip("torch")
    path = tmp_path / "plan_tune.txt"
    env = dict(os.environ, OPS_FFT_PLAN_TUNE_CACHE=str(path))

    def child():
        r = subprocess.run([sys.executable, "-c", _CHILD, ROOT], env=env, capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr[-2000:]
        return json.loads(r.stdout.strip().splitlines()[-1])

    a = child()
    assert a["tuned"] == 1 and a["cand"] >= 1 and path.exists()
    b = child()                                   # a new process reads the file
    assert b["tuned"] == 1 and b["cand"] == 0 and b["kernel"] == a["kernel"]
    lines = path.read_text().splitlines()
    path.write_text("garbage line\n" + "\n".join(l.rsplit(" ", 1)[0] + " 3" for l in lines) + "\n")
    c = child()                                   # every line damaged: re-tuned, no error
    assert c["tuned"] == 1 and c["cand"] >= 1
