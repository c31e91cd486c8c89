#!/usr/bin/env python
"""Benchmark of the batched FP32 transform path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--reps R] [--impl ours|reference]
                    [--workload cfg2|cfg1|cfg3|cfg4|cfg5|long|c2c3d|fp64] [--no-extras]

Prints ONE JSON line (rank 0).  Default workload (cfg2): the 1D R2C -> C2R
round trip with gradients at N = 3000 (2^3*3*5^3) and N = 1024, batch 4096,
x ~ N(0,1) float32, loss = sum(w*|X|^2) with w ~ U[0,1].  One step runs,
for each N: X = R2C(x), y = C2R(X) and dx = dL/dx = R2C-adjoint(2*w*X), the
weights 2w multiplied into X as the adjoint kernel loads it
(aclfftExecR2CAdjointWeighted).  `value` counts the algorithmic bytes of
the three transforms (one read of each transform's input + one write of its
output; the weights' reads are not counted) per second of the whole step.

Timing: inputs resident in HBM, rotating buffer sets whose total exceeds
2x the L2 size, W warm-up steps, then the K steps captured in one CUDA graph
on the launch stream, replayed R (>= 20) times, each replay between barriers
and device synchronisation and timed with CUDA events on that stream;
`value` comes from the median replay, max over ranks.  `roofline` times a
graph of K launches of the dominant kernel (R2C, N=3000) over the same
buffer sets the same way (median of R replays, divided by K); `e2e` repeats
the step through the C ABI with host (pinned) buffers, so the host<->device
copies are inside the timing; `cpu_baseline` times the reference's golden
path (torch.fft on the host cores) on the same workload.

With the default workload the line also carries, under `config`, the
comparison (C2C N = 65536 and 16384, batch 64) of the split-precision tensor-core forms against
the FP32 Stockham form with their FP64 errors, the per-length fractions of
the HBM roofline at N = 4096-65536, the same step run through the
torch.autograd wrappers (loss.backward()), the 2D/3D and double-precision
forms, and the other benchmark configurations (C2C 4096 x 256, the 2D
2048^2 x 8 step, the ragged launch).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "ops-fft_gb300"))

METRIC = "Batched C2C/R2C GB/s & % HBM roofline; split-TC vs FP32 Stockham at 1e-6 err"
FALLBACK_HBM_GBS = 6800.0

# DRAM traffic per launch of the dominant kernel measured by ncu
# (dram__bytes_read.sum + dram__bytes_write.sum), summarised under profiles/.
# Writes of a launch mostly stay in L2 when the kernel ends, so this is below
# the algorithmic read+write bytes.
NCU_TRAFFIC = {
    ("cfg2", "dominant"): 53330432,  # R2C N=3000 batch=4096: 49.22 MB read + 4.11 MB written
    ("cfg1", "dominant"): 8472064,   # C2C 4096 x 256 (row codelet): 8.47 MB read, the 8.4 MB output left in L2
    ("cfg3", "dominant"): 68792064,  # TF32x3 N=65536 x 64, both passes: 67.19 MB read + 1.60 MB written
    ("cfg4", "dominant"): 970750000,  # 2D forward: row pass 268.5 + 214.7 MB, column-tile pass 268.5 + 219.0 MB
    ("long", "dominant"): 487250944,  # C2C 65536 x 512 on 16-CTA clusters: 268.73 MB read + 218.52 MB written
    ("cfg5", "dominant"): 1086378752,  # ragged launch: 567.78 MB read + 518.60 MB written (workspace round trip)
}


def max_over_ranks(x, dist, device):
    """x maximised over all ranks of the process group (x itself without one).
    Every rank runs a full replica of the workload on its own GPU, so the
    whole job lasts as long as the slowest rank."""
    if dist is None:
        return x
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_gbs(alg_bytes_per_step, world, steps, seconds):
    """Algorithmic bytes of all ranks' steps per second of the slowest rank."""
    return alg_bytes_per_step * world * steps / seconds / 1e9


def _peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", FALLBACK_HBM_GBS)), "measured"
    return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during timing."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.tmp = None

    def start(self):
        try:
            self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=self.tmp, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.tmp.flush()
        rows = []
        with open(self.tmp.name) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.tmp.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(s):
            try:
                return float(s)
            except ValueError:
                return None

        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------- workloads
class Cfg2:
    """R2C -> C2R round trip with gradients, N in (3000, 1024), batch 4096.

    The two lengths are independent batches: the N=1024 chain runs on a
    second stream forked from and joined back to the launch stream inside
    each step, so its launches overlap the N=3000 chain (one step is still
    all the work of both lengths)."""

    name = "r2c_c2r_roundtrip_grad"

    def __init__(self, torch, A, dev, stream, nsets):
        self.torch, self.A = torch, A
        self.sizes = (3000, 1024)
        self.batch = 4096
        g = torch.Generator(device="cpu").manual_seed(12345)
        self.sets = []
        self.plans = {}
        self.stream = stream
        self.dev = dev
        self.side = torch.cuda.Stream(dev)
        self.streams = {3000: stream, 1024: self.side}
        for n in self.sizes:
            pr = A.Plan.plan1d(n, A.R2C, self.batch)
            pc = A.Plan.plan1d(n, A.C2R, self.batch)
            pr.set_stream(self.streams[n])
            pc.set_stream(self.streams[n])
            self.plans[n] = (pr, pc)
        for _ in range(nsets):
            s = {}
            for n in self.sizes:
                nb = n // 2 + 1
                x = torch.randn((self.batch, n), generator=g).to(dev)
                w2 = (2 * torch.rand((self.batch, nb), generator=g)).to(dev)
                s[n] = dict(x=x, w2=w2, X=torch.empty((self.batch, nb), dtype=torch.complex64, device=dev),
                            y=torch.empty_like(x), gx=torch.empty_like(x))
            self.sets.append(s)
        self.bytes_per_transform = {n: self.batch * (n * 4 + (n // 2 + 1) * 8) for n in self.sizes}
        self.alg_bytes_per_step = sum(3 * b for b in self.bytes_per_transform.values())
        self.launches_per_step = 3 * len(self.sizes)
        self.dominant = ("R2C N=3000 batch=4096 (fused even/odd post-process)", self.bytes_per_transform[3000])
        self.set_bytes = sum(t.numel() * t.element_size() for t in self.sets[0][3000].values()) + sum(
            t.numel() * t.element_size() for t in self.sets[0][1024].values())

    def step(self, i, dom_events=None):
        torch = self.torch
        s = self.sets[i % len(self.sets)]
        self.side.wait_stream(self.stream)  # fork: the step's inputs are ready
        for n in (1024, 3000):
            b = s[n]
            pr, pc = self.plans[n]
            with torch.cuda.stream(self.streams[n]):
                if dom_events is not None and n == 3000:
                    e0, e1 = dom_events
                    e0.record()
                    pr.exec_r2c(b["x"], b["X"])
                    e1.record()
                else:
                    pr.exec_r2c(b["x"], b["X"])
                pc.exec_c2r(b["X"], b["y"])
                # dL/dx = R2C adjoint of 2wX: the weights are applied as the
                # adjoint loads X (no separate elementwise pass)
                pr.exec_r2c_adjoint_weighted(b["X"], b["w2"], b["gx"])
        self.stream.wait_stream(self.side)  # join: the step ends when both chains are done

    def dom_call(self, i):
        b = self.sets[i % len(self.sets)][3000]
        self.plans[3000][0].exec_r2c(b["x"], b["X"])

    # host-buffer variant through the same C ABI (the reference's calling
    # convention: host pointers in and out, return means done)
    def make_host(self):
        torch = self.torch
        self.host = {}
        for n in self.sizes:
            s = self.sets[0][n]
            self.host[n] = {k: torch.empty(v.shape, dtype=v.dtype, pin_memory=True) for k, v in s.items()}
            for k, v in s.items():
                self.host[n][k].copy_(v.cpu())
            # host buffers: the gradient 2wX is formed on the host and passed
            # to the plain adjoint (the weighted entry takes device pointers)
            self.host[n]["G"] = torch.empty(s["X"].shape, dtype=torch.complex64, pin_memory=True)
            self.host[n]["G"].copy_((s["X"] * s["w2"]).cpu())
        h2d = sum(self.host[n][k].numel() * self.host[n][k].element_size()
                  for n in self.sizes for k in ("x", "X", "G"))
        d2h = sum(self.host[n][k].numel() * self.host[n][k].element_size()
                  for n in self.sizes for k in ("X", "y", "gx"))
        return h2d, d2h

    def step_host(self):
        # host buffers: each exec copies in, runs and synchronises its plan's
        # stream (the reference's calling convention).  The two lengths are
        # independent plans, so the N=1024 chain runs on a second host thread
        # (distinct plans may be used concurrently; ctypes releases the GIL)
        import threading

        errors = []

        def chain(n):
            try:
                self.torch.cuda.set_device(self.dev)
                h = self.host[n]
                pr, pc = self.plans[n]
                pr.exec_r2c(h["x"], h["X"])
                pc.exec_c2r(h["X"], h["y"])
                pr.exec_r2c_adjoint(h["G"], h["gx"])
            except Exception as e:  # noqa: BLE001 - re-raised on the calling thread
                errors.append(e)

        side = threading.Thread(target=chain, args=(1024,))
        side.start()
        chain(3000)
        side.join()
        if errors:
            raise errors[0]

    # CPU baseline: FP32 port of the reference path on a sample of rows
    def cpu_sample(self, O, rows, nthreads):
        import numpy as np

        rng = np.random.default_rng(0)
        done = 0
        t0 = time.perf_counter()
        for n in self.sizes:
            x = rng.standard_normal((rows, n)).astype(np.float32)
            X = O.port_r2c(x, nthreads)
            O.port_c2r(X, n, nthreads)
            Gh = X.copy()
            Gh[:, 1:(n + 1) // 2] *= 0.5  # R2C adjoint = C2R of the halved interior bins
            O.port_c2r(Gh, n, nthreads)
            done += 3 * rows * (n * 4 + (n // 2 + 1) * 8)
        return done, time.perf_counter() - t0

    def config(self):
        return {"workload": "1D R2C->C2R round trip with gradients (loss sum(w*|X|^2))", "n": list(self.sizes),
                "batch": self.batch, "dtype": "float32 / complex64 interleaved",
                "step": "per N: X = R2C(x), y = C2R(X), dx = R2C adjoint of 2wX (weights applied as the adjoint "
                        "loads X); the N=1024 chain on a second stream forked from and joined to the launch stream"}


class C2CWorkload:
    """Plain batched C2C (cfg1: 4096 x 256; cfg3: 65536 x 64 and 16384 x 64).

    ``prec`` selects the DFT-stage arithmetic (aclfftSetPrecisionMode): the
    FP32 Stockham kernels or the split-precision tensor-core forms."""

    FORM_NAMES = {0: "fp32 stockham", 1: "tf32x3 tensor-core", 2: "bf16x3 tensor-core"}

    def __init__(self, torch, A, dev, stream, nsets, sizes, name, uniform, prec=0):
        self.torch, self.A = torch, A
        self.sizes = sizes
        self.name = name
        self.stream = stream
        g = torch.Generator(device="cpu").manual_seed(12345)
        self.plans = {}
        self.sets = []
        for n, b in sizes:
            p = A.Plan.plan1d(n, A.C2C, b)
            p.set_stream(stream)
            self.plans[n] = p
        self.set_prec(prec)
        for _ in range(nsets):
            s = {}
            for n, b in sizes:
                if uniform:
                    x = torch.complex(torch.rand((b, n), generator=g) * 2 - 1, torch.rand((b, n), generator=g) * 2 - 1)
                else:
                    x = torch.complex(torch.randn((b, n), generator=g), torch.randn((b, n), generator=g))
                s[n] = dict(x=x.to(dev), y=torch.empty((b, n), dtype=torch.complex64, device=dev))
            self.sets.append(s)
        self.bytes_per_transform = {n: 16 * n * b for n, b in sizes}
        self.alg_bytes_per_step = sum(self.bytes_per_transform.values())
        self.dom_n = sizes[0][0]
        self.set_bytes = sum(16 * n * b for n, b in sizes)
        self._describe()

    def set_prec(self, prec):
        self.prec = prec
        for p in self.plans.values():
            p.set_precision(prec)
            p.set_stream(self.stream)
        if hasattr(self, "bytes_per_transform"):
            self._describe()

    def _describe(self):
        self.launches_per_step = sum(self.plans[n].info().nsteps for n, _ in self.sizes)
        n0, b0 = self.sizes[0]
        self.dominant = (f"C2C N={n0} batch={b0} ({self.FORM_NAMES[self.prec]})", self.bytes_per_transform[n0])

    def fp64_errors(self):
        """rel-L2 / max-abs of this form against torch's complex128 FFT of the
        same (first) input set, per length."""
        torch = self.torch
        out = {}
        s = self.sets[0]
        for n, _ in self.sizes:
            self.plans[n].exec_c2c(s[n]["x"], s[n]["y"], self.A.FORWARD)
            torch.cuda.synchronize()
            ref = torch.fft.fft(s[n]["x"].to(torch.complex128), dim=-1)
            d = s[n]["y"].to(torch.complex128) - ref
            out[str(n)] = {"rel_l2": float(torch.linalg.vector_norm(d) / torch.linalg.vector_norm(ref)),
                           "max_abs": float(d.abs().max())}
        return out

    def step(self, i, dom_events=None):
        s = self.sets[i % len(self.sets)]
        for n, _ in self.sizes:
            if dom_events is not None and n == self.dom_n:
                dom_events[0].record()
                self.plans[n].exec_c2c(s[n]["x"], s[n]["y"], self.A.FORWARD)
                dom_events[1].record()
            else:
                self.plans[n].exec_c2c(s[n]["x"], s[n]["y"], self.A.FORWARD)

    def dom_call(self, i):
        s = self.sets[i % len(self.sets)][self.dom_n]
        self.plans[self.dom_n].exec_c2c(s["x"], s["y"], self.A.FORWARD)

    def make_host(self):
        torch = self.torch
        self.host = {}
        for n, _ in self.sizes:
            s = self.sets[0][n]
            self.host[n] = {k: torch.empty(v.shape, dtype=v.dtype, pin_memory=True) for k, v in s.items()}
            self.host[n]["x"].copy_(s["x"].cpu())
        b = sum(16 * n * bb for n, bb in self.sizes) // 2
        return b, b

    def step_host(self):
        for n, _ in self.sizes:
            self.plans[n].exec_c2c(self.host[n]["x"], self.host[n]["y"], self.A.FORWARD)

    def cpu_sample(self, O, rows, nthreads):
        import numpy as np

        rng = np.random.default_rng(0)
        done = 0
        t0 = time.perf_counter()
        for n, b in self.sizes:
            r = max(1, min(b, rows * 4096 // n))
            x = (rng.standard_normal((r, n)) + 1j * rng.standard_normal((r, n))).astype(np.complex64)
            O.port_c2c(x, -1, nthreads)
            done += 16 * n * r
        return done, time.perf_counter() - t0

    def config(self):
        return {"workload": self.name, "sizes": [list(s) for s in self.sizes], "dtype": "complex64 interleaved"}


class OneExecWorkload:
    """One forward exec per step of a plan beyond the benchmark configurations, for
    measurement and profiling: ``c2c3d`` a 3D C2C of 512^3 (z rows, then
    512-point column tiles along y and x); ``fp64`` a double-precision Z2Z of
    4096 x 2048 (three FP64 Stockham passes)."""

    def __init__(self, torch, A, dev, stream, nsets, kind):
        self.torch, self.A, self.kind = torch, A, kind
        g = torch.Generator(device="cpu").manual_seed(12345)
        if kind == "c2c3d":
            self.shape, dt = (512, 512, 512), torch.complex64
            self.plan = A.Plan.plan3d(512, 512, 512)
            self.call = "exec_c2c"
            self.name = "3D C2C 512x512x512 forward"
        else:
            self.shape, dt = (2048, 4096), torch.complex128
            self.plan = A.Plan.plan1d(4096, A.Z2Z, 2048)
            self.call = "exec_z2z"
            self.name = "1D Z2Z (FP64) N=4096 batch=2048 forward"
        self.plan.set_stream(stream)
        self.sets = []
        for _ in range(nsets):
            x = torch.complex(torch.randn(self.shape, generator=g, dtype=dt.to_real()),
                              torch.randn(self.shape, generator=g, dtype=dt.to_real()))
            self.sets.append(dict(x=x.to(dev), y=torch.empty(self.shape, dtype=dt, device=dev)))
        per = 2 * self.sets[0]["x"].numel() * self.sets[0]["x"].element_size()
        self.alg_bytes_per_step = per
        self.launches_per_step = self.plan.info().nsteps
        self.dominant = (self.name, per)
        self.set_bytes = per

    def _exec(self, s):
        getattr(self.plan, self.call)(s["x"], s["y"], self.A.FORWARD)

    def step(self, i, dom_events=None):
        s = self.sets[i % len(self.sets)]
        if dom_events is not None:
            dom_events[0].record()
        self._exec(s)
        if dom_events is not None:
            dom_events[1].record()

    def dom_call(self, i):
        self._exec(self.sets[i % len(self.sets)])

    def make_host(self):
        torch = self.torch
        s = self.sets[0]
        self.host = {k: torch.empty(v.shape, dtype=v.dtype, pin_memory=True) for k, v in s.items()}
        self.host["x"].copy_(s["x"].cpu())
        b = self.alg_bytes_per_step // 2
        return b, b

    def step_host(self):
        self._exec(self.host)

    def cpu_sample(self, O, rows, nthreads):
        import numpy as np

        rng = np.random.default_rng(0)
        t0 = time.perf_counter()
        if self.kind == "c2c3d":
            # a 64 x 512 x 512 slab: rows, then the two strided axes
            x = (rng.standard_normal((64, 512, 512)) + 1j * rng.standard_normal((64, 512, 512))).astype(np.complex64)
            y = O.port_c2c(x.reshape(-1, 512), -1, nthreads).reshape(x.shape)
            y = O.port_c2c(np.ascontiguousarray(y.transpose(0, 2, 1)).reshape(-1, 512), -1, nthreads)
            O.port_c2c(y.reshape(64, 512 * 512).T.copy(), -1, nthreads)
            return 16 * x.size, time.perf_counter() - t0
        r = max(1, min(2048, rows))
        x = rng.standard_normal((r, 4096)) + 1j * rng.standard_normal((r, 4096))
        O.c2c(x, -1)
        return 32 * x.size, time.perf_counter() - t0

    def config(self):
        return {"workload": self.name, "shape": list(self.shape),
                "dtype": "complex64" if self.kind == "c2c3d" else "complex128",
                "launches_per_step": self.launches_per_step}


class Cfg4:
    """2D C2C 2048 x 2048, batch 8: forward, inverse normalised by 1/(2048^2),
    and the backward pass of L = sum Re(conj(Y) * G) (the adjoint of the
    forward transform applied to G)."""

    def __init__(self, torch, A, dev, stream, nsets):
        self.torch, self.A = torch, A
        self.b, self.nx, self.ny = 8, 2048, 2048
        g = torch.Generator(device="cpu").manual_seed(12345)
        shape = (self.b, self.nx, self.ny)
        self.pf = A.Plan.plan2d(self.b, self.nx, self.ny, A.C2C)
        self.pi = A.Plan.plan2d(self.b, self.nx, self.ny, A.C2C)
        self.pi.set_norm(A.NORM_BACKWARD)
        for p in (self.pf, self.pi):
            p.set_stream(stream)
        self.sets = []
        for _ in range(nsets):
            x = torch.complex(torch.rand(shape, generator=g) * 2 - 1, torch.rand(shape, generator=g) * 2 - 1)
            G = torch.complex(torch.randn(shape, generator=g), torch.randn(shape, generator=g))
            self.sets.append(dict(x=x.to(dev), G=G.to(dev), Y=torch.empty(shape, dtype=torch.complex64, device=dev),
                                  Z=torch.empty(shape, dtype=torch.complex64, device=dev),
                                  gx=torch.empty(shape, dtype=torch.complex64, device=dev)))
        per = 16 * self.b * self.nx * self.ny
        self.alg_bytes_per_step = 3 * per
        self.launches_per_step = 3 * self.pf.info().nsteps
        self.dominant = ("2D C2C 2048x2048 batch=8 forward (row + column pass)", per)
        self.set_bytes = 5 * per // 2

    def step(self, i, dom_events=None):
        s = self.sets[i % len(self.sets)]
        if dom_events is not None:
            dom_events[0].record()
        self.pf.exec_c2c(s["x"], s["Y"], self.A.FORWARD)
        if dom_events is not None:
            dom_events[1].record()
        self.pi.exec_c2c(s["Y"], s["Z"], self.A.BACKWARD)
        self.pf.exec_c2c_adjoint(s["G"], s["gx"], self.A.FORWARD)

    def dom_call(self, i):
        s = self.sets[i % len(self.sets)]
        self.pf.exec_c2c(s["x"], s["Y"], self.A.FORWARD)

    def make_host(self):
        torch = self.torch
        s = self.sets[0]
        self.host = {k: torch.empty(v.shape, dtype=v.dtype, pin_memory=True) for k, v in s.items()}
        for k, v in s.items():
            self.host[k].copy_(v.cpu())
        per = 8 * self.b * self.nx * self.ny
        return 3 * per, 3 * per

    def step_host(self):
        h = self.host
        self.pf.exec_c2c(h["x"], h["Y"], self.A.FORWARD)
        self.pi.exec_c2c(h["Y"], h["Z"], self.A.BACKWARD)
        self.pf.exec_c2c_adjoint(h["G"], h["gx"], self.A.FORWARD)

    def fp64_errors(self):
        torch = self.torch
        s = self.sets[0]
        self.step(0)
        torch.cuda.synchronize()
        x = s["x"][0].to(torch.complex128)
        ref = torch.fft.fft2(x)
        y = s["Y"][0].to(torch.complex128)
        rt = s["Z"].to(torch.complex128) - s["x"].to(torch.complex128)
        return {"forward_image0_rel_l2": float(torch.linalg.vector_norm(y - ref) / torch.linalg.vector_norm(ref)),
                "round_trip_rel_l2": float(torch.linalg.vector_norm(rt) / torch.linalg.vector_norm(s["x"]))}

    def cpu_sample(self, O, rows, nthreads):
        import numpy as np

        rng = np.random.default_rng(0)
        m = max(1, min(8, rows // 64))
        x = (rng.uniform(-1, 1, (m, self.nx, self.ny)) + 1j * rng.uniform(-1, 1, (m, self.nx, self.ny))).astype(
            np.complex64)
        t0 = time.perf_counter()
        # the port transforms rows; a 2D transform is rows then columns
        y = O.port_c2c(x.reshape(-1, self.ny), -1, nthreads).reshape(m, self.nx, self.ny)
        O.port_c2c(np.ascontiguousarray(y.transpose(0, 2, 1)).reshape(-1, self.nx), -1, nthreads)
        return 16 * m * self.nx * self.ny, time.perf_counter() - t0

    def config(self):
        return {"workload": "2D C2C 2048x2048 batch=8: forward, inverse (1/N^2), backward of sum Re(conj(Y) G)",
                "dtype": "complex64 interleaved", "launches_per_transform": self.pf.info().nsteps}


class Cfg5:
    """Ragged batch: 10000 1D transforms, lengths log-uniform over the 7-smooth
    integers in [16, 32768], 70% C2C / 30% R2C, x ~ N(0,1), one persistent
    launch per step (replayed CUDA graph, autotuned per-length plans)."""

    untuned = False

    def __init__(self, torch, A, dev, stream, nsets):
        import numpy as np

        self.torch, self.A = torch, A
        self.lengths, self.types = A.ragged_lengths(10000, seed=12345)
        self.ino, self.outo, ci, co = A.ragged_layout(self.lengths, self.types)
        self.plan = A.RaggedPlan(self.lengths, self.types, self.ino, self.outo)
        self.plan.set_stream(stream)
        if Cfg5.untuned:
            self.plan.set_options(autotune=False, graph=False)
        g = torch.Generator(device="cpu").manual_seed(12345)
        self.sets = []
        for _ in range(nsets):
            self.sets.append(dict(x=torch.randn(ci // 4, generator=g).to(dev),
                                  y=torch.zeros(co // 4, dtype=torch.float32, device=dev)))
        n = self.lengths.astype(np.int64)
        c2c = self.types == A.C2C
        self.alg_bytes_per_step = int(np.sum(np.where(c2c, 16 * n, 4 * n + 8 * (n // 2 + 1))))
        self.launches_per_step = 1
        self.dominant = ("ragged persistent launch (10000 transforms)", self.alg_bytes_per_step)
        self.set_bytes = ci + co
        self.in_bytes, self.out_bytes = ci, co

    def step(self, i, dom_events=None):
        s = self.sets[i % len(self.sets)]
        if dom_events is not None:
            dom_events[0].record()
        self.plan.exec(s["x"], s["y"], self.A.FORWARD)
        if dom_events is not None:
            dom_events[1].record()

    def dom_call(self, i):
        s = self.sets[i % len(self.sets)]
        self.plan.exec(s["x"], s["y"], self.A.FORWARD)

    def make_host(self):
        torch = self.torch
        self.hx = torch.empty(self.in_bytes // 4, dtype=torch.float32, pin_memory=True)
        self.hx.copy_(self.sets[0]["x"].cpu())
        self.hy = torch.empty(self.out_bytes // 4, dtype=torch.float32, pin_memory=True)
        return self.in_bytes, self.out_bytes

    def step_host(self):
        # the ragged entry point takes device pointers: the host path is the
        # copy in, the exec and the copy out, all on the plan's stream
        s = self.sets[0]
        s["x"].copy_(self.hx, non_blocking=True)
        self.plan.exec(s["x"], s["y"], self.A.FORWARD)
        self.hy.copy_(s["y"], non_blocking=True)

    def fp64_errors(self, sample=300):
        """Per-transform rel-L2 against torch's complex128 FFT for the first
        `sample` transforms: worst and median."""
        import numpy as np

        torch = self.torch
        s = self.sets[0]
        self.plan.exec(s["x"], s["y"], self.A.FORWARD)
        torch.cuda.synchronize()
        errs = []
        for n, t, io, oo in list(zip(self.lengths, self.types, self.ino, self.outo))[:sample]:
            n = int(n)
            if t == self.A.C2C:
                x = s["x"][io // 4: io // 4 + 2 * n].view(torch.complex64).to(torch.complex128)
                ref = torch.fft.fft(x)
                y = s["y"][oo // 4: oo // 4 + 2 * n].view(torch.complex64).to(torch.complex128)
            else:
                x = s["x"][io // 4: io // 4 + n].to(torch.float64)
                ref = torch.fft.rfft(x)
                y = s["y"][oo // 4: oo // 4 + 2 * (n // 2 + 1)].view(torch.complex64).to(torch.complex128)
            errs.append(float(torch.linalg.vector_norm(y - ref) / torch.linalg.vector_norm(ref)))
        return {"transforms_checked": len(errs), "worst_rel_l2": max(errs), "median_rel_l2": float(np.median(errs))}

    def cpu_sample(self, O, rows, nthreads):
        import numpy as np

        rng = np.random.default_rng(0)
        done = 0
        t0 = time.perf_counter()
        k = 0
        budget = rows * 4096 * 16  # bytes of transforms to sample
        for n, t in zip(self.lengths, self.types):
            n = int(n)
            if t == self.A.C2C:
                x = (rng.standard_normal((1, n)) + 1j * rng.standard_normal((1, n))).astype(np.complex64)
                O.port_c2c(x, -1, nthreads)
                done += 16 * n
            else:
                x = rng.standard_normal((1, n)).astype(np.float32)
                O.port_r2c(x, nthreads)
                done += 4 * n + 8 * (n // 2 + 1)
            k += 1
            if done >= budget:
                break
        self.cpu_transforms = k
        return done, time.perf_counter() - t0

    def config(self):
        inf = self.plan.info()
        return {"workload": "ragged batch: 10000 1D transforms in one persistent launch",
                "lengths": "log-uniform over 2^a 3^b 5^c 7^d in [16, 32768] (seed 12345)",
                "kinds": "70% C2C / 30% R2C", "classes": inf.classes, "long_transforms": inf.long_transforms,
                "work_items": inf.items, "tuned_classes": inf.tuned_classes, "cuda_graph": bool(inf.graph),
                "device_resident_bytes": int(self.set_bytes * len(self.sets) + inf.workspace_bytes +
                                             inf.twiddle_entries * 8)}


class LongWorkload:
    """Large batched C2C and R2C at N = 4096, 16384, 65536 (the lengths of
    the 70%-of-HBM target): 256 MB of complex input per C2C launch (128 MB
    of real input per R2C launch), far above the L2, x ~ N(0,1).  One step
    runs every (kind, N) once; each launch is timed with CUDA events so the
    per-length roofline fractions are reported next to the aggregate."""

    name = "long_c2c_r2c"
    LENGTHS = (4096, 16384, 65536)
    POINTS = 1 << 25  # complex points per C2C launch

    def __init__(self, torch, A, dev, stream, nsets):
        self.torch, self.A = torch, A
        g = torch.Generator(device=dev).manual_seed(12345)  # drawn on the GPU: 1 GB per set
        self.items = []  # (kind, n, batch, plan, bytes)
        for n in self.LENGTHS:
            b = self.POINTS // n
            for kind in ("C2C", "R2C"):
                p = A.Plan.plan1d(n, getattr(A, kind), b)
                p.set_stream(stream)
                byt = 16 * n * b if kind == "C2C" else b * (4 * n + 8 * (n // 2 + 1))
                self.items.append((kind, n, b, p, byt))
        self.sets = []
        for _ in range(nsets):
            s = {}
            for kind, n, b, _, _ in self.items:
                if kind == "C2C":
                    x = torch.complex(torch.randn((b, n), generator=g, device=dev),
                                      torch.randn((b, n), generator=g, device=dev))
                    y = torch.empty_like(x)
                else:
                    x = torch.randn((b, n), generator=g, device=dev)
                    y = torch.empty((b, n // 2 + 1), dtype=torch.complex64, device=dev)
                s[(kind, n)] = (x, y)
            self.sets.append(s)
        self.alg_bytes_per_step = sum(it[4] for it in self.items)
        self.launches_per_step = sum(it[3].info().nsteps for it in self.items)
        dom = max(self.items, key=lambda it: it[4] if it[0] == "C2C" and it[1] == 65536 else 0)
        self.dom_key = (dom[0], dom[1])
        self.dominant = (f"C2C N=65536 batch={dom[2]} (thread-block cluster, {dom[3].info().cluster_ctas} CTAs)",
                         dom[4])
        self.set_bytes = sum(x.numel() * x.element_size() + y.numel() * y.element_size()
                             for x, y in self.sets[0].values())
        self.per_item_ms = {}

    def _run(self, kind, p, x, y):
        if kind == "C2C":
            p.exec_c2c(x, y, self.A.FORWARD)
        else:
            p.exec_r2c(x, y)

    def step(self, i, dom_events=None):
        s = self.sets[i % len(self.sets)]
        for kind, n, b, p, _ in self.items:
            x, y = s[(kind, n)]
            if dom_events is not None:
                ev = self.item_events[(kind, n)]
                e0 = self.torch.cuda.Event(enable_timing=True)
                e1 = self.torch.cuda.Event(enable_timing=True)
                e0.record()
                self._run(kind, p, x, y)
                e1.record()
                ev.append((e0, e1))
            else:
                self._run(kind, p, x, y)

    def item_call(self, key, i):
        it = next(it for it in self.items if (it[0], it[1]) == key)
        x, y = self.sets[i % len(self.sets)][key]
        self._run(it[0], it[3], x, y)

    def dom_call(self, i):
        self.item_call(self.dom_key, i)

    def reset_item_events(self):
        self.item_events = {(it[0], it[1]): [] for it in self.items}

    def item_times_ms(self):
        return {k: statistics.mean(a.elapsed_time(b) for a, b in v) for k, v in self.item_events.items() if v}

    def make_host(self):
        torch = self.torch
        self.host = {}
        h2d = d2h = 0
        for kind, n, b, _, _ in self.items:
            x, y = self.sets[0][(kind, n)]
            hx = torch.empty(x.shape, dtype=x.dtype, pin_memory=True)
            hx.copy_(x.cpu())
            hy = torch.empty(y.shape, dtype=y.dtype, pin_memory=True)
            self.host[(kind, n)] = (hx, hy)
            h2d += hx.numel() * hx.element_size()
            d2h += hy.numel() * hy.element_size()
        return h2d, d2h

    def step_host(self):
        for kind, n, b, p, _ in self.items:
            hx, hy = self.host[(kind, n)]
            self._run(kind, p, hx, hy)

    def cpu_sample(self, O, rows, nthreads):
        import numpy as np

        rng = np.random.default_rng(0)
        done = 0
        t0 = time.perf_counter()
        for n in self.LENGTHS:
            r = max(1, rows * 4096 // n)
            x = (rng.standard_normal((r, n)) + 1j * rng.standard_normal((r, n))).astype(np.complex64)
            O.port_c2c(x, -1, nthreads)
            xr = rng.standard_normal((r, n)).astype(np.float32)
            O.port_r2c(xr, nthreads)
            done += r * (16 * n + 4 * n + 8 * (n // 2 + 1))
        return done, time.perf_counter() - t0

    def config(self):
        return {"workload": "large batched 1D C2C and R2C, N = 4096, 16384, 65536 (inputs far above L2)",
                "sizes": [[kind, n, b] for kind, n, b, _, _ in self.items],
                "dtype": "complex64 interleaved / float32 real"}


def make_workload(name, torch, A, dev, stream, nsets):
    if name == "cfg2":
        return Cfg2(torch, A, dev, stream, nsets)
    if name == "cfg1":
        return C2CWorkload(torch, A, dev, stream, nsets, [(4096, 256)], "1D C2C forward N=4096 batch=256", True)
    if name == "cfg3":
        return C2CWorkload(torch, A, dev, stream, nsets, [(65536, 64), (16384, 64)],
                           "1D C2C forward N=65536,16384 batch=64 (split-precision TF32x3 tensor-core form)", False,
                           prec=A.PREC_TF32X3)
    if name == "cfg4":
        return Cfg4(torch, A, dev, stream, nsets)
    if name == "cfg5":
        return Cfg5(torch, A, dev, stream, nsets)
    if name == "long":
        return LongWorkload(torch, A, dev, stream, nsets)
    if name in ("c2c3d", "fp64"):
        return OneExecWorkload(torch, A, dev, stream, nsets, name)
    raise SystemExit(f"unknown workload {name}")


# ------------------------------------------------------------- CPU baseline
# The reference's own CPU implementation of this path is its golden path:
# torch.fft on the host (pocketfft), called by its test-data generators,
#   rfft            src/rfft1_d/tests/rfft1_d_data/gen_data.py:88
#   irfft * n       src/irfft1_d/tests/irfft1_d_data/gen_data.py:62
#   fft / ifft * n  src/fft1_d/tests/fft1_d_data/gen_data.py:71-86
#   fft2 / ifft2    src/fft2_d/tests/fft2_d_data/gen_data.py:59-61
# (its transform kernels are Ascend C and do not run on this host).  Each
# golden step below runs the same transforms as the GPU step of the workload,
# on seeded CPU inputs of the same shapes, and returns the algorithmic bytes.
def golden_step(name, torch, fraction=1.0):
    """(step closure, algorithmic bytes per step, description) of the
    reference's golden path for workload `name` on `fraction` of its batch."""
    g = torch.Generator().manual_seed(12345)
    F = torch.fft

    def rows(b):
        return max(1, int(round(b * fraction)))

    if name == "cfg2":
        data = []
        for n in (3000, 1024):
            b = rows(4096)
            nb = n // 2 + 1
            half = torch.ones(nb)
            half[1:(n + 1) // 2] = 0.5
            data.append((n, torch.randn((b, n), generator=g), 2 * torch.rand((b, nb), generator=g), half))

        def step():
            for n, x, w2, half in data:
                X = F.rfft(x, dim=1)
                F.irfft(X, n=n, dim=1).mul_(n)
                G = X * w2
                F.irfft(G * half, n=n, dim=1).mul_(n)   # R2C adjoint: C2R of G, interior bins halved

        byt = sum(3 * x.shape[0] * (n * 4 + (n // 2 + 1) * 8) for n, x, _, _ in data)
        return step, byt, "per N in (3000, 1024): rfft, irfft*n, 2wX, irfft*n of the halved-interior gradient"
    if name in ("cfg1", "cfg3"):
        sizes = [(4096, 256)] if name == "cfg1" else [(65536, 64), (16384, 64)]
        xs = [torch.complex(torch.randn((rows(b), n), generator=g), torch.randn((rows(b), n), generator=g))
              for n, b in sizes]

        def step():
            for x in xs:
                F.fft(x, dim=1)

        return step, sum(16 * x.numel() for x in xs), "torch.fft.fft per length"
    if name == "cfg4":
        b = rows(8)
        x = torch.complex(torch.rand((b, 2048, 2048), generator=g) * 2 - 1, torch.rand((b, 2048, 2048), generator=g) * 2 - 1)
        G = torch.complex(torch.randn(x.shape, generator=g), torch.randn(x.shape, generator=g))

        def step():
            Y = F.fft2(x)
            F.ifft2(Y)
            F.ifft2(G).mul_(2048 * 2048)  # adjoint of the unnormalised forward

        return step, 3 * 16 * x.numel(), "fft2, ifft2 (1/N^2), ifft2*N^2 of G"
    if name == "cfg5":
        import numpy as np

        sys.path.insert(0, os.path.join(ROOT, "ops-fft_gb300"))
        import aclfft as A  # only its seeded workload recipe (pure Python)

        lengths, types = A.ragged_lengths(10000, seed=12345)
        cnt = rows(len(lengths))
        items = []
        for n, t in zip(lengths[:cnt], types[:cnt]):
            n = int(n)
            if t == A.C2C:
                items.append((True, torch.complex(torch.randn(n, generator=g), torch.randn(n, generator=g))))
            else:
                items.append((False, torch.randn(n, generator=g)))

        def step():
            for c2c, x in items:
                F.fft(x) if c2c else F.rfft(x)

        byt = int(sum(16 * x.numel() if c else 4 * x.numel() + 8 * (x.numel() // 2 + 1) for c, x in items))
        return step, byt, f"{cnt} of the 10000 ragged transforms, one torch.fft call each"
    if name == "long":
        data = []
        for n in (4096, 16384, 65536):
            b = rows((1 << 25) // n)
            data.append((torch.complex(torch.randn((b, n), generator=g), torch.randn((b, n), generator=g)),
                         torch.randn((b, n), generator=g)))

        def step():
            for xc, xr in data:
                F.fft(xc, dim=1)
                F.rfft(xr, dim=1)

        byt = sum(16 * xc.numel() + 4 * xr.numel() + 8 * xr.shape[0] * (xr.shape[1] // 2 + 1) for xc, xr in data)
        return step, byt, "torch.fft.fft and rfft per length"
    if name == "c2c3d":
        # the reference has no 3D path: torch.fft.fftn on the same volume
        x = torch.complex(torch.randn((512, 512, 512), generator=g), torch.randn((512, 512, 512), generator=g))

        def step():
            F.fftn(x)

        return step, 16 * x.numel(), "torch.fft.fftn of the 512^3 volume (no 3D path in the reference)"
    if name == "fp64":
        # the reference's double-precision entries are stubs: torch.fft in FP64
        b = rows(2048)
        x = torch.complex(torch.randn((b, 4096), generator=g, dtype=torch.float64),
                          torch.randn((b, 4096), generator=g, dtype=torch.float64))

        def step():
            F.fft(x, dim=1)

        return step, 32 * x.numel(), "torch.fft.fft in complex128 (the reference's Z2Z is a stub)"
    raise SystemExit(f"unknown workload {name}")


def time_golden(name, torch, threads, target_s, fraction=1.0, max_reps=50):
    """GB/s of the golden path on `threads` host threads: one warm-up step,
    then steps until about target_s seconds have passed."""
    torch.set_num_threads(threads)
    step, byt, what = golden_step(name, torch, fraction)
    step()
    reps, t = 0, 0.0
    while reps < max_reps and (reps < 2 or t < target_s):
        t0 = time.perf_counter()
        step()
        t += time.perf_counter() - t0
        reps += 1
    return byt * reps / t / 1e9, reps, what


def cpu_baseline(wl, name, torch):
    """The golden path on all host cores (the reported baseline), on one core,
    and the FP32 port of the reference's arch35 algorithm (secondary)."""
    cores = os.cpu_count() or 1
    v_all, reps, what = time_golden(name, torch, cores, 6.0)
    one_frac = 1.0 if name in ("cfg1", "cfg3", "cfg2") else 0.125
    v_one, reps1, _ = time_golden(name, torch, 1, 4.0, fraction=one_frac, max_reps=10)
    torch.set_num_threads(cores)
    port = None
    try:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O

        done, dt = wl.cpu_sample(O, 64, cores)
        port = round(done / dt / 1e9, 3)
    except Exception as e:  # noqa: BLE001 - the port is informational only
        port = f"unavailable: {type(e).__name__}"
    return {"value": round(v_all, 3), "unit": "GB/s", "cores": cores, "kind": "reference",
            "sample": f"the reference's golden path, torch {torch.__version__} torch.fft on CPU ({what}), "
                      f"full batch of the workload, {reps} steps on {cores} threads",
            "single_thread_value": round(v_one, 3),
            "single_thread_sample": f"{one_frac:g} of the batch, {reps1} steps on 1 thread",
            "port_value": port,
            "port_sample": "FP32 port of the reference's arch35 Stockham algorithm (oracle/oracle_fft.c port_*), "
                           "64 rows per length"}


# ------------------------------------------------------------------ timing
class GraphTimer:
    """Times fn(0..nk-1) as ONE CUDA graph on the work stream: captured,
    replayed once untimed, then `reps` replays, each bracketed by a barrier
    and device synchronisation and timed with CUDA events on that stream.
    Returns the per-replay milliseconds (None if the capture fails)."""

    def __init__(self, torch, stream, dist, notes):
        self.torch, self.stream, self.dist, self.notes = torch, stream, dist, notes

    def __call__(self, fn, nk, reps):
        torch = self.torch
        g = torch.cuda.CUDAGraph()
        try:
            with torch.cuda.graph(g, stream=self.stream):
                for i in range(nk):
                    fn(i)
        except Exception as e:  # noqa: BLE001 - report and time eagerly instead
            self.notes.append(f"graph capture failed ({type(e).__name__}: {str(e)[:120]}), eager launches")
            torch.cuda.synchronize()
            return None
        g.replay()
        torch.cuda.synchronize()
        out = []
        for _ in range(reps):
            t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            if self.dist:
                self.dist.barrier()
            torch.cuda.synchronize()
            t0.record(self.stream)
            g.replay()
            t1.record(self.stream)
            torch.cuda.synchronize()
            out.append(t0.elapsed_time(t1))
        if self.dist:
            self.dist.barrier()
        del g
        return out

    def eager(self, fn, nk, reps):
        torch = self.torch
        out = []
        for _ in range(reps):
            t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            if self.dist:
                self.dist.barrier()
            torch.cuda.synchronize()
            t0.record(self.stream)
            for i in range(nk):
                fn(i)
            t1.record(self.stream)
            torch.cuda.synchronize()
            out.append(t0.elapsed_time(t1))
        return out


def spread(v):
    return {"median": round(statistics.median(v), 5), "min": round(min(v), 5), "max": round(max(v), 5),
            "reps": len(v)}


def measure(wl, timer, nk, reps, warmup, torch):
    """(median ms of nk steps, per-replay ms list, median ms per dominant
    launch, per-item median ms for the long workload or None)."""
    for i in range(warmup):
        wl.step(i)
    torch.cuda.synchronize()
    steps = timer(wl.step, nk, reps) or timer.eager(wl.step, nk, reps)
    dom = timer(wl.dom_call, nk, reps) or timer.eager(wl.dom_call, nk, reps)
    per = None
    if isinstance(wl, LongWorkload):
        per = {}
        for key in [(it[0], it[1]) for it in wl.items]:
            f = lambda i, k=key: wl.item_call(k, i)
            t = timer(f, nk, reps) or timer.eager(f, nk, reps)
            per[key] = statistics.median(t) / nk
    return statistics.median(steps), steps, statistics.median(dom) / nk, per


def nsets_for(set_bytes, l2):
    return max(1, -(-2 * l2 // max(set_bytes, 1)) + (1 if set_bytes < 4 * l2 else 0))


def extra_split_tc_forms(torch, A, dev, stream, timer, nk, reps, warmup, l2, peak):
    """C2C N = 65536 and 16384, batch 64, in every arithmetic
    form: plain FP32 Stockham and the TF32x3 / BF16x3 split-precision
    tensor-core forms, each with GB/s, its dominant launch and its rel-L2 /
    max-abs error against torch's complex128 FFT of the same inputs."""
    probe_bytes = 16 * (65536 * 64 + 16384 * 64)
    wl = make_workload("cfg3", torch, A, dev, stream, nsets_for(probe_bytes, l2))
    forms = {}
    for prec in (A.PREC_FP32, A.PREC_TF32X3, A.PREC_BF16X3):
        wl.set_prec(prec)
        ms, _, dom, _ = measure(wl, timer, nk, reps, warmup, torch)
        forms[wl.FORM_NAMES[prec]] = {
            "GB/s": round(wl.alg_bytes_per_step * nk / (ms / 1e3) / 1e9, 1),
            "frac_of_measured_hbm": round(wl.alg_bytes_per_step * nk / (ms / 1e3) / 1e9 / peak, 3),
            "dominant_us": round(dom * 1e3, 2), "launches_per_step": wl.launches_per_step,
            "fp64_error": wl.fp64_errors()}
    del wl
    torch.cuda.empty_cache()
    fp32 = forms["fp32 stockham"]["GB/s"]
    best_tc = max((k for k in forms if k != "fp32 stockham" and
                   max(e["rel_l2"] for e in forms[k]["fp64_error"].values()) <= 1e-6),
                  key=lambda k: forms[k]["GB/s"], default=None)
    return {"workload": "C2C N=65536 and N=16384, batch 64, x ~ N(0,1)", "forms": forms,
            "fp64_reference": "torch.fft.fft in complex128 on the same device inputs",
            "best_split_form_within_1e-6": best_tc,
            "split_beats_fp32_within_1e-6": bool(best_tc and forms[best_tc]["GB/s"] > fp32)}


def extra_other_configs(torch, A, dev, stream, timer, nk, reps, warmup, l2, peak):
    """The remaining benchmark configurations measured in the same run, each
    its own workload with rotating buffer sets above 2x L2: C2C 4096 x 256,
    the 2D 2048^2 x 8 forward / inverse / backward step and the ragged
    10000-transform persistent launch; GB/s of algorithmic bytes, fraction
    of the measured HBM copy peak, the dominant launch and FP64 errors."""
    names = {"cfg1": "C2C N=4096 batch=256", "cfg4": "2D C2C 2048x2048 batch=8 forward + inverse + backward",
             "cfg5": "ragged 10000 transforms (70% C2C / 30% R2C, N in [16, 32768]) in one persistent launch"}
    out = {}
    for name, label in names.items():
        wl = make_workload(name, torch, A, dev, stream, 1)
        ns = nsets_for(wl.set_bytes, l2)
        if ns > 1:
            del wl
            torch.cuda.empty_cache()
            wl = make_workload(name, torch, A, dev, stream, ns)
        ms, _, dom, _ = measure(wl, timer, nk, reps, warmup, torch)
        gbs = wl.alg_bytes_per_step * nk / (ms / 1e3) / 1e9
        dom_gbs = wl.dominant[1] / (dom / 1e3) / 1e9
        out[label] = {"GB/s": round(gbs, 1), "frac_of_measured_hbm": round(gbs / peak, 3),
                      "ms_per_step": round(ms / nk, 4), "buffer_sets": ns,
                      "dominant": wl.dominant[0], "dominant_us": round(dom * 1e3, 2),
                      "dominant_frac_of_measured_hbm": round(dom_gbs / peak, 3), "fp64_error": wl.fp64_errors()}
        del wl
        torch.cuda.empty_cache()
    return out


def extra_long_lengths(torch, A, dev, stream, timer, nk, reps, warmup, l2, peak):
    """Batched C2C and R2C at N = 4096, 16384, 65536 with 2^25 complex points
    per C2C launch (inputs far above L2): per-length launch time and fraction
    of the measured HBM copy peak (the N = 4096-65536 >= 70 % target)."""
    wl = make_workload("long", torch, A, dev, stream, 2)
    _, _, _, per = measure(wl, timer, nk, reps, warmup, torch)
    out = {}
    for (kind, n), t_ms in per.items():
        byt = next(it[4] for it in wl.items if (it[0], it[1]) == (kind, n))
        gbs = byt / (t_ms / 1e3) / 1e9
        out[f"{kind} {n}"] = {"batch": next(it[2] for it in wl.items if (it[0], it[1]) == (kind, n)),
                              "us": round(t_ms * 1e3, 1), "GB/s": round(gbs, 1),
                              "frac_of_measured_hbm": round(gbs / peak, 3)}
    del wl
    torch.cuda.empty_cache()
    return out


def extra_multidim(torch, A, dev, stream, timer, nk, reps, warmup, peak):
    """2D and 3D forms beyond the reference's 2D C2C of 32-128 squares: per
    exec call on device buffers the median time, GB/s of one read of the
    input plus one write of the output, its fraction of the measured HBM copy
    peak, the launches per call, and cuFFT (torch.fft, unnormalised) on the
    same shape for scale.  Inputs and outputs are above the L2 size."""
    g = torch.Generator(device=dev).manual_seed(7)
    b, nx = 8, 2048
    xr = torch.rand((b, nx, nx), generator=g, device=dev) * 2 - 1
    xc = torch.complex(xr, torch.rand((b, nx, nx), generator=g, device=dev) * 2 - 1)
    yc = torch.empty_like(xc)
    Xh = torch.empty((b, nx, nx // 2 + 1), dtype=torch.complex64, device=dev)
    yr = torch.empty_like(xr)
    v = torch.complex(torch.rand((512,) * 3, generator=g, device=dev), torch.rand((512,) * 3, generator=g, device=dev))
    w = torch.empty_like(v)
    cases = [
        ("2D C2C 8x2048x2048", A.Plan.plan2d(b, nx, nx, A.C2C), lambda p: p.exec_c2c(xc, yc, A.FORWARD),
         lambda: torch.fft.fft2(xc, out=yc), 2 * xc.numel() * 8),
        ("2D R2C 8x2048x2048", A.Plan.plan2d(b, nx, nx, A.R2C), lambda p: p.exec_r2c(xr, Xh),
         lambda: torch.fft.rfft2(xr, out=Xh), xr.numel() * 4 + Xh.numel() * 8),
        ("2D C2R 8x2048x2048", A.Plan.plan2d(b, nx, nx, A.C2R), lambda p: p.exec_c2r(Xh, yr),
         lambda: torch.fft.irfft2(Xh, s=(nx, nx), norm="forward", out=yr), xr.numel() * 4 + Xh.numel() * 8),
        ("3D C2C 512^3", A.Plan.plan3d(512, 512, 512), lambda p: p.exec_c2c(v, w, A.FORWARD),
         lambda: torch.fft.fftn(v, out=w), 2 * v.numel() * 8),
    ]
    out = {}
    for name, plan, call, lib, byt in cases:
        plan.set_stream(stream)
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                call(plan)
                lib()
        torch.cuda.synchronize()
        t = timer(lambda i, p=plan, c=call: c(p), nk, reps) or timer.eager(lambda i, p=plan, c=call: c(p), nk, reps)
        tl = timer(lambda i: lib(), nk, reps) or timer.eager(lambda i: lib(), nk, reps)
        us = statistics.median(t) / nk * 1e3
        us_lib = statistics.median(tl) / nk * 1e3
        gbs = byt / (us / 1e6) / 1e9
        out[name] = {"us": round(us, 1), "GB/s": round(gbs, 1), "frac_of_measured_hbm": round(gbs / peak, 3),
                     "launches": plan.info().nsteps, "workspace_MB": round(plan.work_size() / 1e6, 1),
                     "cufft_us": round(us_lib, 1)}
        plan.destroy()
    del xr, xc, yc, Xh, yr, v, w
    torch.cuda.empty_cache()
    return out


def extra_double(torch, A, dev, stream, timer, nk, reps, warmup, peak):
    """Double precision (Z2Z / D2Z, one exec each on device buffers): time,
    GB/s of one read plus one write, nominal FP64 GFLOP/s (5 N log2 N per
    complex transform, half for a real one), and cuFFT (torch.fft on
    complex128 / float64) on the same shapes for scale."""
    import math

    g = torch.Generator(device=dev).manual_seed(9)
    z = torch.complex(torch.randn((2048, 4096), generator=g, device=dev, dtype=torch.float64),
                      torch.randn((2048, 4096), generator=g, device=dev, dtype=torch.float64))
    zo = torch.empty_like(z)
    r = torch.randn((4096, 3000), generator=g, device=dev, dtype=torch.float64)
    ro = torch.empty((4096, 1501), dtype=torch.complex128, device=dev)
    cases = [
        ("Z2Z 4096 x 2048", A.Plan.plan1d(4096, A.Z2Z, 2048), lambda p: p.exec_z2z(z, zo, A.FORWARD),
         lambda: torch.fft.fft(z, out=zo), 2 * z.numel() * 16, 2048 * 5 * 4096 * math.log2(4096)),
        ("D2Z 3000 x 4096", A.Plan.plan1d(3000, A.D2Z, 4096), lambda p: p.exec_d2z(r, ro),
         lambda: torch.fft.rfft(r, out=ro), r.numel() * 8 + ro.numel() * 16, 4096 * 2.5 * 3000 * math.log2(3000)),
    ]
    out = {}
    for name, plan, call, lib, byt, flops in cases:
        plan.set_stream(stream)
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                call(plan)
                lib()
        torch.cuda.synchronize()
        t = timer(lambda i, p=plan, c=call: c(p), nk, reps) or timer.eager(lambda i, p=plan, c=call: c(p), nk, reps)
        tl = timer(lambda i: lib(), nk, reps) or timer.eager(lambda i: lib(), nk, reps)
        us = statistics.median(t) / nk * 1e3
        out[name] = {"us": round(us, 1), "GB/s": round(byt / (us / 1e6) / 1e9, 1),
                     "frac_of_measured_hbm": round(byt / (us / 1e6) / 1e9 / peak, 3),
                     "fp64_GFLOP/s_nominal": round(flops / (us / 1e6) / 1e9, 1), "launches": plan.info().nsteps,
                     "cufft_us": round(statistics.median(tl) / nk * 1e3, 1)}
        plan.destroy()
    del z, zo, r, ro
    torch.cuda.empty_cache()
    return out


def extra_autograd(torch, dev, stream, nk, reps, warmup):
    """The headline step through the torch.autograd wrappers (torch_fft):
    X = rfft(x), y = irfft(X, n), loss = sum(w*|X|^2), loss.backward() -
    the gradient runs the library's R2C adjoint kernel.  Timed as a CUDA
    graph like the headline step; the gradient is compared with the explicit
    adjoint call of the headline step."""
    import torch_fft as TF

    g = torch.Generator(device="cpu").manual_seed(12345)
    b = 4096
    data = []
    for n in (3000, 1024):
        x = torch.randn((b, n), generator=g).to(dev).requires_grad_(True)
        w = torch.rand((b, n // 2 + 1), generator=g).to(dev)
        data.append((n, x, w))

    def step(i):
        for n, x, w in data:
            x.grad = None
            X = TF.rfft(x)
            TF.irfft(X.detach(), n)
            loss = (w * (X.real ** 2 + X.imag ** 2)).sum()
            loss.backward()

    with torch.cuda.stream(stream):
        for i in range(warmup):
            step(i)
    torch.cuda.synchronize()
    # parity of the autograd gradient with the explicit adjoint (2wX -> R2C adjoint)
    import aclfft as A

    errs = {}
    for n, x, w in data:
        with torch.no_grad():
            X = torch.fft.rfft(x.double())
            ref = torch.fft.irfft(2 * w.double() * X * torch.cat(
                [torch.ones(1, device=dev), torch.full(((n + 1) // 2 - 1,), 0.5, device=dev),
                 torch.ones(n // 2 + 1 - (n + 1) // 2, device=dev)]).double(), n=n) * n
            errs[str(n)] = float(torch.linalg.vector_norm(x.grad.double() - ref) / torch.linalg.vector_norm(ref))
    gr = torch.cuda.CUDAGraph()
    note = "one CUDA graph of the steps (forward + backward captured)"
    try:
        with torch.cuda.graph(gr, stream=stream):
            for i in range(nk):
                step(i)
        gr.replay()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            t0.record(stream)
            gr.replay()
            t1.record(stream)
            torch.cuda.synchronize()
            ts.append(t0.elapsed_time(t1))
    except Exception as e:  # noqa: BLE001
        note = f"eager (graph capture failed: {type(e).__name__})"
        ts = []
        for _ in range(reps):
            t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            with torch.cuda.stream(stream):
                t0.record(stream)
                for i in range(nk):
                    step(i)
                t1.record(stream)
            torch.cuda.synchronize()
            ts.append(t0.elapsed_time(t1))
    ms = statistics.median(ts) / nk
    byt = sum(3 * b * (n * 4 + (n // 2 + 1) * 8) for n in (3000, 1024))
    TF.clear_cache()
    return {"step": "per N in (3000, 1024): X = torch_fft.rfft(x), irfft(X), loss = sum(w|X|^2), loss.backward()",
            "ms_per_step": round(ms, 4), "GB/s": round(byt / (ms / 1e3) / 1e9, 1), "timing": note,
            "grad_rel_l2_vs_fp64_adjoint": errs}


# ------------------------------------------------------------------- main
def self_launch(gpus):
    """`bench.py --gpus N` outside a launcher: run N ranks under
    torch.distributed.run on this node (127.0.0.1) with the same arguments."""
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={gpus}",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__)] + sys.argv[1:]
    return subprocess.call(cmd)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--reps", type=int, default=21, help="timed replays of the K-step graph (median reported)")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cfg2")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="cfg2: skip the split-TC forms, per-length and autograd sub-measurements")
    ap.add_argument("--ragged-untuned", action="store_true",
                    help="cfg5: no autotuning and no graph replay (kernel profiling)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    args.reps = max(args.reps, 20)
    Cfg5.untuned = args.ragged_untuned

    if "WORLD_SIZE" not in os.environ and args.gpus > 1:
        return self_launch(args.gpus)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world != args.gpus:
        raise SystemExit(f"--gpus {args.gpus} but the launcher started WORLD_SIZE={world} ranks")

    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch
    import aclfft as A

    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    # all work runs on one non-default stream (the plans launch there, torch's
    # elementwise kernels too), so the timed steps can be captured in a CUDA graph
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    l2 = torch.cuda.get_device_properties(dev).L2_cache_size
    probe = make_workload(args.workload, torch, A, dev, stream, 1)
    nsets = nsets_for(probe.set_bytes, l2)
    del probe
    torch.cuda.empty_cache()
    wl = make_workload(args.workload, torch, A, dev, stream, nsets)
    notes = []
    timer = GraphTimer(torch, stream, dist, notes)
    nk, reps = args.steps, args.reps
    peak, peak_kind = _peaks()

    forms = None
    if isinstance(wl, C2CWorkload):
        # every arithmetic form of the same workload, for comparison; the
        # headline line is then timed in the workload's own form
        forms = {}
        own = wl.prec
        for prec in (A.PREC_FP32, A.PREC_BF16X3, A.PREC_TF32X3):
            wl.set_prec(prec)
            f_ms, _, f_dom, _ = measure(wl, timer, nk, reps, args.warmup, torch)
            forms[wl.FORM_NAMES[prec]] = {
                "GB/s": round(wl.alg_bytes_per_step * nk / (f_ms / 1e3) / 1e9, 1),
                "dominant_us": round(f_dom * 1e3, 2), "launches_per_step": wl.launches_per_step,
                "fp64_error": wl.fp64_errors()}
        wl.set_prec(own)
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    time.sleep(0.3)
    ms, replays, dom_ms, per_item = measure(wl, timer, nk, reps, args.warmup, torch)
    clk = clocks.stop()
    ms = max_over_ranks(ms, dist, dev)
    ms_per_step = ms / nk
    value = whole_job_gbs(wl.alg_bytes_per_step, world, nk, ms / 1e3)

    achieved = wl.dominant[1] / (dom_ms / 1e3) / 1e9
    traffic = NCU_TRAFFIC.get((args.workload, "dominant"))
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic, "peak_source": peak_kind,
                "kernel": wl.dominant[0], "alg_bytes_per_launch": wl.dominant[1],
                "avg_launch_us": round(dom_ms * 1e3, 2),
                "timing": f"median of {reps} replays of a graph of {nk} launches, divided by {nk}"}

    e2e = None
    if not args.no_e2e:
        h2d, d2h = wl.make_host()
        for _ in range(2):
            wl.step_host()
        torch.cuda.synchronize()
        ke = 3 if isinstance(wl, LongWorkload) else max(3, min(nk, 30))
        if dist:
            dist.barrier()
        ts = time.perf_counter()
        for _ in range(ke):
            wl.step_host()
        torch.cuda.synchronize()
        te = time.perf_counter() - ts
        te = max_over_ranks(te, dist, dev)
        e2e = {"value": round(whole_job_gbs(wl.alg_bytes_per_step, world, ke, te), 2), "unit": "GB/s",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "path": "aclfftExec* with pinned host buffers (library stages and synchronises)",
               "steps_timed": ke}

    extras = {}
    if args.workload == "cfg2" and not args.no_extras:
        del wl
        torch.cuda.empty_cache()
        extras["split_tc_vs_fp32"] = extra_split_tc_forms(torch, A, dev, stream, timer, nk, reps, args.warmup, l2,
                                                          peak)
        extras["per_length_n4096_65536"] = extra_long_lengths(torch, A, dev, stream, timer, nk, max(5, reps // 4),
                                                              args.warmup, l2, peak)
        extras["autograd_step"] = extra_autograd(torch, dev, stream, nk, max(5, reps // 4), args.warmup)
        extras["multidim_2d_3d"] = extra_multidim(torch, A, dev, stream, timer, nk, max(5, reps // 4), args.warmup,
                                                  peak)
        extras["double_precision"] = extra_double(torch, A, dev, stream, timer, nk, max(5, reps // 4), args.warmup,
                                                  peak)
        extras["other_configs"] = extra_other_configs(torch, A, dev, stream, timer, nk, max(5, reps // 4),
                                                      args.warmup, l2, peak)
        wl = make_workload(args.workload, torch, A, dev, stream, 1)

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(wl, args.workload, torch)

    if rank == 0:
        cfg = wl.config()
        cfg["l2_strategy"] = f"{nsets} rotating buffer sets, {nsets * wl.set_bytes / 1e6:.0f} MB total > 2x L2 ({l2 / 1e6:.0f} MB)"
        cfg["parallelism"] = f"replicas x{world} (independent batches, no collective)"
        cfg["timing"] = (notes[-1] if notes else
                         f"one CUDA graph of {nk} steps replayed {reps} times, each replay timed with CUDA events "
                         f"on the launch stream between barriers; value from the median replay")
        cfg["replay_ms"] = spread(replays)
        if isinstance(wl, (Cfg4, Cfg5)):
            cfg["fp64_error"] = wl.fp64_errors()
        if isinstance(wl, LongWorkload):
            per = {}
            for (kind, n), t_ms in per_item.items():
                byt = next(it[4] for it in wl.items if (it[0], it[1]) == (kind, n))
                gbs = byt / (t_ms / 1e3) / 1e9
                per[f"{kind} {n}"] = {"us": round(t_ms * 1e3, 1), "GB/s": round(gbs, 1),
                                      "frac_of_measured_hbm": round(gbs / peak, 3)}
            cfg["per_length"] = per
        if forms is not None:
            cfg["forms"] = forms
            cfg["fp64_reference"] = "torch.fft.fft in complex128 on the same device inputs"
        cfg.update(extras)
        line = {"metric": METRIC, "value": round(value, 1), "unit": "GB/s", "n_gpus": world, "steps": nk,
                "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded, the workload's shapes and distributions)",
                "config": cfg, "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
                "gpu_launches": wl.launches_per_step * nk, "clocks": clk}
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def run_reference(args, rank, world):
    """The reference's own CPU implementation of the path: its golden
    torch.fft path on the host cores (all threads), on the same workload and
    full batch as our arm, K timed steps after W warm-up steps.  Under
    torchrun only rank 0 runs and prints."""
    if rank != 0:
        return
    import torch

    cores = os.cpu_count() or 1
    torch.set_num_threads(cores)
    fraction = 1.0 if args.workload in ("cfg1", "cfg2", "cfg3", "cfg4", "cfg5") else 0.125
    step, byt, what = golden_step(args.workload, torch, fraction)
    for _ in range(args.warmup):
        step()
    ts = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        step()
        ts.append(time.perf_counter() - t0)
    t = sum(ts)
    value = byt * args.steps / t / 1e9
    cfg = {"workload": args.workload, "sample": f"{fraction:g} of the batch per step ({what})",
           "same_config": fraction == 1.0}
    sample = (f"the reference's golden path, torch {torch.__version__} torch.fft on CPU ({what}), {fraction:g} of "
              f"the workload's batch per step, {cores} threads")
    line = {"metric": METRIC, "value": round(value, 3), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(t / args.steps * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded, the workload's shapes and distributions)",
            "impl": "reference", "config": cfg,
            "cpu_baseline": {"value": round(value, 3), "unit": "GB/s", "cores": cores, "kind": "reference",
                             "sample": sample},
            "e2e": {"value": round(value, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


if __name__ == "__main__":
    sys.exit(main())
