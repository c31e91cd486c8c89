"""torch.autograd wrappers over the aclfft C ABI (forward and adjoint kernels).

    import torch_fft as F
    X = F.rfft(x)            # x: (..., n) float32 CUDA tensor
    y = F.irfft(X, n)        # unnormalised, like the reference (n * irfft)
    Z = F.fft(z, inverse=False)

Every forward and backward call is one aclfftExec* / aclfftExec*Adjoint call
on the current torch stream.  Plans are cached per (kind, n, batch, device,
stream): a plan's stream and workspace are never shared by two streams, and
a per-plan lock serialises the host-side calls of threads that share a
stream (a plan is not thread-safe).
Gradients follow torch's complex convention (dL/dRe + i dL/dIm): the
backward of fft is the opposite-direction transform, the backward of rfft is
the R2C adjoint (C2R of the gradient with interior bins halved) and the
backward of irfft is the C2R adjoint (R2C of the gradient, interior bins
doubled).
"""
from __future__ import annotations

import threading

import torch

import aclfft as A

_plans = {}
_lock = threading.Lock()


def _plan(kind: int, n: int, batch: int, device: torch.device):
    """The cached plan for this shape on the current stream of `device`, and
    the lock that guards its use."""
    stream = torch.cuda.current_stream(device)
    key = (kind, n, batch, device.index, stream.cuda_stream)
    with _lock:
        entry = _plans.get(key)
        if entry is None:
            with torch.cuda.device(device):
                p = A.Plan.plan1d(n, kind, batch)
            p.set_stream(stream)  # bound once: the key includes the stream
            entry = (p, threading.Lock())
            _plans[key] = entry
    return entry


def _run(kind: int, n: int, batch: int, device: torch.device, method: str, *args) -> None:
    p, plock = _plan(kind, n, batch, device)
    with plock:
        getattr(p, method)(*args)


def clear_cache() -> None:
    with _lock:
        for p, _ in _plans.values():
            p.destroy()
        _plans.clear()


def _rows(x: torch.Tensor, n: int):
    if not x.is_cuda:
        raise ValueError("aclfft torch wrappers take CUDA tensors")
    x = x.contiguous()
    batch = x.numel() // n if n else 0
    return x, batch


class _C2C(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x: torch.Tensor, inverse: bool):
        n = x.shape[-1]
        x, b = _rows(x.to(torch.complex64), n)
        y = torch.empty_like(x)
        _run(A.C2C, n, b, x.device, "exec_c2c", x, y, A.BACKWARD if inverse else A.FORWARD)
        ctx.inverse = inverse
        return y

    @staticmethod
    def backward(ctx, g: torch.Tensor):
        n = g.shape[-1]
        g, b = _rows(g.to(torch.complex64), n)
        gx = torch.empty_like(g)
        _run(A.C2C, n, b, g.device, "exec_c2c_adjoint", g, gx, A.BACKWARD if ctx.inverse else A.FORWARD)
        return gx, None


class _R2C(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x: torch.Tensor):
        n = x.shape[-1]
        x, b = _rows(x.to(torch.float32), n)
        out = torch.empty(x.shape[:-1] + (n // 2 + 1,), dtype=torch.complex64, device=x.device)
        _run(A.R2C, n, b, x.device, "exec_r2c", x, out)
        ctx.n = n
        return out

    @staticmethod
    def backward(ctx, g: torch.Tensor):
        n = ctx.n
        g, b = _rows(g.to(torch.complex64), n // 2 + 1)
        gx = torch.empty(g.shape[:-1] + (n,), dtype=torch.float32, device=g.device)
        _run(A.R2C, n, b, g.device, "exec_r2c_adjoint", g, gx)
        return gx


class _C2R(torch.autograd.Function):
    @staticmethod
    def forward(ctx, X: torch.Tensor, n: int):
        X, b = _rows(X.to(torch.complex64), n // 2 + 1)
        out = torch.empty(X.shape[:-1] + (n,), dtype=torch.float32, device=X.device)
        _run(A.C2R, n, b, X.device, "exec_c2r", X, out)
        ctx.n = n
        return out

    @staticmethod
    def backward(ctx, g: torch.Tensor):
        n = ctx.n
        g, b = _rows(g.to(torch.float32), n)
        gX = torch.empty(g.shape[:-1] + (n // 2 + 1,), dtype=torch.complex64, device=g.device)
        _run(A.C2R, n, b, g.device, "exec_c2r_adjoint", g, gX)
        return gX, None


def fft(x: torch.Tensor, inverse: bool = False) -> torch.Tensor:
    """Unnormalised C2C over the last axis (inverse: exp(+2 pi i kn/N), no 1/N)."""
    return _C2C.apply(x, inverse)


def rfft(x: torch.Tensor) -> torch.Tensor:
    """R2C over the last axis: n real samples -> n//2+1 bins."""
    return _R2C.apply(x)


def irfft(X: torch.Tensor, n: int) -> torch.Tensor:
    """Unnormalised C2R (n * torch.fft.irfft) over the last axis."""
    return _C2R.apply(X, n)
