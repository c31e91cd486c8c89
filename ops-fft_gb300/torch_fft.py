"""torch.autograd wrappers over the aclfft C ABI (forward and adjoint kernels).

    import torch_fft as F
    X = F.rfft(x)            # x: (..., n) float32 CUDA tensor
    y = F.irfft(X, n)        # unnormalised, like the reference (n * irfft)
    Z = F.fft(z, inverse=False)
    X2 = F.rfft2(x2)         # (..., nx, ny) -> (..., nx, ny//2+1)
    y2 = F.irfft2(X2, (nx, ny))
    Z2 = F.fft2(z2); Z3 = F.fftn(z3)   # 2D / 3D C2C over the last axes
    X3 = F.rfftn(x3)         # (..., nx, ny, nz) -> (..., nx, ny, nz//2+1)
    y3 = F.irfftn(X3, (nx, ny, nz))

complex128 / float64 tensors run in double precision (Z2Z, D2Z and Z2D of
rank 1-3); everything else in single precision.

Every forward and backward call is one aclfftExec* / aclfftExec*Adjoint call
on the current torch stream (3D: one call per leading batch item, the 3D
plans have no batch).  Plans are cached per (kind, dims, batch, device,
stream): a plan's stream and workspace are never shared by two streams, and
a per-plan lock serialises the host-side calls of threads that share a
stream (a plan is not thread-safe).
Gradients follow torch's complex convention (dL/dRe + i dL/dIm): the
backward of fft is the opposite-direction transform, the backward of rfft is
the R2C adjoint (C2R of the gradient with interior bins halved) and the
backward of irfft is the C2R adjoint (R2C of the gradient, interior bins
doubled); the 2D and 3D forms compose the same way along their slower
axes.
"""
from __future__ import annotations

import math
import threading

import torch

import aclfft as A

_plans = {}
_lock = threading.Lock()


def _plan(kind: int, dims: tuple, batch: int, device: torch.device):
    """The cached plan for this shape on the current stream of `device`, and
    the lock that guards its use."""
    stream = torch.cuda.current_stream(device)
    key = (kind, dims, batch, device.index, stream.cuda_stream)
    with _lock:
        entry = _plans.get(key)
        if entry is None:
            with torch.cuda.device(device):
                if len(dims) == 1:
                    p = A.Plan.plan1d(dims[0], kind, batch)
                elif len(dims) == 2:
                    p = A.Plan.plan2d(batch, dims[0], dims[1], kind)
                else:
                    p = A.Plan.plan3d(*dims, kind)
            p.set_stream(stream)  # bound once: the key includes the stream
            entry = (p, threading.Lock())
            _plans[key] = entry
    return entry


def _run(kind: int, dims: tuple, batch: int, device: torch.device, method: str, x, y, *rest) -> None:
    if len(dims) == 3 and batch > 1:  # one batch-1 plan, one call per volume
        p, plock = _plan(kind, dims, 1, device)
        xv, yv = x.reshape(batch, -1), y.reshape(batch, -1)
        with plock:
            for i in range(batch):
                getattr(p, method)(xv[i], yv[i], *rest)
        return
    p, plock = _plan(kind, dims, batch, device)
    with plock:
        getattr(p, method)(x, y, *rest)


def clear_cache() -> None:
    with _lock:
        for p, _ in _plans.values():
            p.destroy()
        _plans.clear()


def _rows(x: torch.Tensor, per: int):
    """Contiguous x and the number of transforms of `per` elements in it."""
    if not x.is_cuda:
        raise ValueError("aclfft torch wrappers take CUDA tensors")
    x = x.contiguous()
    batch = x.numel() // per if per else 0
    return x, batch


def _half(dims: tuple) -> tuple:
    return tuple(dims[:-1]) + (dims[-1] // 2 + 1,)


def _interior(n: int, value: float, device, dtype) -> torch.Tensor:
    """Per-bin factor of an n-point real transform's n//2+1 bins: `value` on
    the interior bins, 1 at DC and (even n) Nyquist."""
    w = torch.full((n // 2 + 1,), value, dtype=dtype, device=device)
    w[0] = 1
    if n % 2 == 0:
        w[-1] = 1
    return w


class _C2C(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x: torch.Tensor, inverse: bool, nd: int):
        dims = tuple(x.shape[-nd:])
        dbl = x.dtype == torch.complex128
        x, b = _rows(x.to(torch.complex128 if dbl else torch.complex64), math.prod(dims))
        y = torch.empty_like(x)
        _run(A.Z2Z if dbl else A.C2C, dims, b, x.device, "exec_z2z" if dbl else "exec_c2c", x, y,
             A.BACKWARD if inverse else A.FORWARD)
        ctx.inverse = inverse
        ctx.dims = dims
        ctx.dbl = dbl
        return y

    @staticmethod
    def backward(ctx, g: torch.Tensor):
        if ctx.dbl:
            # the adjoint of an unnormalised transform is the opposite-direction one
            g, b = _rows(g.to(torch.complex128), math.prod(ctx.dims))
            gx = torch.empty_like(g)
            _run(A.Z2Z, ctx.dims, b, g.device, "exec_z2z", g, gx, A.FORWARD if ctx.inverse else A.BACKWARD)
            return gx, None, None
        g, b = _rows(g.to(torch.complex64), math.prod(ctx.dims))
        gx = torch.empty_like(g)
        _run(A.C2C, ctx.dims, b, g.device, "exec_c2c_adjoint", g, gx, A.BACKWARD if ctx.inverse else A.FORWARD)
        return gx, None, None


class _R2C(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x: torch.Tensor, nd: int):
        dims = tuple(x.shape[-nd:])
        dbl = x.dtype == torch.float64
        x, b = _rows(x.to(torch.float64 if dbl else torch.float32), math.prod(dims))
        out = torch.empty(x.shape[:-1] + (dims[-1] // 2 + 1,), dtype=torch.complex128 if dbl else torch.complex64,
                          device=x.device)
        _run(A.D2Z if dbl else A.R2C, dims, b, x.device, "exec_d2z" if dbl else "exec_r2c", x, out)
        ctx.dims = dims
        ctx.dbl = dbl
        return out

    @staticmethod
    def backward(ctx, g: torch.Tensor):
        dims = ctx.dims
        if ctx.dbl:
            # R2C adjoint: C2R of the gradient with its interior bins halved
            n = dims[-1]
            g = g.to(torch.complex128) * _interior(n, 0.5, g.device, torch.float64)
            g, b = _rows(g, math.prod(_half(dims)))
            gx = torch.empty(g.shape[:-1] + (n,), dtype=torch.float64, device=g.device)
            _run(A.Z2D, dims, b, g.device, "exec_z2d", g, gx)
            return gx, None
        g, b = _rows(g.to(torch.complex64), math.prod(_half(dims)))
        gx = torch.empty(g.shape[:-1] + (dims[-1],), dtype=torch.float32, device=g.device)
        _run(A.R2C, dims, b, g.device, "exec_r2c_adjoint", g, gx)
        return gx, None


class _C2R(torch.autograd.Function):
    @staticmethod
    def forward(ctx, X: torch.Tensor, dims: tuple):
        if tuple(X.shape[-len(dims):]) != _half(dims):
            raise ValueError(f"C2R to {dims} takes (..., {', '.join(map(str, _half(dims)))}) bins, got {tuple(X.shape)}")
        dbl = X.dtype == torch.complex128
        X, b = _rows(X.to(torch.complex128 if dbl else torch.complex64), math.prod(_half(dims)))
        out = torch.empty(X.shape[:-1] + (dims[-1],), dtype=torch.float64 if dbl else torch.float32, device=X.device)
        _run(A.Z2D if dbl else A.C2R, dims, b, X.device, "exec_z2d" if dbl else "exec_c2r", X, out)
        ctx.dims = dims
        ctx.dbl = dbl
        return out

    @staticmethod
    def backward(ctx, g: torch.Tensor):
        dims = ctx.dims
        if ctx.dbl:
            # C2R adjoint: R2C of the gradient with its interior bins doubled
            n = dims[-1]
            g, b = _rows(g.to(torch.float64), math.prod(dims))
            gX = torch.empty(g.shape[:-1] + (n // 2 + 1,), dtype=torch.complex128, device=g.device)
            _run(A.D2Z, dims, b, g.device, "exec_d2z", g, gX)
            return gX * _interior(n, 2.0, g.device, torch.float64), None
        g, b = _rows(g.to(torch.float32), math.prod(dims))
        gX = torch.empty(g.shape[:-1] + (dims[-1] // 2 + 1,), dtype=torch.complex64, device=g.device)
        _run(A.C2R, dims, b, g.device, "exec_c2r_adjoint", g, gX)
        return gX, None


def fft(x: torch.Tensor, inverse: bool = False) -> torch.Tensor:
    """Unnormalised C2C over the last axis (inverse: exp(+2 pi i kn/N), no 1/N)."""
    return _C2C.apply(x, inverse, 1)


def rfft(x: torch.Tensor) -> torch.Tensor:
    """R2C over the last axis: n real samples -> n//2+1 bins."""
    return _R2C.apply(x, 1)


def irfft(X: torch.Tensor, n: int) -> torch.Tensor:
    """Unnormalised C2R (n * torch.fft.irfft) over the last axis."""
    return _C2R.apply(X, (n,))


def fft2(x: torch.Tensor, inverse: bool = False) -> torch.Tensor:
    """Unnormalised 2D C2C over the last two axes."""
    return _C2C.apply(x, inverse, 2)


def rfft2(x: torch.Tensor) -> torch.Tensor:
    """2D R2C over the last two axes: (nx, ny) real -> (nx, ny//2+1) bins."""
    return _R2C.apply(x, 2)


def irfft2(X: torch.Tensor, s: tuple) -> torch.Tensor:
    """Unnormalised 2D C2R (nx * ny * torch.fft.irfft2) to real shape s = (nx, ny)."""
    return _C2R.apply(X, (int(s[0]), int(s[1])))


def fftn(x: torch.Tensor, inverse: bool = False) -> torch.Tensor:
    """Unnormalised 3D C2C over the last three axes."""
    return _C2C.apply(x, inverse, 3)


def rfftn(x: torch.Tensor) -> torch.Tensor:
    """3D R2C over the last three axes: (nx, ny, nz) real -> (nx, ny, nz//2+1) bins."""
    return _R2C.apply(x, 3)


def irfftn(X: torch.Tensor, s: tuple) -> torch.Tensor:
    """Unnormalised 3D C2R (nx * ny * nz * torch.fft.irfftn) to real shape s = (nx, ny, nz)."""
    return _C2R.apply(X, tuple(int(v) for v in s))
