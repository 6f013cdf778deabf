"""Differentiable N-body steps on the GPU kernels.

`acc(r, m, e2)` is the softened gravitational acceleration of one particle
set (tupan/lib/src/acc_kernel_common.h:7-37 with i-set = j-set) as a
torch.autograd.Function: forward = tg_acc, backward = tg_acc_vjp, the
hand-written vector-Jacobian product (a tidal-tensor contraction, O(N^2) and
tiled like the forward).  Positions are (3, N) float64 CUDA tensors
(structure of arrays), masses and per-particle eps2 are (N,).

`leapfrog` chains kick-drift-kick steps (the SIA21 kdk propagator of
tupan/integrator/sia.py:324-337, with the last kick's acceleration reused
as the next step's first) and recomputes the forward of each block of
`checkpoint_every` steps during the backward pass (torch.utils.checkpoint),
so memory grows with steps / checkpoint_every instead of steps.
"""
import torch
from torch.utils.checkpoint import checkpoint

from . import _native

PREC = {"float64": _native.PREC_FP64, "ds32": _native.PREC_DS32, "float32": _native.PREC_DS32,
        "ds32x": _native.PREC_DS32X}


def _stream():
    return _native.current_stream()


def _check_set(r, m, e2):
    if r.dim() != 2 or r.shape[0] != 3:
        raise ValueError("positions must have shape (3, N)")
    for t in (r, m, e2):
        if not (t.is_cuda and t.dtype == torch.float64):
            raise TypeError("expected float64 CUDA tensors")


def acc_forward(r, m, e2, prec):
    """a (3, N) = acceleration of every particle due to all others."""
    r = r.contiguous()
    n = r.shape[1]
    a = torch.empty_like(r)
    p = [m.data_ptr(), r[0].data_ptr(), r[1].data_ptr(), r[2].data_ptr(), e2.data_ptr()]
    _native.call_device("acc", n, p, n, p, (), [a[0].data_ptr(), a[1].data_ptr(), a[2].data_ptr()],
                        prec, _stream())
    return a


def acc_vjp(r, m, e2, g, prec):
    """(dL/dr, dL/dm) for upstream gradient g = dL/da."""
    r, g = r.contiguous(), g.contiguous()
    n = r.shape[1]
    rb = torch.empty_like(r)
    mb = torch.empty_like(m)
    rc = _native.lib.tg_acc_vjp(n, m.data_ptr(), r[0].data_ptr(), r[1].data_ptr(), r[2].data_ptr(),
                                e2.data_ptr(), g[0].data_ptr(), g[1].data_ptr(), g[2].data_ptr(),
                                rb[0].data_ptr(), rb[1].data_ptr(), rb[2].data_ptr(), mb.data_ptr(),
                                int(prec), _stream())
    _native.check(rc, "tg_acc_vjp")
    return rb, mb


class AccFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, r, m, e2, prec):
        ctx.save_for_backward(r, m, e2)
        ctx.prec = prec
        return acc_forward(r, m, e2, prec)

    @staticmethod
    def backward(ctx, g):
        r, m, e2 = ctx.saved_tensors
        rb, mb = acc_vjp(r, m, e2, g, ctx.prec)
        return rb, (mb if ctx.needs_input_grad[1] else None), None, None


def acc(r, m, e2, prec="ds32"):
    _check_set(r, m, e2)
    return AccFunction.apply(r, m, e2, PREC[prec])


def _kdk_block(r, v, a, m, e2, dt, nsteps, prec):
    for _ in range(nsteps):
        v = v + a * (0.5 * dt)
        r = r + v * dt
        a = acc(r, m, e2, prec)
        v = v + a * (0.5 * dt)
    return r, v, a


def leapfrog(r, v, m, e2, dt, steps, prec="ds32", checkpoint_every=8):
    """Kick-drift-kick leapfrog; returns (r, v) after `steps` steps."""
    a = acc(r, m, e2, prec)
    done = 0
    while done < steps:
        k = min(checkpoint_every, steps - done) if checkpoint_every else steps - done
        if checkpoint_every and torch.is_grad_enabled():
            r, v, a = checkpoint(_kdk_block, r, v, a, m, e2, dt, k, prec, use_reentrant=False)
        else:
            r, v, a = _kdk_block(r, v, a, m, e2, dt, k, prec)
        done += k
    return r, v


def loss_to_target(r, target):
    """Mean over particles of the squared distance to the target positions."""
    return ((r - target) ** 2).sum(0).mean()
