"""Differentiable PO propagation for PyTorch.

`propagate(mode, src7, cur, gmode, ncx, ncy, tgt7, k, ds=None, dt=None, ...)`
returns the mode's output rows (n_out, nt) as a float64 CUDA tensor and is
differentiable with respect to:

  cur  (12, ns)  the source currents (c2Bundle row order, real rows); for
                 the scalar mode the (2, ns) field (re, im)
  ds   (ns,)     displacement of each source point along its normal
  dt   (nt,)     displacement of each target point along its normal (near
                 field and scalar)

Displaced points move along their (frozen) normals with their areas frozen,
the reference's surface-error convention (reference
src/common/InterfaceReflector.cpp:852-866). The forward pass calls
po_run_dev, the backward pass po_adjoint_dev; both queue on the current
stream and recompute the Green's function (nothing of size ns*nt is kept).
Chains (feed -> reflector -> far field) compose through autograd: the output
currents of a JM stage are the `cur` input of the next stage.
"""
import torch

from . import engine


def _displaced(g7, d):
    if d is None:
        return g7
    out = g7.clone()
    out[0:3] += d.unsqueeze(0) * g7[3:6]
    return out


class POFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, cur, ds, dt, mode, src7, gmode, ncx, ncy, tgt7, k, epsilon, t_dir, precision):
        s7 = _displaced(src7, ds).contiguous()
        t7 = _displaced(tgt7, dt).contiguous() if mode != "FF" else tgt7
        cur_c = cur.detach().contiguous()
        m_zero = bool(mode != "scalar" and not torch.any(cur_c[6:] != 0).item())
        out = engine.propagate_dev(mode, s7, cur_c, gmode, ncx, ncy, t7, k, epsilon, t_dir, precision,
                                   m_zero=m_zero)
        ctx.save_for_backward(cur_c, s7, t7)
        ctx.meta = (mode, gmode, ncx, ncy, k, epsilon, t_dir, precision, m_zero,
                    ds is not None, dt is not None)
        return out

    @staticmethod
    def backward(ctx, gout):
        cur, s7, t7 = ctx.saved_tensors
        mode, gmode, ncx, ncy, k, epsilon, t_dir, precision, m_zero, has_ds, has_dt = ctx.meta
        ns, nt = s7.shape[1], t7.shape[1]
        want_cur = ctx.needs_input_grad[0]
        want_ds = has_ds and ctx.needs_input_grad[1]
        want_dt = has_dt and ctx.needs_input_grad[2] and mode != "FF"
        gc = torch.empty(tuple(cur.shape), dtype=torch.float64, device=s7.device) if want_cur else None
        gs = torch.empty(ns, dtype=torch.float64, device=s7.device) if want_ds else None
        gt = torch.empty(nt, dtype=torch.float64, device=s7.device) if want_dt else None
        if want_cur or want_ds or want_dt:
            engine.adjoint_dev(mode, s7, cur, gmode, ncx, ncy, t7, k, gout.contiguous(), epsilon, t_dir,
                               precision, m_zero=m_zero, grad_cur=gc, grad_ds=gs, grad_dt=gt)
        return (gc, gs, gt) + (None,) * 10


def propagate(mode, src7, cur, gmode, ncx, ncy, tgt7, k, ds=None, dt=None, epsilon=1.0, t_dir=-1.0,
              precision="mixed"):
    """Differentiable propagation (see the module docstring)."""
    return POFunction.apply(cur, ds, dt, mode, src7, gmode, ncx, ncy, tgt7, k, epsilon, t_dir, precision)
