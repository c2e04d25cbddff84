"""CIC gather with its VJP, backed by ``pmx_gather``/``pmx_gather_adj``
(pmwd/gather.py:8-144)."""

import torch

from . import _lib
from .scatter import _check_ptcl, _spec, _val_args


class _GatherFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, disp, mesh, val, pmid, conf, offset, cell_size):
        n, dim = pmid.shape
        mesh = mesh.to(torch.float32).contiguous()
        chan_shape = tuple(mesh.shape[dim:])
        chan = 1
        for c in chan_shape:
            chan *= c
        vt, vs = _val_args(val, n, chan_shape, disp.device)
        out = torch.empty((n,) + chan_shape, dtype=torch.float32, device=disp.device)
        spec = _spec(conf, dim, mesh.shape[:dim], offset, cell_size)
        _lib.call('pmx_gather', spec, _lib.ptr(pmid), _lib.ptr(disp), n, _lib.ptr(mesh), chan,
                  _lib.ptr(vt), vs, _lib.ptr(out), _lib.stream_ptr(disp.device))
        ctx.save_for_backward(pmid, disp, mesh)
        ctx.meta = (conf, offset, cell_size, chan, dim, torch.is_tensor(val) and val.ndim == 0,
                    torch.is_tensor(val) and val.ndim > 0)
        return out

    @staticmethod
    def backward(ctx, val_cot):
        pmid, disp, mesh = ctx.saved_tensors
        conf, offset, cell_size, chan, dim, val0d, valnd = ctx.meta
        n = pmid.shape[0]
        val_cot = val_cot.to(torch.float32).contiguous()
        disp_cot = torch.empty_like(disp)
        mesh_cot = torch.zeros_like(mesh)
        spec = _spec(conf, dim, mesh.shape[:dim], offset, cell_size)
        _lib.call('pmx_gather_adj', spec, _lib.ptr(pmid), _lib.ptr(disp), n, _lib.ptr(mesh), chan,
                  _lib.ptr(val_cot), _lib.ptr(disp_cot), _lib.ptr(mesh_cot),
                  _lib.stream_ptr(disp.device))
        vc = None
        if ctx.needs_input_grad[2]:
            vc = val_cot.sum() if val0d else val_cot
        return disp_cot, mesh_cot, vc, None, None, None, None


def gather(ptcl, conf, mesh, val=0, offset=0, cell_size=None):
    """Gather particle values from a mesh multilinearly (gather.py:8-30).
    Differentiable in ``ptcl.disp``, ``mesh`` and ``val``."""
    pmid, disp = ptcl.pmid, ptcl.disp
    _check_ptcl(pmid, disp)
    if not torch.is_tensor(mesh):
        mesh = torch.as_tensor(mesh, dtype=torch.float32, device=disp.device)
    return _GatherFn.apply(disp.contiguous(), mesh, val, pmid.contiguous(), conf, offset,
                           cell_size)
