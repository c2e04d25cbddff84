"""CIC scatter with its VJP, backed by ``pmx_scatter``/``pmx_scatter_adj``
(pmwd/scatter.py:8-150)."""

import torch

from . import _lib


def _check_ptcl(pmid, disp):
    if not (pmid.is_cuda and disp.is_cuda):
        raise ValueError('particles must be CUDA tensors (the mesh operators run on the GPU)')
    if pmid.dtype != torch.int16 or disp.dtype != torch.float32:
        raise ValueError('pmid must be int16 and disp float32')


def _val_args(val, n, chan_shape, device):
    """(tensor-or-None, scalar) for the C ABI; val is None, a number, a 0-d
    tensor or an (n, *chan) tensor."""
    if torch.is_tensor(val) and val.ndim > 0:
        if tuple(val.shape[1:]) != tuple(chan_shape) or val.shape[0] != n:
            raise ValueError(f'channel shape mismatch: {tuple(chan_shape)} != {tuple(val.shape[1:])}')
        return val.to(device=device, dtype=torch.float32).contiguous(), 0.0
    if chan_shape != ():
        raise ValueError(f'channel shape mismatch: {tuple(chan_shape)} != ()')
    return None, float(torch.as_tensor(val, dtype=torch.float32))


def _spec(conf, dim, mesh_spatial, offset, cell_size):
    return _lib.make_spec(dim, conf.mesh_shape, mesh_spatial, conf.cell_size, offset, cell_size)


class _ScatterFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, disp, mesh, val, pmid, conf, offset, cell_size, val_is_default):
        n, dim = pmid.shape
        chan_shape = tuple(mesh.shape[dim:])
        chan = 1
        for c in chan_shape:
            chan *= c
        vt, vs = _val_args(val, n, chan_shape, disp.device)
        out = mesh.to(torch.float32).contiguous().clone()
        spec = _spec(conf, dim, mesh.shape[:dim], offset, cell_size)
        _lib.call('pmx_scatter', spec, _lib.ptr(pmid), _lib.ptr(disp), n, _lib.ptr(vt), vs, chan,
                  _lib.ptr(out), _lib.stream_ptr(disp.device))
        ctx.save_for_backward(pmid, disp, vt)
        ctx.meta = (conf, offset, cell_size, vs, chan, chan_shape, dim,
                    torch.is_tensor(val) and val.ndim == 0)
        return out

    @staticmethod
    def backward(ctx, mesh_cot):
        pmid, disp, vt = ctx.saved_tensors
        conf, offset, cell_size, vs, chan, chan_shape, dim, val0d = ctx.meta
        n = pmid.shape[0]
        mesh_cot = mesh_cot.to(torch.float32).contiguous()
        disp_cot = torch.empty_like(disp)
        need_val = ctx.needs_input_grad[2]
        val_cot = torch.empty((n, chan), dtype=torch.float32, device=disp.device) if need_val else None
        spec = _spec(conf, dim, mesh_cot.shape[:dim], offset, cell_size)
        _lib.call('pmx_scatter_adj', spec, _lib.ptr(pmid), _lib.ptr(disp), n, _lib.ptr(vt), vs,
                  chan, _lib.ptr(mesh_cot), _lib.ptr(disp_cot), _lib.ptr(val_cot),
                  _lib.stream_ptr(disp.device))
        if need_val:
            val_cot = val_cot.sum() if val0d else val_cot.reshape((n,) + chan_shape)
        return disp_cot, mesh_cot, val_cot, None, None, None, None, None


def scatter(ptcl, conf, mesh=None, val=None, offset=0, cell_size=None):
    """Scatter particle values to a mesh multilinearly (scatter.py:8-30).

    ``mesh`` defaults to zeros of ``conf.mesh_shape + val.shape[1:]`` and
    ``val`` to ``conf.mesh_size / conf.ptcl_num``.  Differentiable in
    ``ptcl.disp``, ``mesh`` and ``val``.
    """
    pmid, disp = ptcl.pmid, ptcl.disp
    _check_ptcl(pmid, disp)
    default = val is None
    if default:
        val = conf.mesh_size / conf.ptcl_num
    if mesh is None:
        vshape = tuple(val.shape[1:]) if torch.is_tensor(val) and val.ndim > 0 else ()
        mesh = torch.zeros(tuple(conf.mesh_shape) + vshape, dtype=torch.float32,
                           device=disp.device)
    return _ScatterFn.apply(disp.contiguous(), mesh, val, pmid.contiguous(), conf, offset,
                            cell_size, default)
