"""The large single simulation (512^3 particles on a 1024^3 mesh, box 1024
Mpc/h, 2LPT at a = 1/64, 100-step time grid) at full size, through properties
that need no oracle run at this size:

* mass conservation: the CIC density of the 2LPT state sums to the number of
  mesh cells (mean 1);
* reversibility: 4 forward steps of the multi-step path, then the 4 reverse
  steps of the adjoint, bring the particles back to their initial
  displacements and velocities within the float32 bound measured at small
  sizes (the reverse steps rebuild the trajectory instead of storing it);
* the forward state of the multi-step path equals 4 single steps up to the
  order of the float32 atomic adds.
"""

import ctypes
import importlib

import numpy as np
import pytest
import torch

import pmwd_gb300 as pg
from pmwd_gb300 import _lib

gnb = importlib.import_module('pmwd_gb300.nbody')

pytestmark = pytest.mark.gpu

COSMO = dict(A_s_1e9=2.1, n_s=0.965, Omega_m=0.3, Omega_b=0.05, h=0.7)
K = 4


def rel(a, b):
    return float((a.double() - b.double()).norm() / b.double().norm())


def test_c4_mass_and_reversibility(cuda):
    conf = pg.Configuration(2.0, (512,) * 3, 2, a_nbody_maxstep=(1 - 1 / 64) / 100)
    assert conf.mesh_shape == (1024,) * 3
    cosmo = pg.boltzmann(pg.Cosmology(conf, **COSMO), conf)
    with torch.no_grad():
        ptcl, _ = pg.lpt(pg.linear_modes(pg.white_noise(0, conf, device=cuda), cosmo, conf),
                         cosmo, conf)
    pmid = ptcl.pmid.contiguous()
    disp0 = ptcl.disp.detach().contiguous()
    vel0 = ptcl.vel.detach().contiguous()
    del ptcl
    N, M = conf.ptcl_num, conf.mesh_size
    spec = _lib.make_spec(3, conf.mesh_shape, conf.mesh_shape, conf.cell_size)
    st = _lib.stream_ptr(cuda)

    # mass conservation of one CIC deposit (float32 atomics, float64 sum)
    dens = torch.zeros(conf.mesh_shape, dtype=torch.float32, device=cuda)
    _lib.call('pmx_scatter', spec, pmid, disp0, N, None, float(M / N), 1, dens, st)
    total = float(dens.double().sum())
    del dens
    assert abs(total / M - 1) < 1e-5, total / M

    fwd = gnb.op_factors(gnb.forward_ops(conf), cosmo, conf).detach()
    adj = gnb.op_factors(gnb.adjoint_ops(conf), cosmo, conf).detach()
    f_fwd = np.ascontiguousarray(fwd.to(torch.float32).numpy().reshape(-1, 3)[:K])
    f_adj = np.ascontiguousarray(adj.to(torch.float32).numpy().reshape(-1, 3)[-K:])
    Om = float(cosmo.Omega_m)
    ws = _lib.Workspace(conf.mesh_shape, adjoint=True)
    disp, vel = disp0.clone(), vel0.clone()
    acc = torch.empty_like(disp)
    _lib.call('pmx_force', ws.handle, spec, pmid, disp, N, N, Om, acc, st)
    d1, v1, a1 = disp.clone(), vel.clone(), acc.clone()
    for i in range(K):
        _lib.call('pmx_nbody_step', ws.handle, spec, pmid, d1, v1, a1, N, N,
                  (_lib.c_f * 3)(*f_fwd[i]), Om, st)
    _lib.call('pmx_nbody_steps', ws.handle, spec, pmid, disp, vel, acc, N, N, K,
              f_fwd.ctypes.data_as(ctypes.c_void_p), Om, st)
    assert rel(disp, d1) < 1e-5 and rel(vel, v1) < 1e-5 and rel(acc, a1) < 1e-5
    del d1, v1, a1
    moved = rel(disp, disp0)
    disp_cot = torch.zeros_like(disp)
    vel_cot = torch.zeros_like(disp)
    alpha = torch.zeros_like(disp)
    dots = torch.zeros((K, 4), dtype=torch.float64, device=cuda)
    _lib.call('pmx_nbody_adj_steps', ws.handle, spec, pmid, disp, vel, acc, disp_cot, vel_cot,
              alpha, N, N, K, f_adj.ctypes.data_as(ctypes.c_void_p), Om, dots, st)
    back_d, back_v = rel(disp, disp0), rel(vel, vel0)
    print(f'C4: mass {total / M - 1:.1e}; {K} steps moved disp by {moved:.2e} (rel), '
          f'reverse error disp {back_d:.2e}, vel {back_v:.2e}')
    assert moved > 1e-3
    assert back_d < 1e-4 and back_v < 1e-3


def test_c4_force_fused_matches_cufft3d(cuda):
    """One force and one force VJP at full size (512^3 particles displaced
    around the lattice, 1024^3 mesh): the fused x-pass path (the 1024-point
    six-step transform between slab-wise 2-D cuFFT planes, which the run
    above and the benchmark use) against the same calls on a workspace of
    3-D cuFFT plans and the one-pass Fourier kernels."""
    conf = pg.Configuration(2.0, (512,) * 3, 2)
    grid = pg.Particles.gen_grid(conf, device=cuda)
    gen = torch.Generator(device=cuda).manual_seed(3)
    pmid = grid.pmid
    disp = (grid.disp + 1.5 * torch.randn(grid.disp.shape, generator=gen, device=cuda)).contiguous()
    cot = torch.randn(disp.shape, generator=gen, device=cuda)
    del grid
    N = conf.ptcl_num
    spec = _lib.make_spec(3, conf.mesh_shape, conf.mesh_shape, conf.cell_size)
    st = _lib.stream_ptr(cuda)
    res = []
    for cufft3d in (False, True):
        ws = _lib.Workspace(conf.mesh_shape, adjoint=True, cufft3d=cufft3d)
        acc = torch.empty_like(disp)
        _lib.call('pmx_force', ws.handle, spec, pmid, disp, N, N, 0.3, acc, st)
        acc_v, dc = torch.empty_like(disp), torch.empty_like(disp)
        om = torch.zeros((), dtype=torch.float64, device=cuda)
        _lib.call('pmx_force_vjp', ws.handle, spec, pmid, disp, N, N, 0.3, cot, acc_v, dc, om, st)
        torch.cuda.synchronize()
        res.append((acc, acc_v, dc, float(om)))
        del ws
    (a_f, av_f, dc_f, om_f), (a_3, av_3, dc_3, om_3) = res
    e_acc, e_dc, e_om = rel(a_f, a_3), rel(dc_f, dc_3), abs(om_f / om_3 - 1)
    print(f'C4 force fused vs 3-D cuFFT: acc {e_acc:.2e}, disp cot {e_dc:.2e}, Omega_m term '
          f'{e_om:.2e}')
    assert e_acc < 1e-5
    assert rel(av_f, a_3) < 1e-5 and rel(av_3, a_3) < 1e-5
    assert e_dc < 1e-4
    assert e_om < 1e-4
