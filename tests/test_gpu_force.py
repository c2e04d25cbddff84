"""GPU parity of the Poisson force, the leapfrog and the reversible adjoint
against the CPU oracle, through the C ABI and the pmwd-style API."""

import numpy as np
import pytest
import torch

from oracle import cosmo as oc, ics, nbody as onb, pm
import pmwd_gb300 as pg
from pmwd_gb300 import _lib
import importlib
gnb = importlib.import_module("pmwd_gb300.nbody")

pytestmark = pytest.mark.gpu

RTOL_ACC = 1e-5       # single force step, relative L2 (float32 FFT rounding)


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def T(x, dev):
    return torch.from_numpy(np.ascontiguousarray(x)).to(dev)


def make(ptcl, mesh, spacing, std, seed=0, a_step=1 / 8):
    oconf = oc.OConf(spacing, ptcl, mesh, float_dtype=np.float32, a_nbody_maxstep=a_step)
    gconf = pg.Configuration(spacing, ptcl, mesh, a_nbody_maxstep=a_step)
    pmid, disp = ics.gen_grid(oconf)
    rng = np.random.default_rng(seed)
    disp = (disp + rng.normal(0, std, disp.shape)).astype(np.float32)
    vel = rng.normal(0, 0.1, disp.shape).astype(np.float32)
    return oconf, gconf, pmid, disp, vel


@pytest.mark.parametrize('ptcl, mesh, spacing', [((16, 16, 16), 2, 1.0), ((12, 20, 8), 1, 2.0),
                                                  ((32, 32, 32), 1, 4.0)])
def test_force_matches_oracle(cuda, ptcl, mesh, spacing):
    oconf, gconf, pmid, disp, vel = make(ptcl, mesh, spacing, 1.5 * spacing)
    acc_o = pm.gravity(pmid, disp, 0.3, oconf)
    ws = _lib.workspace(gconf.mesh_shape)
    spec = _lib.make_spec(3, gconf.mesh_shape, gconf.mesh_shape, gconf.cell_size)
    acc = torch.empty((len(pmid), 3), dtype=torch.float32, device=cuda)
    _lib.call('pmx_force', ws.handle, spec, T(pmid, cuda), T(disp, cuda),
              len(pmid), gconf.ptcl_num, 0.3, _lib.ptr(acc), _lib.stream_ptr(cuda))
    assert rel_l2(acc.cpu().numpy(), acc_o) < RTOL_ACC


XPASS_CASES = [((32, 32, 32), 2, 1.0), ((32, 16, 24), 4, 2.0), ((64, 64, 64), 1, 2.0),
               ((128, 64, 32), 1, 1.0), ((128, 128, 128), 2, 2.0)]
# x passes of 512 and 1024 points (the Split<512> and Split<1024> six-step
# transforms the 512^3-particle / 1024^3-mesh run uses) on cheap anisotropic
# meshes: (512, 32, 32), (1024, 32, 32), (1024, 64, 64)
XPASS_LONG = [((128, 8, 8), 4, 1.0), ((256, 8, 8), 4, 1.0), ((256, 16, 16), 4, 1.0)]


def _force_both_paths(cuda, gconf, pmid, disp, cot=None,
                      variants=({}, {'cufft3d': True})):
    """pmx_force / pmx_force_vjp on workspaces built with each set of
    keyword flags in `variants` (default: the fused x-pass path and the 3-D
    cuFFT path)."""
    out = []
    for kw in variants:
        ws = _lib.Workspace(gconf.mesh_shape, adjoint=True, **kw)
        spec = _lib.make_spec(3, gconf.mesh_shape, gconf.mesh_shape, gconf.cell_size)
        n = len(pmid)
        P, D = T(pmid, cuda), T(disp, cuda)
        acc = torch.empty((n, 3), dtype=torch.float32, device=cuda)
        if cot is None:
            _lib.call('pmx_force', ws.handle, spec, P, D, n, gconf.ptcl_num, 0.3, acc,
                      _lib.stream_ptr(cuda))
            out.append(acc.cpu().numpy())
        else:
            dc = torch.empty((n, 3), dtype=torch.float32, device=cuda)
            om = torch.zeros((), dtype=torch.float64, device=cuda)
            _lib.call('pmx_force_vjp', ws.handle, spec, P, D, n, gconf.ptcl_num, 0.3,
                      T(cot, cuda), acc, dc, om, _lib.stream_ptr(cuda))
            out.append((acc.cpu().numpy(), dc.cpu().numpy(), float(om)))
        del ws
    return out


@pytest.mark.parametrize('ptcl, mesh, spacing', XPASS_CASES + XPASS_LONG)
def test_fused_xpass_force_matches_oracle(cuda, ptcl, mesh, spacing):
    """Power-of-two n0 (64..1024; the cases here reach 64, 128, 256, 512 and
    1024) takes the fused x-pass path (slab-wise 2-D cuFFT planes); it must
    match the oracle and the 3-D cuFFT path."""
    oconf, gconf, pmid, disp, vel = make(ptcl, mesh, spacing, 1.5 * spacing)
    acc_o = pm.gravity(pmid, disp, 0.3, oconf)
    fast, ref3d = _force_both_paths(cuda, gconf, pmid, disp)
    assert rel_l2(fast, acc_o) < RTOL_ACC
    assert rel_l2(ref3d, acc_o) < RTOL_ACC
    assert rel_l2(fast, ref3d) < RTOL_ACC


@pytest.mark.parametrize('ptcl, mesh, spacing', XPASS_CASES[:3] + XPASS_LONG)
def test_fused_xpass_force_vjp_matches_oracle(cuda, ptcl, mesh, spacing):
    oconf, gconf, pmid, disp, vel = make(ptcl, mesh, spacing, 1.5 * spacing)
    cot = np.random.default_rng(12).normal(size=disp.shape).astype(np.float32)
    oconf64 = oc.OConf(spacing, ptcl, mesh, float_dtype=np.float64)
    acc_o, dc_o, om_o = pm.gravity_vjp(pmid, disp.astype(np.float64), 0.3, oconf64,
                                       cot.astype(np.float64))
    (a_f, dc_f, om_f), (a_3, dc_3, om_3) = _force_both_paths(cuda, gconf, pmid, disp, cot)
    for a, dc, om in ((a_f, dc_f, om_f), (a_3, dc_3, om_3)):
        assert rel_l2(a, acc_o) < RTOL_ACC
        assert rel_l2(dc, dc_o) < 1e-4
        assert abs(om / om_o - 1) < 1e-4


PLANE_CASES = [((16, 64, 64), 4, 1.0), ((16, 128, 128), 4, 1.0), ((16, 256, 256), 4, 1.0)]


@pytest.mark.parametrize('ptcl, mesh, spacing', PLANE_CASES)
def test_plane_transforms_match_cufft_and_oracle(cuda, ptcl, mesh, spacing):
    """Square power-of-two (y, z) planes of 256^2, 512^2 and 1024^2 through
    the cluster plane kernels and through slab-wise 2-D cuFFT: force and
    force VJP must match each other, the 3-D cuFFT path and the oracle."""
    oconf, gconf, pmid, disp, vel = make(ptcl, mesh, spacing, 1.5 * spacing)
    variants = ({'plane': True}, {}, {'cufft3d': True})
    acc_o = pm.gravity(pmid, disp, 0.3, oconf)
    accs = _force_both_paths(cuda, gconf, pmid, disp, variants=variants)
    for a in accs:
        assert rel_l2(a, acc_o) < RTOL_ACC
    assert rel_l2(accs[0], accs[1]) < RTOL_ACC
    cot = np.random.default_rng(5).normal(size=disp.shape).astype(np.float32)
    res = _force_both_paths(cuda, gconf, pmid, disp, cot, variants=variants)
    for a, dc, om in res[1:]:
        assert rel_l2(res[0][0], a) < RTOL_ACC
        assert rel_l2(res[0][1], dc) < 1e-4
        assert abs(res[0][2] / om - 1) < 1e-4


@pytest.mark.parametrize('ptcl, mesh', [((16, 16, 16), 2), ((10, 12, 14), 1)])
def test_force_vjp_matches_oracle(cuda, ptcl, mesh):
    oconf, gconf, pmid, disp, vel = make(ptcl, mesh, 2.0, 2.0)
    cot = np.random.default_rng(9).normal(size=disp.shape).astype(np.float32)
    oconf64 = oc.OConf(2.0, ptcl, mesh, float_dtype=np.float64)
    acc_o, dc_o, om_o = pm.gravity_vjp(pmid, disp.astype(np.float64), 0.3, oconf64,
                                       cot.astype(np.float64))
    ws = _lib.workspace(gconf.mesh_shape)
    spec = _lib.make_spec(3, gconf.mesh_shape, gconf.mesh_shape, gconf.cell_size)
    n = len(pmid)
    acc = torch.empty((n, 3), dtype=torch.float32, device=cuda)
    dc = torch.empty((n, 3), dtype=torch.float32, device=cuda)
    om = torch.zeros((), dtype=torch.float64, device=cuda)
    _lib.call('pmx_force_vjp', ws.handle, spec, T(pmid, cuda), T(disp, cuda),
              n, gconf.ptcl_num, 0.3, T(cot, cuda), _lib.ptr(acc), _lib.ptr(dc),
              _lib.ptr(om), _lib.stream_ptr(cuda))
    assert rel_l2(acc.cpu().numpy(), acc_o) < RTOL_ACC
    assert rel_l2(dc.cpu().numpy(), dc_o) < 1e-4
    assert abs(float(om) / om_o - 1) < 1e-4


def test_gravity_autograd_api(cuda):
    """gravity() through torch autograd equals the explicit VJP."""
    oconf, gconf, pmid, disp, vel = make((16, 16, 16), 2, 1.0, 1.0)
    cosmo = pg.SimpleLCDM(gconf)
    Om = cosmo.Omega_m.clone().requires_grad_(True)
    cosmo = cosmo.replace(Omega_m=Om)
    D = T(disp, cuda).requires_grad_(True)
    ptcl = pg.Particles(gconf, T(pmid, cuda), D)
    acc = pg.gravity(0.5, ptcl, cosmo, gconf)
    cot = torch.randn_like(acc)
    (acc * cot).sum().backward()
    oconf64 = oc.OConf(1.0, (16, 16, 16), 2, float_dtype=np.float64)
    _, dc_o, om_o = pm.gravity_vjp(pmid, disp.astype(np.float64), 0.3, oconf64,
                                   cot.cpu().numpy().astype(np.float64))
    assert rel_l2(D.grad.cpu().numpy(), dc_o) < 1e-4
    assert abs(float(Om.grad) / om_o - 1) < 1e-4


def _run_gpu_nbody(gconf, pmid, disp, vel, cosmo, dev):
    ptcl = pg.Particles(gconf, T(pmid, dev), T(disp, dev), vel=T(vel, dev))
    out, _ = pg.nbody(ptcl, None, cosmo, gconf)
    return out


@pytest.fixture(scope='module', params=[(16, 2), (32, 2)], ids=['32mesh', '64mesh_xpass'])
def nb_case(request):
    side, ratio = request.param
    oconf, gconf, pmid, disp, vel = make((side,) * 3, ratio, 4.0, 0.5, a_step=1 / 8)
    ocos = oc.with_tables(oc.simple_lcdm(), oconf)
    gcos = pg.boltzmann(pg.SimpleLCDM(gconf), gconf)
    return oconf, gconf, pmid, disp, vel, ocos, gcos


def test_nbody_forward_matches_oracle(cuda, nb_case):
    oconf, gconf, pmid, disp, vel, ocos, gcos = nb_case
    st = onb.nbody(onb.State(pmid, disp, vel), ocos, oconf)
    out = _run_gpu_nbody(gconf, pmid, disp, vel, gcos, cuda)
    # position RMS within 1e-3 of the particle spacing (the stated full-run bar)
    rms = np.sqrt(np.mean((out.disp.cpu().numpy().astype(np.float64) - st.disp) ** 2))
    assert rms < 1e-3 * oconf.ptcl_spacing
    assert rel_l2(out.disp.cpu().numpy(), st.disp) < 1e-4
    assert rel_l2(out.vel.cpu().numpy(), st.vel) < 1e-4
    assert rel_l2(out.acc.cpu().numpy(), st.acc) < 1e-4


def test_fused_step_equals_generic_ops(cuda, nb_case):
    """The fused step kernels reproduce the reference op sequence run op by
    op (bit-identical float32 arithmetic except for atomic order)."""
    oconf, gconf, pmid, disp, vel, ocos, gcos = nb_case
    fused = _run_gpu_nbody(gconf, pmid, disp, vel, gcos, cuda)
    gconf2 = gconf.replace(symp_splits=((0.0, 0.5), (1.0, 0.5), (0.0, 0.0)))
    assert not gnb._is_fused(gconf2)
    generic = _run_gpu_nbody(gconf2, pmid, disp, vel, pg.boltzmann(pg.SimpleLCDM(gconf2), gconf2),
                             cuda)
    # only the order of the float32 atomic adds differs (8 steps amplify it
    # to ~1e-6)
    assert rel_l2(generic.disp.cpu().numpy(), fused.disp.cpu().numpy()) < 1e-5
    assert rel_l2(generic.vel.cpu().numpy(), fused.vel.cpu().numpy()) < 1e-5


def test_multistep_equals_single_steps(cuda, nb_case):
    """pmx_nbody_steps / pmx_nbody_adj_steps (consecutive steps joined in one
    particle pass) against the same steps called one by one: the float32
    updates are the same, only the order of the atomic adds differs.  The
    forward state agrees to 1e-5 after 8 steps; the adjoint's outputs
    amplify the atomic-order noise, so they are held to 10x the difference
    between two runs of the one-by-one path (at least 1e-3)."""
    import ctypes
    oconf, gconf, pmid, disp, vel, ocos, gcos = nb_case
    fwd = gnb.op_factors(gnb.forward_ops(gconf), gcos, gconf).detach()
    adj = gnb.op_factors(gnb.adjoint_ops(gconf), gcos, gconf).detach()
    f_fwd = np.ascontiguousarray(fwd.to(torch.float32).numpy().reshape(-1, 3))
    f_adj = np.ascontiguousarray(adj.to(torch.float32).numpy().reshape(-1, 3))
    nst = f_fwd.shape[0]
    n = len(pmid)
    spec = _lib.make_spec(3, gconf.mesh_shape, gconf.mesh_shape, gconf.cell_size)
    st = _lib.stream_ptr(cuda)
    Om = float(gcos.Omega_m)
    out = []
    for multi in (False, False, True):
        ws = _lib.Workspace(gconf.mesh_shape, adjoint=True)
        P_, D, V = T(pmid, cuda), T(disp, cuda), T(vel, cuda)
        A = torch.empty_like(D)
        rng = np.random.default_rng(2)
        dc, vc = T(rng.normal(size=disp.shape).astype(np.float32), cuda), torch.zeros_like(D)
        al = torch.zeros_like(D)
        dots = torch.zeros((nst, 4), dtype=torch.float64, device=cuda)
        _lib.call('pmx_force', ws.handle, spec, P_, D, n, gconf.ptcl_num, Om, A, st)
        if multi:
            _lib.call('pmx_nbody_steps', ws.handle, spec, P_, D, V, A, n, gconf.ptcl_num, nst,
                      f_fwd.ctypes.data_as(ctypes.c_void_p), Om, st)
            fwd_state = [t.cpu().numpy() for t in (D, V, A)]
            _lib.call('pmx_nbody_adj_steps', ws.handle, spec, P_, D, V, A, dc, vc, al, n,
                      gconf.ptcl_num, nst, f_adj.ctypes.data_as(ctypes.c_void_p), Om, dots, st)
        else:
            for i in range(nst):
                _lib.call('pmx_nbody_step', ws.handle, spec, P_, D, V, A, n, gconf.ptcl_num,
                          (_lib.c_f * 3)(*f_fwd[i]), Om, st)
            fwd_state = [t.cpu().numpy() for t in (D, V, A)]
            for i in range(nst):
                _lib.call('pmx_nbody_adj_step', ws.handle, spec, P_, D, V, A, dc, vc, al, n,
                          gconf.ptcl_num, (_lib.c_f * 3)(*f_adj[i]), Om, dots[i], st)
        out.append((fwd_state, [t.cpu().numpy() for t in (D, V, A, dc, vc, dots)]))
        del ws
    for a, b in zip(out[0][0], out[2][0]):
        assert rel_l2(b, a) < 1e-5
    names = ('disp', 'vel', 'acc', 'disp_cot', 'vel_cot', 'dots')
    cot_full = 0.0
    for name, a, a2, b in zip(names, out[0][1], out[1][1], out[2][1]):
        floor = rel_l2(a2, a)
        full = rel_l2(b, a)
        if name == 'dots':
            # the dots are sums over the cotangents: a particle whose
            # cotangent jumped at a cell boundary (below) moves them too
            assert full < max(1e-3, 10 * floor, 2 * cot_full), (name, full, floor, cot_full)
        elif name.endswith('_cot'):
            cot_full = max(cot_full, full)
            # The CIC weight gradient is piecewise constant: a rounding-level
            # difference in a reconstructed position can move a particle
            # across a cell boundary and change its cotangent by O(1) (about
            # one such particle per run at this size).  Those particles are
            # dropped (at most 0.2%); the rest are held to the noise bound,
            # and the whole array to a bound that only a real bug exceeds.
            e = np.linalg.norm((b - a).reshape(len(a), -1), axis=1)
            keep = np.argsort(e)[:len(e) - len(e) // 500]
            rest = rel_l2(b[keep], a[keep])
            assert rest < max(1e-3, 10 * floor), (name, rest, full, floor)
            assert full < 3e-2, (name, rest, full, floor)
        else:
            assert full < max(1e-3, 10 * floor), (name, full, floor)


def test_factors_match_oracle(nb_case):
    oconf, gconf, pmid, disp, vel, ocos, gcos = nb_case
    ops = gnb.forward_ops(gconf)
    f = gnb.op_factors(ops, gcos, gconf).detach().numpy()
    ref = []
    for o in ops:
        if o[0] == 'kick':
            ref.append(oc.kick_factor(*o[1:], ocos, oconf))
        elif o[0] == 'drift':
            ref.append(oc.drift_factor(*o[1:], ocos, oconf))
    np.testing.assert_allclose(f, ref, rtol=1e-8)
    adj = gnb.op_factors(gnb.adjoint_ops(gconf), gcos, gconf).detach().numpy().reshape(-1, 3)
    fwd = f.reshape(-1, 3)[::-1]
    np.testing.assert_array_equal(adj[:, 0], -fwd[:, 2])
    np.testing.assert_array_equal(adj[:, 1], -fwd[:, 1])
    np.testing.assert_array_equal(adj[:, 2], -fwd[:, 0])


def robust_rel(b, a, frac=1 / 500):
    """rel_l2 over particles after dropping the worst fraction of them."""
    e = np.linalg.norm((np.asarray(b, np.float64) - a).reshape(len(a), -1), axis=1)
    keep = np.argsort(e)[:len(e) - int(len(e) * frac)]
    return rel_l2(np.asarray(b)[keep], np.asarray(a)[keep])


def test_nbody_adjoint_matches_oracle(cuda, nb_case):
    """Reversible adjoint: cotangents at the start, per-factor
    sensitivities and the Omega_m force term against the oracle's
    nbody_adj (which itself matches float64 autograd).

    The CIC weight gradient is piecewise constant, so a particle that float32
    rounding puts on the other side of a cell boundary than the float64
    oracle gets an O(1) different cotangent, which the remaining adjoint
    steps spread to its neighbours.  Repeated runs of the 64^3-mesh case
    show discrete outcomes: no such event (sensitivities within 1e-5..6e-5
    of the oracle), or one of two events (cotangents 3.2e-4 / 1.3e-3,
    sensitivities 5e-4 / 2e-3).  The cotangents are therefore compared
    without the 0.2% of particles farthest off, and the particle sums
    (sensitivities, Omega_m term) within 5e-3, which an error in the
    adjoint itself exceeds by orders of magnitude."""
    oconf, gconf, pmid, disp, vel, ocos, gcos = nb_case
    rng = np.random.default_rng(11)
    dcot = rng.normal(size=disp.shape).astype(np.float32)
    vcot = rng.normal(size=disp.shape).astype(np.float32)
    oconf64 = oc.OConf(oconf.ptcl_spacing, oconf.ptcl_grid_shape, oconf.mesh_shape,
                       float_dtype=np.float64, a_nbody_maxstep=oconf.a_nbody_maxstep)
    ocos64 = oc.with_tables(oc.simple_lcdm(), oconf64)
    st1 = onb.nbody(onb.State(pmid, disp.astype(np.float64), vel.astype(np.float64)), ocos64,
                    oconf64)
    st0, cot0, sens = onb.nbody_adj(st1, onb.Cot(dcot.astype(np.float64), vcot.astype(np.float64)),
                                    ocos64, oconf64)

    D = T(disp, cuda).requires_grad_(True)
    V = T(vel, cuda).requires_grad_(True)
    Om = gcos.Omega_m.clone().requires_grad_(True)
    cos = gcos.replace(Omega_m=Om)
    ptcl = pg.Particles(gconf, T(pmid, cuda), D, vel=V)
    out, _ = pg.nbody(ptcl, None, cos, gconf)
    ((out.disp * T(dcot, cuda)).sum() + (out.vel * T(vcot, cuda)).sum()).backward()
    for got, want in ((D.grad, cot0.disp), (V.grad, cot0.vel)):
        got = got.cpu().numpy()
        assert robust_rel(got, want) < 1e-3, (robust_rel(got, want), rel_l2(got, want))
        assert rel_l2(got, want) < 1e-2

    # explicit adjoint API: per-factor sensitivities and the Omega_m term
    ptcl1 = out.replace(disp=out.disp.detach(), vel=out.vel.detach(), acc=out.acc.detach())
    cot = pg.Particles(gconf, ptcl1.pmid, T(dcot, cuda), vel=T(vcot, cuda))
    p0, c0, fgrad, omg = gnb.nbody_adj(ptcl1, cot, None, gcos, gconf)
    ref = np.array([s for *_, s in sens['factors']])
    assert rel_l2(fgrad.numpy(), ref) < 5e-3
    assert abs(float(omg) / sens['Omega_m'] - 1) < 5e-3
    # the reconstructed initial state returns to the start
    assert rel_l2(p0.disp.cpu().numpy(), disp) < 1e-4


def test_reversibility_plain_and_kahan(cuda):
    """Forward to a=1 then reverse=True back to a_start returns to the 2LPT
    state (docs/examples/adjoint.ipynb, 'Reversibility'); the compensated
    (Kahan) updates keep the float32 rounding of the disp/vel sums from
    accumulating.  Stated bound: relative RMS error of disp and vel <= 3e-3
    for 32^3 particles, 64^3 mesh, 32 steps.  The error is float32 rounding
    amplified over 64 steps, so it moves with the order of the atomic adds
    (a different particle-kernel grid gave plain vel 2.04e-3 instead of
    2.0e-3; disp 5e-4)."""
    conf = pg.Configuration(4.0, (32, 32, 32), 2, a_nbody_maxstep=(1 - 1 / 64) / 32)
    cosmo = pg.boltzmann(pg.SimpleLCDM(conf), conf)
    with torch.no_grad():
        modes = pg.linear_modes(pg.white_noise(0, conf, device=cuda), cosmo, conf)
        p0, _ = pg.lpt(modes, cosmo, conf)
    errs = {}
    for kahan in (False, True):
        c = conf.replace(kahan=kahan)
        with torch.no_grad():
            p1, _ = pg.nbody(p0, None, cosmo, c)
            p2, _ = pg.nbody(p1, None, cosmo, c, reverse=True)
        ed = float((p2.disp - p0.disp).double().std() / p0.disp.double().std())
        ev = float((p2.vel - p0.vel).double().std() / p0.vel.double().std())
        errs[kahan] = (ed, ev)
    print('reversibility (disp, vel) plain', errs[False], 'kahan', errs[True])
    for ed, ev in errs.values():
        assert ed < 3e-3 and ev < 3e-3
    assert errs[True][0] <= 1.5 * errs[False][0] + 1e-7


@pytest.mark.parametrize('shuffle', [False, True], ids=['lagrangian', 'shuffled'])
def test_window_deposit_equals_direct_atomics(cuda, shuffle):
    """Warp-window deposits (shared-memory accumulation flushed with 16-byte
    vector reductions) give the same force and VJP as one global atomic per
    contribution; a shuffled particle order sends most contributions through
    the window's fallback path."""
    oconf, gconf, pmid, disp, vel = make((32, 32, 32), 2, 1.0, 2.0)
    if shuffle:
        perm = np.random.default_rng(5).permutation(len(pmid))
        pmid, disp = pmid[perm], disp[perm]
    cot = np.random.default_rng(6).normal(size=disp.shape).astype(np.float32)
    acc_o = pm.gravity(pmid, disp, 0.3, oconf)
    out = []
    for window in (True, False):
        ws = _lib.Workspace(gconf.mesh_shape, adjoint=True, window=window)
        spec = _lib.make_spec(3, gconf.mesh_shape, gconf.mesh_shape, gconf.cell_size)
        n = len(pmid)
        acc = torch.empty((n, 3), dtype=torch.float32, device=cuda)
        dc = torch.empty((n, 3), dtype=torch.float32, device=cuda)
        om = torch.zeros((), dtype=torch.float64, device=cuda)
        _lib.call('pmx_force_vjp', ws.handle, spec, T(pmid, cuda), T(disp, cuda), n,
                  gconf.ptcl_num, 0.3, T(cot, cuda), acc, dc, om, _lib.stream_ptr(cuda))
        out.append((acc.cpu().numpy(), dc.cpu().numpy(), float(om)))
        del ws
    (a1, d1, o1), (a2, d2, o2) = out
    assert rel_l2(a1, acc_o) < RTOL_ACC
    assert rel_l2(a1, a2) < 1e-6
    assert rel_l2(d1, d2) < 1e-5
    assert abs(o1 / o2 - 1) < 5e-5   # a float64 sum over ~1e5 float32 terms in any order


@pytest.mark.parametrize('state', ['lattice', 'halos', 'shuffled_halos'])
def test_aggregated_deposits_equal_direct_atomics(cuda, state):
    """Warp-aggregated deposits (PMX_WS_AGG: lanes whose particles share a
    base cell sum in shared memory, one lane reduces) against one atomic per
    contribution: the force, its VJP and a multi-step forward + adjoint run.
    'halos' pulls the particles into a few dense clumps (many lanes of a warp
    share cells: the aggregated path), 'lattice' barely moves them (no shared
    cells: the direct path of the same kernels)."""
    import ctypes
    oconf, gconf, pmid, disp, vel = make((32, 32, 32), 2, 1.0, 0.05)
    if state != 'lattice':
        pos = ics.pos(pmid, disp, oconf)
        rng = np.random.default_rng(8)
        centres = rng.uniform(0, oconf.box_size[0], (6, 3))
        near = centres[np.argmin(((pos[:, None, :] - centres[None]) ** 2).sum(-1), axis=1)]
        # 95% of the way to the nearest of six centres, plus a little scatter
        pos = pos + 0.95 * (near - pos) + rng.normal(0, 0.3, pos.shape)
        disp = (pos - pmid.astype(np.float64) * oconf.cell_size).astype(np.float32)
        if state == 'shuffled_halos':
            perm = rng.permutation(len(pmid))
            pmid, disp, vel = pmid[perm], disp[perm], vel[perm]
    cot = np.random.default_rng(6).normal(size=disp.shape).astype(np.float32)
    gcos = pg.boltzmann(pg.SimpleLCDM(gconf), gconf)
    fwd = gnb.op_factors(gnb.forward_ops(gconf), gcos, gconf).detach()
    adj = gnb.op_factors(gnb.adjoint_ops(gconf), gcos, gconf).detach()
    f_fwd = np.ascontiguousarray(fwd.to(torch.float32).numpy().reshape(-1, 3))[:4]
    f_adj = np.ascontiguousarray(adj.to(torch.float32).numpy().reshape(-1, 3))[-4:]
    out = []
    for agg in (True, False, False):
        ws = _lib.Workspace(gconf.mesh_shape, adjoint=True, agg=agg)
        spec = _lib.make_spec(3, gconf.mesh_shape, gconf.mesh_shape, gconf.cell_size)
        n, st = len(pmid), _lib.stream_ptr(cuda)
        P, D, V = T(pmid, cuda), T(disp, cuda), T(vel, cuda)
        acc = torch.empty((n, 3), dtype=torch.float32, device=cuda)
        dc = torch.empty((n, 3), dtype=torch.float32, device=cuda)
        om = torch.zeros((), dtype=torch.float64, device=cuda)
        _lib.call('pmx_force_vjp', ws.handle, spec, P, D, n, gconf.ptcl_num, 0.3, T(cot, cuda), acc,
                  dc, om, st)
        res = [acc.cpu().numpy(), dc.cpu().numpy(), float(om)]
        A = torch.empty_like(D)
        _lib.call('pmx_force', ws.handle, spec, P, D, n, gconf.ptcl_num, 0.3, A, st)
        _lib.call('pmx_nbody_steps', ws.handle, spec, P, D, V, A, n, gconf.ptcl_num, 4,
                  f_fwd.ctypes.data_as(ctypes.c_void_p), 0.3, st)
        res.append(D.cpu().numpy())
        vc, al = T(cot, cuda), torch.zeros_like(D)
        dcot = torch.zeros_like(D)
        dots = torch.zeros((4, 4), dtype=torch.float64, device=cuda)
        _lib.call('pmx_nbody_adj_steps', ws.handle, spec, P, D, V, A, dcot, vc, al, n,
                  gconf.ptcl_num, 4, f_adj.ctypes.data_as(ctypes.c_void_p), 0.3, dots, st)
        res += [D.cpu().numpy(), vc.cpu().numpy()]
        out.append(res)
        del ws
    (a1, d1, o1, x1, y1, v1), (a2, d2, o2, x2, y2, v2), (_, _, _, _, _, v3) = out
    # one force: only the order of the float32 adds differs
    assert rel_l2(a1, a2) < 1e-5
    assert rel_l2(d1, d2) < 1e-4
    assert abs(o1 / o2 - 1) < 1e-4
    # 4 forward steps, then 4 reverse steps (which amplify the order noise)
    assert rel_l2(x1, x2) < 1e-5 and rel_l2(y1, y2) < 1e-4
    # the adjoint's vel_cot: a rounding-level change of a reconstructed
    # position (here: another summation order of the deposits) can move a
    # particle across a cell boundary, where the CIC weight gradient jumps
    # and its cotangent changes by O(1).  As in the multi-step test, 0.2% of
    # the particles are set aside; the rest are held to ten times the
    # difference between two runs of the direct path (at least 1e-3), and
    # the whole array to 3e-2 or ten times that difference.
    def kept(a, b):
        e = np.linalg.norm(a - b, axis=1)
        keep = np.argsort(e)[:len(e) - len(e) // 500]
        return rel_l2(a[keep], b[keep])
    assert kept(v1, v2) < max(1e-3, 10 * kept(v3, v2)), (kept(v1, v2), kept(v3, v2))
    assert rel_l2(v1, v2) < max(3e-2, 10 * rel_l2(v3, v2)), (rel_l2(v1, v2), rel_l2(v3, v2))


@pytest.mark.parametrize('case', ['near_lattice', 'scattered'])
def test_tma_staged_gather_equals_global_loads(cuda, case):
    """Forward gathers staged through shared memory by cp.async.bulk.tensor
    (PMX_WS_TMA) against the same kernels reading global memory: the force
    and a multi-step run.  'near_lattice' stages almost every warp (boxes
    at the periodic boundary and warps spanning more than the box read
    global memory); 'scattered' displacements of several cells send most
    warps through the global path.  No wait may give up."""
    import ctypes
    std = 0.05 if case == 'near_lattice' else 3.0
    oconf, gconf, pmid, disp, vel = make((32, 32, 64), 2, 1.0, std)
    acc_o = pm.gravity(pmid, disp, 0.3, oconf)
    gcos = pg.boltzmann(pg.SimpleLCDM(gconf), gconf)
    fwd = gnb.op_factors(gnb.forward_ops(gconf), gcos, gconf).detach()
    f_fwd = np.ascontiguousarray(fwd.to(torch.float32).numpy().reshape(-1, 3))[:4]
    out = []
    for tma in (True, False):
        ws = _lib.Workspace(gconf.mesh_shape, adjoint=True, tma=tma)
        spec = _lib.make_spec(3, gconf.mesh_shape, gconf.mesh_shape, gconf.cell_size)
        n, st = len(pmid), _lib.stream_ptr(cuda)
        P, D, V = T(pmid, cuda), T(disp, cuda), T(vel, cuda)
        A = torch.empty_like(D)
        _lib.call('pmx_force', ws.handle, spec, P, D, n, gconf.ptcl_num, 0.3, A, st)
        a0 = A.cpu().numpy()
        _lib.call('pmx_nbody_steps', ws.handle, spec, P, D, V, A, n, gconf.ptcl_num, 4,
                  f_fwd.ctypes.data_as(ctypes.c_void_p), 0.3, st)
        gave_up = _lib.c_i32()
        _lib.check(_lib.load().pmx_workspace_tma_status(ws.handle, ctypes.byref(gave_up)), 'status')
        out.append((a0, D.cpu().numpy(), V.cpu().numpy(), A.cpu().numpy(), gave_up.value))
        del ws
    (a1, d1, v1, f1, e1), (a2, d2, v2, f2, e2) = out
    assert e1 == 0 and e2 == 0
    assert rel_l2(a1, acc_o) < RTOL_ACC and rel_l2(a1, a2) < 1e-6
    assert rel_l2(d1, d2) < 1e-5 and rel_l2(v1, v2) < 1e-5 and rel_l2(f1, f2) < 1e-5
