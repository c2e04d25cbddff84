"""GPU initial conditions and analysis against the oracle: linear modes,
2LPT displacements/velocities (lpt.py:136-212) and the power spectrum
(spec_util.py:50-147); plus the published LPT statistics of the reference's
quickstart notebook as a statistical pin."""

import numpy as np
import pytest
import torch

from oracle import cosmo as oc, ics
import pmwd_gb300 as pg

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = np.asarray(a, np.complex128)   # real or complex (Fourier modes)
    b = np.asarray(b, np.complex128)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.fixture(scope='module')
def ic_case():
    oconf = oc.OConf(4.0, (32, 32, 32), 2, float_dtype=np.float32)
    gconf = pg.Configuration(4.0, (32, 32, 32), 2)
    ocos = oc.with_tables(oc.simple_lcdm(), oconf)
    gcos = pg.boltzmann(pg.SimpleLCDM(gconf), gconf)
    noise = np.random.default_rng(0).standard_normal((32, 32, 32), dtype=np.float32)
    return oconf, gconf, ocos, gcos, noise


def test_linear_modes_and_lpt_match_oracle(cuda, ic_case):
    oconf, gconf, ocos, gcos, noise = ic_case
    m_o = ics.linear_modes(noise, ocos, oconf)
    m_g = pg.linear_modes(torch.from_numpy(noise).to(cuda), gcos, gconf)
    assert rel_l2(m_g.cpu().numpy(), m_o) < 1e-5
    pmid_o, disp_o, vel_o = ics.lpt(m_o, ocos, oconf)
    ptcl, obs = pg.lpt(m_g, gcos, gconf)
    assert obs is None
    np.testing.assert_array_equal(ptcl.pmid.cpu().numpy(), pmid_o)
    grid = ics.gen_grid(oconf)[1]
    assert rel_l2(ptcl.disp.cpu().numpy() - grid, disp_o - grid) < 1e-4
    assert rel_l2(ptcl.vel.cpu().numpy(), vel_o) < 1e-4


def test_powspec_matches_oracle(cuda, ic_case):
    oconf, gconf, ocos, gcos, noise = ic_case
    f = np.random.default_rng(3).normal(size=(32, 32, 32)).astype(np.float32)
    k_o, P_o, N_o, b_o = ics.powspec(f, 2.0)
    from pmwd_gb300.spec_util import powspec
    k_g, P_g, N_g, b_g = powspec(torch.from_numpy(f).to(cuda), 2.0)
    np.testing.assert_allclose(N_g.cpu().numpy(), N_o)
    np.testing.assert_allclose(k_g.cpu().numpy(), k_o, rtol=1e-12)
    np.testing.assert_allclose(P_g.cpu().numpy(), P_o, rtol=1e-5)
    np.testing.assert_allclose(b_g.cpu().numpy(), b_o, rtol=1e-12)


@pytest.mark.parametrize('shape, bins', [((32, 32, 32), 1), ((24, 20, 15), 1j / 4),
                                         ((40, 36, 18), 2), ((64, 64, 64), 0.5),
                                         ((64, 64, 64), 0.03)])
def test_powspec_kernel_matches_oracle(cuda, shape, bins):
    """pmx_powspec_bin (one pass over the complex64 spectrum) against the
    oracle's digitize/bincount, linear and log bins, odd and even grids; the
    power-of-two grids cover warp-private bins (29), block-shared bins (112)
    and block-shared bins above 48 KB of shared memory (1848)."""
    from pmwd_gb300.spec_util import powspec
    f = np.random.default_rng(4).normal(size=shape).astype(np.float32)
    k_o, P_o, N_o, b_o = ics.powspec(f, 1.5, bins=bins)
    k_g, P_g, N_g, b_g = powspec(torch.from_numpy(f).to(cuda), 1.5, bins=bins)
    np.testing.assert_array_equal(N_g.cpu().numpy(), N_o)
    np.testing.assert_allclose(k_g.cpu().numpy(), k_o, rtol=1e-12)
    np.testing.assert_allclose(P_g.cpu().numpy(), P_o, rtol=1e-5)
    np.testing.assert_allclose(b_g.cpu().numpy(), b_o, rtol=1e-12)


@pytest.mark.parametrize('shape, bins', [((32, 64, 16), 1j / 3), ((64, 32, 32), 0.5),
                                         ((2, 16, 32, 8), 2), ((32, 16, 32), 1j / 3),
                                         ((16, 512, 16), 1j / 3), ((16, 512, 16), 1),
                                         ((8, 1024, 8), 1j / 3), ((8, 1024, 8), 1)])
def test_powspec_half_axis_major_layout(cuda, shape, bins):
    """torch's CUDA rfftn stores (n0, n1, n2h) half-axis major; the kernel
    bins that layout in place (pmx_powspec_bin_zmajor) and must give the
    sums of the transposed, contiguous copy (pmx_powspec_bin), also for a
    cross spectrum, a leading batch axis and the CIC deconvolution window.

    n1 = 16 takes the row kernel's half-axis-major branch; n1 = 32..1024 the
    run kernel, whose lanes walk runs of n1/32 cells: at n1 = 512 and 1024
    a run of 16 or 32 cells crosses several bins (flushes inside a run) and
    the lanes' last bins merge at the end of each row."""
    from pmwd_gb300 import spec_util as su
    rng = np.random.default_rng(7)
    f = torch.from_numpy(rng.normal(size=shape).astype(np.float32)).to(cuda)
    g = torch.from_numpy(rng.normal(size=shape).astype(np.float32)).to(cuda)
    F, G = su.fftfwd(f, axes=(-3, -2, -1)), su.fftfwd(g, axes=(-3, -2, -1))
    grid = tuple(shape[-3:])
    bnum, bcut, edges, right = su._getbins(grid, bins, True)
    for GG, deconv in ((None, None), (G, None), (None, 2)):
        su._GEOMETRY.clear()
        k1, P1, N1 = su._bin_cuda(F, GG, grid, edges, right, bnum, deconv)
        su._GEOMETRY.clear()
        k2, P2, N2 = su._bin_cuda(F.contiguous(), None if GG is None else GG.contiguous(), grid,
                                  edges, right, bnum, deconv)
        np.testing.assert_allclose(k1.cpu().numpy(), k2.cpu().numpy(), rtol=1e-12)
        np.testing.assert_array_equal(N1.cpu().numpy(), N2.cpu().numpy())
        np.testing.assert_allclose(P1.cpu().numpy(), P2.cpu().numpy(), rtol=1e-5)


@pytest.mark.parametrize('shape, bins', [((16, 512, 16), 1j / 3), ((8, 1024, 8), 1)])
def test_powspec_long_runs_match_oracle(cuda, shape, bins):
    """The run kernel at n1 = 512 and 1024 (runs of 16 and 32 cells per
    lane) through the public powspec, against the oracle's float64
    digitize/bincount, with and without the CIC deconvolution."""
    from pmwd_gb300.spec_util import powspec
    f = np.random.default_rng(8).normal(size=shape).astype(np.float32)
    for deconv in (None, 2):
        k_o, P_o, N_o, b_o = ics.powspec(f, 1.0, bins=bins, deconv=deconv)
        k_g, P_g, N_g, b_g = powspec(torch.from_numpy(f).to(cuda), 1.0, bins=bins,
                                     deconv=deconv)
        np.testing.assert_array_equal(N_g.cpu().numpy(), N_o)
        np.testing.assert_allclose(k_g.cpu().numpy(), k_o, rtol=1e-12)
        np.testing.assert_allclose(P_g.cpu().numpy(), P_o, rtol=1e-5)


@pytest.mark.parametrize('shape', [(2, 16, 18, 20), (2, 16, 32, 8)])
def test_powspec_kernel_cross_deconv_batch(cuda, shape):
    """Cross spectrum with a leading channel axis, CIC deconvolution and
    tuple bins: the CUDA kernel path (generic grid, and power-of-two grid
    with its cached geometry sums) against the same function on CPU tensors
    (the digitize/bincount restatement in torch); each case twice, so the
    second call of a power-of-two grid reuses the cached sums."""
    from pmwd_gb300.spec_util import powspec
    rng = np.random.default_rng(5)
    f = rng.normal(size=shape).astype(np.float32)
    g = (f + 0.3 * rng.normal(size=f.shape)).astype(np.float32)
    bins = (0, 0.05, 0.1, 0.2, 0.3, 0.45, 0.6)
    for kw in ({}, {'g': g}, {'g': g, 'deconv': 2}, {'deconv': 2, 'cut_zero': False}):
        cpu = powspec(torch.from_numpy(f), 2.0, bins=bins,
                      **{k: torch.from_numpy(v) if k == 'g' else v for k, v in kw.items()})
        for _ in range(2):
            dev = powspec(torch.from_numpy(f).to(cuda), 2.0, bins=bins,
                          **{k: torch.from_numpy(v).to(cuda) if k == 'g' else v
                             for k, v in kw.items()})
            for a, b in zip(dev, cpu):
                np.testing.assert_allclose(a.cpu().numpy(), b.numpy(), rtol=1e-6, atol=0)


def test_lpt_graph_replay_matches_eager(cuda):
    """Calls without gradients replay a CUDA graph of the 2LPT device work;
    the graph takes the growth factors as an input, so one graph serves
    several cosmologies.  It matches the eager path, which runs when the
    modes need a gradient."""
    import importlib
    glpt = importlib.import_module('pmwd_gb300.lpt')
    conf = pg.Configuration(2.0, (32, 32, 32), 2)
    glpt._GRAPHS.clear()
    for Om in (0.3, 0.25):
        cos = pg.boltzmann(pg.SimpleLCDM(conf).replace(
            Omega_m=torch.tensor(Om, dtype=torch.float64)), conf)
        modes = pg.linear_modes(pg.white_noise(1, conf, device=cuda), cos, conf)
        with torch.no_grad():
            g, _ = pg.lpt(modes, cos, conf)
        e, _ = pg.lpt(modes.clone().requires_grad_(True), cos, conf)
        assert len(glpt._GRAPHS) == 1
        assert torch.equal(g.pmid, e.pmid)
        assert rel_l2(g.disp.cpu().numpy(), e.disp.detach().cpu().numpy()) < 1e-6
        assert rel_l2(g.vel.cpu().numpy(), e.vel.detach().cpu().numpy()) < 1e-6


def test_lpt_graph_concurrent_callers(cuda):
    """Host setup threads (as the server runs them) call lpt at once, each
    needing its own graph: the captures are serialised, run on their own
    streams, and every result equals the eager path's."""
    import importlib
    from concurrent.futures import ThreadPoolExecutor
    glpt = importlib.import_module('pmwd_gb300.lpt')
    glpt._GRAPHS.clear()
    confs = [pg.Configuration(2.0, (s, s, s), m) for s in (16, 32) for m in (1, 2)]
    cosmos = [pg.boltzmann(pg.SimpleLCDM(c), c) for c in confs]
    modes = [pg.linear_modes(pg.white_noise(i, c, device=cuda), cos, c)
             for i, (c, cos) in enumerate(zip(confs, cosmos))]
    torch.cuda.synchronize()

    def work(i):
        with torch.no_grad():
            p, _ = pg.lpt(modes[i], cosmos[i], confs[i])
        torch.cuda.current_stream().synchronize()
        return p.disp.cpu().numpy(), p.vel.cpu().numpy()

    with ThreadPoolExecutor(4) as ex:
        got = list(ex.map(work, list(range(len(confs))) * 2))
    for i, c in enumerate(confs):
        e, _ = pg.lpt(modes[i].clone().requires_grad_(True), cosmos[i], c)
        for g in (got[i], got[i + len(confs)]):
            assert rel_l2(g[0], e.disp.detach().cpu().numpy()) < 1e-6
            assert rel_l2(g[1], e.vel.detach().cpu().numpy()) < 1e-6


def test_lpt_graph_capture_leaves_pooled_streams_alone(cuda):
    """torch.cuda.Stream() draws from a fixed pool (32 per device), so a
    graph captured on a pooled stream would also record the work another
    thread launches on that same stream (the server's request and group
    streams are pooled streams).  The 2LPT graphs are captured on a stream
    the library created: work launched on every pooled stream while a graph
    is being built runs, and its events can be queried."""
    import importlib
    import threading
    glpt = importlib.import_module('pmwd_gb300.lpt')
    glpt._GRAPHS.clear()
    streams = [torch.cuda.Stream(device=cuda) for _ in range(64)]
    pooled = {s.cuda_stream for s in streams}
    assert len(pooled) < len(streams)                 # the pool wraps around
    conf = pg.Configuration(2.0, (32, 32, 32), 2)
    cosmo = pg.boltzmann(pg.SimpleLCDM(conf), conf)
    modes = pg.linear_modes(pg.white_noise(3, conf, device=cuda), cosmo, conf)
    counts = torch.zeros(len(streams), device=cuda)
    torch.cuda.synchronize()
    done = threading.Event()

    def build():
        try:
            with torch.no_grad():
                pg.lpt(modes, cosmo, conf)
        finally:
            done.set()

    th = threading.Thread(target=build)
    th.start()
    rounds = 0
    try:
        while not done.is_set() or rounds < 3:
            for i, s in enumerate(streams):
                with torch.cuda.stream(s):
                    counts[i:i + 1].add_(1.0)
                    ev = torch.cuda.Event()
                    ev.record(s)
                ev.query()
            rounds += 1
    finally:
        th.join()
    torch.cuda.synchronize()
    assert torch.all(counts == rounds), counts
    graphs = list(glpt._GRAPHS.values())
    assert graphs and all(g.stream.cuda_stream not in pooled for g in graphs)


def test_lpt_statistics_match_published(cuda):
    """docs/examples/quickstart.ipynb prints, for 256^3 particles, spacing 1,
    2x mesh, SimpleLCDM, after 2LPT at a=1/64: disp.std() = 0.105 and
    vel.std() = 0.007 (3 digits).  Our white noise is a different
    realisation of the same distribution, so agreement is statistical (a few
    percent: the large-scale modes of a 256 Mpc/h box carry cosmic variance)."""
    conf = pg.Configuration(1.0, (256, 256, 256), 2)
    cosmo = pg.boltzmann(pg.SimpleLCDM(conf), conf)
    with torch.no_grad():
        modes = pg.linear_modes(pg.white_noise(0, conf, device=cuda), cosmo, conf)
        ptcl, _ = pg.lpt(modes, cosmo, conf)
    disp_std = float(ptcl.disp.double().std())
    vel_std = float(ptcl.vel.double().std())
    assert abs(disp_std / 0.105 - 1) < 0.05, disp_std
    assert abs(vel_std / 0.007 - 1) < 0.08, vel_std   # printed to one significant digit
