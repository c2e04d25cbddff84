"""Host logic of bench.py without a GPU: the committed DRAM-traffic summary it
reads for roofline.traffic, the algorithmic-byte table behind the per-stage
rates and the step-roofline convention, and the parsing of nvidia-smi clock
samples (the throttle reasons a bench line must report)."""

import importlib.util
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope='module')
def bench():
    spec = importlib.util.spec_from_file_location('bench', os.path.join(ROOT, 'bench.py'))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_traffic_summary_covers_every_own_kernel(bench):
    t = bench.ncu_traffic()
    for stage in bench.OWN_KERNELS:
        assert stage in t and t[stage] > 1e9, stage


def test_algorithmic_bytes_follow_the_convention(bench):
    N, M = 512 ** 3, 1024 ** 3
    Mc = 1024 * 1024 * 513
    ab = bench.algorithmic_bytes(N, M, Mc)
    # one read + one write of input and output per FFT-like pass
    assert ab['r2c'] == 4 * M + 8 * Mc
    assert ab['c2r_x3'] == 3 * (8 * Mc + 4 * M)
    assert ab['poisson_fwd'] == ab['poisson_adj'] == 32 * Mc
    # with Mc = M / 2 (as the step convention rounds it) the forward step's
    # mesh bytes are the convention's 64 M; its joined particle pass moves
    # 54 N where the convention counts separate kick, drift, scatter and
    # gather passes (156 N)
    h = bench.algorithmic_bytes(N, M, M // 2)
    fwd = h['r2c'] + h['poisson_fwd'] + h['c2r_x3'] + h['gather3_kick_kick_drift_deposit']
    assert fwd == 54 * N + 64 * M
    assert fwd <= 156 * N + 64 * M


def _fake_sampler(bench, lines):
    s = bench.ClockSampler(0)

    class P:
        def terminate(self):
            pass

        def wait(self, timeout=None):
            return 0

    s.proc = P()
    s.lines = lines
    return s


def test_clock_samples_report_throttle_reasons(bench):
    fmt = '0, {sm}, 2070, {pw}, 0x0, {hw}, Not Active, Not Active, {cap}'
    lines = [fmt.format(sm=2070, pw=800, hw='Not Active', cap='Not Active'),
             fmt.format(sm=2070, pw=850, hw='Not Active', cap='Active'),
             fmt.format(sm=1980, pw=820, hw='Active', cap='Not Active'),
             fmt.format(sm=600, pw=90, hw='Not Active', cap='Not Active'),   # idle sample
             'garbage line']
    out = _fake_sampler(bench, lines).stop()
    assert out['sm_max_mhz'] == 2070
    assert out['reasons'] == ['hw_slowdown', 'sw_power_cap']
    assert out['sm_mhz'] == 2070          # median of the loaded samples only
    assert out['samples'] == 4 and out['power_w_max'] == 850


def test_clock_samples_without_nvidia_smi(bench):
    s = bench.ClockSampler(0)
    assert s.stop()['reasons'] == ['nvidia-smi unavailable']
