"""Multi-GPU runs are independent replicas (the particle-mesh path does not
shard): the only cross-rank step is the final timing reduction of bench.py.
This runs it as two gloo ranks on CPU."""

import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    import bench
    # rank r took (r+1)*100 ms for its own 1000 particle-steps
    ms, value = bench.replica_throughput(100.0 * (rank + 1), 1000, world, 'cpu')
    q.put((rank, ms, value))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_throughput_two_ranks():
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, value in out:
        assert ms == pytest.approx(200.0)              # max over ranks
        assert value == pytest.approx(2000 / 0.2)       # all ranks' units / slowest time


def test_replica_throughput_single_rank():
    import bench
    ms, value = bench.replica_throughput(50.0, 500, 1, 'cpu')
    assert ms == 50.0 and value == pytest.approx(10000.0)


def test_bench_gpus_flag_launches_replicas():
    """``bench.py --gpus 2`` outside torchrun starts two ranks itself (one
    replica per GPU); with --dry-run they do no GPU work and report
    100 + 10 rank ms, so the printed line must carry n_gpus 2, the slowest
    rank's time and both ranks' particle-steps."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, os.path.join(root, 'bench.py'), '--gpus', '2', '--dry-run',
                        '--steps', '3', '--ptcl', '8'], cwd=root, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith('{')]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line['n_gpus'] == 2 and line['dry_run']
    assert line['ms_per_step'] == pytest.approx(110.0 / 3)
    assert line['value'] == pytest.approx(2 * 8 ** 3 * 3 / 0.110)
