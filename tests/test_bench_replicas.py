"""The N > 1 path of bench.py on the CPU: independent replicas, one per rank, no collective in
the data path.  (a) Two gloo ranks agree on the slowest rank's time and on the whole-job
throughput; (b) under torchrun with two ranks the reference arm runs on rank 0 alone and prints
exactly one JSON line."""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    import bench
    dist.init_process_group('gloo', init_method=f'tcp://127.0.0.1:{port}', rank=rank, world_size=world)
    ms = [120.0, 150.0][rank]           # the second rank is slower
    ms_max = bench.max_over_ranks(ms, dist, 'cpu')
    out[rank] = (ms_max, bench.replica_throughput(world, 5, ms_max))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_timing_is_max_over_ranks():
    ctx = mp.get_context('spawn')
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        ps = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in ps:
            p.start()
        for p in ps:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    assert res[0] == res[1] == (150.0, 2 * 5 / 0.150)


def test_single_process_needs_no_collective():
    sys.path.insert(0, REPO)
    import bench
    assert bench.max_over_ranks(80.0, None, 'cpu') == 80.0
    assert bench.replica_throughput(1, 4, 80.0) == pytest.approx(50.0)


def test_reference_arm_under_torchrun_prints_one_line():
    port = _free_port()
    cmd = [sys.executable, '-m', 'torch.distributed.run', '--nnodes', '1', '--nproc-per-node', '2', '--master-addr', '127.0.0.1',
           '--master-port', str(port), 'bench.py', '--impl', 'reference', '--workload', 'cubes', '--gpus', '2', '--steps', '1',
           '--warmup', '0']
    env = dict(os.environ, OMP_NUM_THREADS='2')
    r = subprocess.run(cmd, cwd=REPO, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith('{')]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d['impl'] == 'reference' and d['value'] > 0 and d['n_gpus'] == 2


def test_reference_arm_2d_prints_one_line():
    """The 2D workload's reference arm (the 2D oracle on the host cores) prints one JSON line."""
    cmd = [sys.executable, 'bench.py', '--impl', 'reference', '--workload', 'stack2d', '--steps', '1', '--warmup', '1']
    r = subprocess.run(cmd, cwd=REPO, capture_output=True, text=True, timeout=600, env=dict(os.environ, OMP_NUM_THREADS='2'))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith('{')]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d['impl'] == 'reference' and d['value'] > 0 and d['cpu_baseline']['cores'] == 2
