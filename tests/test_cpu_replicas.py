"""The N > 1 path of bench.py on CPU: replicas time themselves, the slowest
rank's time is taken over a `gloo` process group, and under torchrun the
reference arm runs on rank 0 alone (the other ranks exit 0 without work)."""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _replica(rank, world_size, port, out_dir):
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group('gloo', rank=rank, world_size=world_size)
    seconds = bench.max_over_ranks(0.5 + rank, dist, device='cpu')      # rank 1 is slower
    rate = bench.whole_job_rate(world_size, 1000, 10, seconds)
    dist.barrier()
    dist.destroy_process_group()
    with open(os.path.join(out_dir, 'r%d.json' % rank), 'w') as fp:
        json.dump({'seconds': seconds, 'rate': rate}, fp)


def test_max_over_ranks_gloo(tmp_path):
    mp.spawn(_replica, args=(2, free_port(), str(tmp_path)), nprocs=2, join=True)
    got = [json.load(open(tmp_path / ('r%d.json' % r))) for r in range(2)]
    assert all(g['seconds'] == 1.5 for g in got)                     # the slowest rank
    assert all(g['rate'] == 2 * 1000 * 10 / 1.5 for g in got)        # whole job over the slowest


def test_reference_arm_under_torchrun():
    cmd = [sys.executable, '-m', 'torch.distributed.run', '--nnodes', '1', '--nproc-per-node', '2',
           '--master-addr', '127.0.0.1', '--master-port', str(free_port()),
           os.path.join(ROOT, 'bench.py'), '--impl', 'reference', '--gpus', '2', '--steps', '1',
           '--warmup', '0', '--agents', '2000']
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith('{')]
    assert len(lines) == 1, r.stdout                                   # rank 0 alone prints
    line = lines[0]
    assert line['impl'] == 'reference' and line['n_gpus'] == 2 and line['value'] > 0
    assert line['cpu_baseline']['kind'] == 'port'
