"""Multi-GPU runs are independent replicas (the transparent pass has no data
exchange between GPUs); the bench's only exchange is the max over ranks of
the timed durations and the sum of the work. Covered here with world_size-2
gloo ranks on the CPU."""
import os
import socket
import subprocess
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    dist.init_process_group('gloo', rank=rank, world_size=world)
    maxes, sums = bench.reduce_replicas([1.5 + rank, 7.0 - 3 * rank], [100 * (rank + 1), rank], world, 'cpu')
    q.put((rank, maxes, sums))
    dist.destroy_process_group()


def test_reduce_replicas_gloo():
    world = 2
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for _, maxes, sums in out:
        assert maxes == [2.5, 7.0]
        assert sums == [300.0, 1.0]


def test_reduce_replicas_single():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_replicas([3.0], [4], 1, 'cpu') == ([3.0], [4.0])


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, RANK='1', WORLD_SIZE='2', LOCAL_RANK='1')
    p = subprocess.run([sys.executable, os.path.join(ROOT, 'bench.py'), '--impl', 'reference', '--gpus', '2',
                        '--steps', '1', '--warmup', '0'], env=env, capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stderr
    assert p.stdout.strip() == ''
