"""The replicas path of bench.py under torchrun (one process per GPU, images
sharded by rank, no collective on the data path): on the CPU with the gloo
backend and world size 2, its rank helpers give every rank the slowest
rank's time after a barrier, and the reference arm runs on rank 0 only.
(On a GPU machine these helpers use NCCL under torchrun, one GPU per rank;
this test stays on the CPU.)"""
import argparse
import contextlib
import io
import os
import socket
import sys

import pytest

torch = pytest.importorskip('torch')

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank),
                      MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    w, r, _ = bench.dist_init()
    slowest = bench.max_over_ranks(10.0 + r, w)  # rank r "took" 10 + r ms
    bench.barrier(w)
    printed = io.StringIO()
    if r == 1:  # the reference arm: every rank but 0 returns at once, silently
        args = argparse.Namespace(steps=1, warmup=0, gpus=w)
        with contextlib.redirect_stdout(printed):
            bench.run_reference(args, w, r)
    bench.barrier(w)
    import torch.distributed as dist
    dist.destroy_process_group()
    with open(os.path.join(out, 'rank%d' % r), 'w') as f:
        f.write('%d %d %r %d' % (w, r, slowest, len(printed.getvalue())))


@pytest.mark.skipif(torch.cuda.is_available(), reason='CPU ranks over gloo')
def test_ranks_gloo_world2(tmp_path):
    import torch.multiprocessing as mp
    mp.spawn(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    for r in range(2):
        w, rr, slowest, printed = open(tmp_path / ('rank%d' % r)).read().split()
        assert (int(w), int(rr)) == (2, r)
        assert float(slowest) == 11.0  # the max over ranks, on every rank
        assert int(printed) == 0
