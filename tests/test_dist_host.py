"""The N>1 bench path on CPU: two gloo ranks on 127.0.0.1.

The imaging path does not shard on this pool (one GPU per box): ``bench.py
--gpus N`` runs N replicas, each on its own GPU, and the job's step time is
the slowest rank's.  These tests cover that host logic without a GPU: the
process group comes up on gloo, every rank receives the max over ranks, and
under the reference arm only rank 0 reports while the others exit quietly.
"""
import argparse
import contextlib
import io
import json
import multiprocessing as mp
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _env(rank, world, port):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))


def _max_worker(rank, world, port, q):
    _env(rank, world, port)
    import torch.distributed as dist

    import bench
    r, w = bench.dist_setup(argparse.Namespace(gpus=world))
    got = bench.max_over_ranks(3.0 + 2.5 * rank, w)
    q.put((rank, r, w, dist.get_backend(), got))
    dist.barrier()
    dist.destroy_process_group()


def _reference_worker(rank, world, port, q):
    _env(rank, world, port)
    import torch.distributed as dist

    import bench
    args = argparse.Namespace(gpus=world, config="small-array", scale="tiny", warmup=3, steps=1,
                              cpu_planes=1, ref_planes=1)
    out = io.StringIO()
    with contextlib.redirect_stdout(out):
        bench.run_reference(args)
    q.put((rank, out.getvalue()))
    if dist.is_initialized():
        dist.destroy_process_group()


def _run(target, world=2, timeout=120):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=target, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=timeout) for _ in procs]
    for p in procs:
        p.join(timeout=timeout)
        assert p.exitcode == 0
    return sorted(res)


def test_two_gloo_ranks_agree_on_the_slowest_step():
    res = _run(_max_worker)
    assert [r[:4] for r in res] == [(0, 0, 2, "gloo"), (1, 1, 2, "gloo")]
    assert all(r[4] == pytest.approx(5.5) for r in res)


def test_reference_arm_reports_on_rank_zero_only():
    res = _run(_reference_worker)
    (r0, out0), (r1, out1) = res
    assert out1 == ""
    line = json.loads(out0.strip().splitlines()[-1])
    assert line["impl"] == "reference"
