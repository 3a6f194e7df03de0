"""The N>1 host logic on CPU with the gloo backend, world size 2.

Ranks split a render by ray range (ear_render_params.first_ray, the oracle
standing in for the GPU on CPU); one all-reduce of the raw histograms
gives the unsplit render.  bench.py's rank setup and max/sum reductions
run under the same launch."""
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    try:
        # CPU ranks: gloo, never two ranks on one GPU
        os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                          WORLD_SIZE=str(world), LOCAL_RANK=str(rank), CUDA_VISIBLE_DEVICES="")
        sys.path.insert(0, str(ROOT))
        import bench
        import oracle
        from ear_gb300 import scenes

        r, wsize, local = bench.dist_init(world)
        assert (r, wsize, local) == (rank, world, rank)
        w = scenes.small_test_room()
        n = 400
        kw = dict(w.render, num_rays=n, raw=True, first_ray=rank * n)
        part = oracle.render(w.vertices, w.material_ids, w.materials, w.source, w.recorders,
                             threads=2, **kw)
        h = torch.from_numpy(np.ascontiguousarray(part["hist64"]))
        dist.all_reduce(h, op=dist.ReduceOp.SUM)
        seg = bench.sum_over_ranks(float(part["counters"]["segments"]), world)
        slowest = bench.max_over_ranks(float(rank + 1), world)
        bench.barrier(world)
        if rank == 0:
            whole = oracle.render(w.vertices, w.material_ids, w.materials, w.source, w.recorders,
                                  threads=2, **dict(kw, num_rays=n * world, first_ray=0))
            ref = whole["hist64"]
            err = float(np.abs(h.numpy() - ref).max() / max(np.abs(ref).max(), 1e-300))
            q.put(("ok", err, seg, float(whole["counters"]["segments"]), slowest))
        dist.destroy_process_group()
    except Exception as e:  # report to the parent instead of hanging it
        q.put(("error", repr(e)))


def test_two_ranks_split_by_ray_range_and_reduce():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
    assert res[0] == "ok", res
    _, err, seg, seg_whole, slowest = res
    assert err < 1e-12
    assert seg == seg_whole
    assert slowest == 2.0
