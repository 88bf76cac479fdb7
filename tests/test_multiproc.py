"""Multi-process paths on CPU (gloo, world size 2): the replica bookkeeping
bench.py uses under torchrun (barrier, max of per-rank times, sum of
per-rank segment counts), and a two-way split of one image by row bands
whose host-side sum equals the one-process image (the only exchange a
sharded render needs)."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_dir):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import importlib
    bench = importlib.import_module("bench")
    # replica timing: max over ranks, segments summed
    t = bench.max_over_ranks(dist, float(10 + rank))
    s = bench.sum_over_ranks(dist, float(100 * (rank + 1)))
    bench.barrier(dist)
    # row-band split of one Cornell render with the oracle
    import oracle
    solrt = importlib.import_module("sol-rs_gb300")
    d = solrt.scenes.cornell()
    c = d.camera
    cam = oracle.camera_look_at(c["eye"], c["center"], c["up"], c["vfov"], 1.0)
    p = solrt.render_params(32, 32, spp=2, max_bounces=3, material_mode=solrt.MATERIAL_LAMBERT,
                            rng_mode=solrt.RNG_PER_SAMPLE, seed=1)
    band = (rank * 16, (rank + 1) * 16)
    acc, _, _ = oracle.OracleScene(d).render(cam, p, rows=band, threads=1)
    part = np.zeros_like(acc)
    part[band[0]:band[1]] = acc[band[0]:band[1]]
    ten = torch.from_numpy(part)
    dist.all_reduce(ten, op=dist.ReduceOp.SUM)
    if rank == 0:
        np.save(os.path.join(out_dir, "sum.npy"), ten.numpy())
        np.save(os.path.join(out_dir, "scalars.npy"), np.array([t, s]))
    dist.destroy_process_group()


def test_two_ranks_gloo(tmp_path, oracle, solrt):
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    t, s = np.load(tmp_path / "scalars.npy")
    assert t == 11.0 and s == 300.0
    d = solrt.scenes.cornell()
    c = d.camera
    cam = oracle.camera_look_at(c["eye"], c["center"], c["up"], c["vfov"], 1.0)
    p = solrt.render_params(32, 32, spp=2, max_bounces=3, material_mode=solrt.MATERIAL_LAMBERT,
                            rng_mode=solrt.RNG_PER_SAMPLE, seed=1)
    full, _, _ = oracle.OracleScene(d).render(cam, p)
    summed = np.load(tmp_path / "sum.npy")
    assert np.array_equal(summed, full)
