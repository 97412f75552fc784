"""Replica-parallel path on CPU: two gloo ranks each contract their shard of
the defect bands (FP64 oracle, cfg0 workload) and the concatenated blocks
equal the single-process result; the timing reductions return the max and
the sum over ranks."""

import os
import socket
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def worker(rank, world, port, basis_dir, defect_dir, out):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as td

    td.init_process_group("gloo", rank=rank, world_size=world)
    import oracle as orc
    from pawpyseed_gb300 import replicas

    b = orc.OracleWavefunction(basis_dir)
    w = orc.OracleWavefunction(defect_dir)
    full = orc.OracleProjector(w, b).pseudo_full()  # [nk][nbS][nbR]
    mine = replicas.shard(w.nband, rank, world)
    block = {i: np.asarray(full)[:, i, :] for i in mine}
    gathered = [None] * world
    td.all_gather_object(gathered, block)
    mx = replicas.max_over_ranks(td, rank + 1.5)
    sm = replicas.sum_over_ranks(td, rank + 1.0)
    if rank == 0:
        merged = {}
        for g in gathered:
            merged.update(g)
        np.save(out, np.stack([merged[i] for i in range(w.nband)], axis=1))
        np.save(out + ".red.npy", np.array([mx, sm]))
    td.barrier()
    td.destroy_process_group()


def test_shards_cover_every_item_once():
    from pawpyseed_gb300.replicas import shard

    for n in (0, 1, 7, 32, 1024):
        for world in (1, 2, 3, 8):
            got = [i for r in range(world) for i in shard(n, r, world)]
            assert got == list(range(n))
            sizes = [len(shard(n, r, world)) for r in range(world)]
            assert max(sizes) - min(sizes) <= 1


def test_two_gloo_ranks_concatenate_to_the_single_result(workload_dirs, tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc

    d = workload_dirs("cfg0")
    out = str(tmp_path / "merged.npy")
    mp.spawn(worker, args=(2, free_port(), d["basis"], d["defect"], out), nprocs=2, join=True)
    merged = np.load(out)
    ref = np.asarray(orc.OracleProjector(orc.OracleWavefunction(d["defect"]),
                                         orc.OracleWavefunction(d["basis"])).pseudo_full())
    assert merged.shape == ref.shape
    assert np.array_equal(merged, ref)
    mx, sm = np.load(out + ".red.npy")
    assert mx == 2.5 and sm == 3.0
