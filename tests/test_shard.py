"""Several ranks on one survey (wemgpu.shard): shot blocks and the image sum, as
world_size-2 gloo process groups on the host. The per-rank operator is the oracle's
restatement of the reference's migration, so no GPU is needed."""
import os
import socket

import numpy as np
import pytest

from conftest import rel_l2


def test_shard_bounds_cover_every_shot_once():
    from wemgpu import shard
    for nshot in (1, 5, 64, 65):
        for world in (1, 2, 3, 8):
            if world > nshot:
                continue
            b = [shard.shard_bounds(nshot, r, world) for r in range(world)]
            assert b[0][0] == 0 and b[-1][1] == nshot
            assert all(b[i][1] == b[i + 1][0] for i in range(world - 1))
            sizes = [hi - lo for lo, hi in b]
            assert max(sizes) - min(sizes) <= 1


def test_shard_shots_rebases_traces():
    from wemgpu import shard, synth
    c = synth.small_case(61, nx=32, nz=4, nt=32, nshot=5)
    s = c["shots"]
    parts = [shard.shard_shots(s, r, 2) for r in range(2)]
    assert sum(p.nshot for p in parts) == 5
    assert np.array_equal(np.concatenate([p.data for p in parts]), s.data)
    assert np.array_equal(np.concatenate([p.trace_cell for p in parts]), s.trace_cell)
    for p in parts:
        assert p.trace_offset[0] == 0 and p.trace_offset[-1] == len(p.data)


def _free_port():
    with socket.socket() as k:
        k.bind(("127.0.0.1", 0))
        return k.getsockname()[1]


def _oracle_migrate(c):
    import oracle as O
    from wemgpu import synth

    def run(shots):
        p = c["params"]
        img = None
        for i in range(shots.nshot):
            d = synth.shot_gather_full(shots, i, p["nmx"])
            m = O.wem_port(dict(p, sx=float(shots.sx[i])), c["vel"], c["wav"], d=d, adj=True, nthreads=1)
            img = m.astype(np.float64) if img is None else img + m
        return img.astype(np.float32)
    return run


def _rank_main(rank, world, port, out_dir):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    sys.path[:0] = [here, os.path.join(root, "oracle"), os.path.join(root, "seismic.jl_gb300")]
    import torch.distributed as dist
    from wemgpu import shard, synth
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        c = synth.small_case(62, nx=64, nz=12, nt=64, nshot=5, pspi=1, nref=3)
        img = shard.migrate_sharded(_oracle_migrate(c), c["shots"], rank, world)
        np.save(os.path.join(out_dir, f"img{rank}.npy"), img)
    finally:
        dist.destroy_process_group()


def test_sharded_migration_equals_single_rank(tmp_path, oracle_mod):
    import torch.multiprocessing as mp
    from wemgpu import synth
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    c = synth.small_case(62, nx=64, nz=12, nt=64, nshot=5, pspi=1, nref=3)
    whole = _oracle_migrate(c)(c["shots"])
    a, b = np.load(tmp_path / "img0.npy"), np.load(tmp_path / "img1.npy")
    assert np.array_equal(a, b)  # every rank ends with the same image
    assert rel_l2(a, whole) < 1e-6
