"""Multi-rank path on CPU (gloo, world size 2): the particle set split across
ranks as the reference's parallel solver splits it, each rank stepping its
slice with per-particle streams keyed by the global index, the boundary
exit counts summed over ranks.  The gathered result equals the single-rank
run bit for bit."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    sys.path[:0] = [str(root), str(root / "oracle"), str(root / "tests")]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from conftest import fields_from_case, load_golden, mesh_from_case
    import oracle
    from cylag_gb300 import shard
    case, meta, _ = load_golden("open")
    n = len(case["position"])
    sl = shard.shard_slice(n, rank, world)
    tags = np.arange(n)[sl]
    o = oracle.OracleSolver(mesh_from_case(case), fields_from_case(case), meta["params"],
                            case["position"][sl], pset=meta.get("pset"), seed=meta["seed"],
                            tags=tags)
    o.solve(meta["nsteps"])
    stats = shard.allreduce_sum(np.array(o.bnd_stats).sum(0), dist)
    pos = shard.gather_rows(o.pos, dist, rank, world)
    tri = shard.gather_rows(o.tri, dist, rank, world)
    t = shard.allreduce_max(float(rank + 1), dist)
    if rank == 0:
        np.savez(out, pos=pos, tri=tri, stats=stats, tmax=t)
    dist.barrier()
    dist.destroy_process_group()


def test_split_matches_reference_rule():
    from cylag_gb300 import shard
    assert shard.split(10, 3) == [(0, 3), (3, 3), (6, 4)]
    assert shard.split(64, 2) == [(0, 32), (32, 32)]
    assert sum(c for _, c in shard.split(12345, 8)) == 12345


def test_two_ranks_equal_one(tmp_path, oracle_lib):
    import torch.multiprocessing as mp
    from conftest import load_golden, run_oracle
    out = str(tmp_path / "r0.npz")
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, join=True,
                       start_method="spawn")
    z = np.load(out)
    case, meta, _ = load_golden("open")
    o = run_oracle(case, meta)
    np.testing.assert_array_equal(z["pos"], o.pos)
    np.testing.assert_array_equal(z["tri"], o.tri)
    np.testing.assert_array_equal(z["stats"], np.array(o.bnd_stats).sum(0))
    assert float(z["tmax"]) == 2.0


def _split_worker(rank, world, port, out):
    """The product's split on each gloo rank: LagrangianParticleSet.
    parallel_split of the same set, then deletions retagged on each rank;
    the ranks' tags gathered on rank 0."""
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    sys.path[:0] = [str(root), str(root / "oracle"), str(root / "tests")]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import cylag_gb300 as cg
    from cylag_gb300 import shard
    from cylag_gb300.core import retag
    rng = np.random.default_rng(3)
    pos = rng.uniform(0, 100, (1003, 2))
    ps = cg.LagrangianParticleSet(pos, dim=2, initial_pool_size=1200)
    ps.parallel_split(rank, world)
    kept = ps._host["tag"][ps._host["tri"] == -2]
    pad = ps._host["tag"][ps._host["tri"] == -1]
    # particles deleted during two iterations, retagged as the step does
    tag = ps._host["tag"].copy()
    tag[[0, 5]] = -2
    tag[[3]] = -3
    new, maxtag = retag(tag, ps.maxtag, ps.tag_stride)
    fresh = new[[0, 3, 5]]
    g = {k: shard.gather_rows(v, dist, rank, world) for k, v in
         (("kept", kept), ("pad", pad), ("fresh", fresh),
          ("kpos", ps._host["position"][ps._host["tri"] == -2]))}
    n = shard.gather_rows(np.array([ps.npart]), dist, rank, world)
    if rank == 0:
        np.savez(out, n=n, **g)
    dist.barrier()
    dist.destroy_process_group()


def test_product_split_gives_disjoint_streams(tmp_path):
    """Two gloo ranks split one particle set as the reference's parallel
    solver does: every active particle kept once with its tag (its PCG32
    stream) and position, pools of n // world entries, and the tags the
    ranks give to padding and to deleted particles never coincide, with
    each other or with the original tags."""
    import torch.multiprocessing as mp
    out = str(tmp_path / "split.npz")
    mp.start_processes(_split_worker, args=(2, _free_port(), out), nprocs=2, join=True,
                       start_method="spawn")
    z = np.load(out)
    rng = np.random.default_rng(3)
    pos = rng.uniform(0, 100, (1003, 2))
    np.testing.assert_array_equal(z["kept"], np.arange(1003))
    np.testing.assert_array_equal(z["kpos"], pos)
    assert z["n"].tolist() == [600, 600]            # 1200 // 2 each, 1003 active split 501/502
    new = np.concatenate([z["pad"], z["fresh"]])
    assert len(np.unique(new)) == len(new)
    assert new.min() > 1199                         # beyond every tag of the unsplit set
