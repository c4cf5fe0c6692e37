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
