"""Particle sharding through the product: the open-boundary fixture run
whole by one Solver, and split in two by Solver(shard=(rank, 2)) run one
after the other on the same GPU (ranks exchange nothing while stepping).
Every particle that stays active ends where the single run puts it, bit for
bit (its stream follows its tag, which the split keeps); the exit counts
summed over the shards equal the single run's; the tags the shards give to
deleted particles never coincide."""
import numpy as np
import pytest

from conftest import fields_from_case, load_golden, mesh_from_case

pytestmark = pytest.mark.gpu


def _run(case, meta, precision, shard=None):
    import cylag_gb300 as cg
    f = fields_from_case(case)
    fs = cg.EulerianFieldSet(mesh_from_case(case), **f)
    ps = cg.LagrangianParticleSet(case["position"], dim=2, **meta.get("pset", {}))
    tag0 = None
    s = cg.Solver(fs, ps, meta["params"], precision=precision, seed=meta["seed"], shard=shard)
    tag0 = ps.tag.copy()
    s.forward(nsteps=meta["nsteps"])
    out = dict(tag0=tag0, tag=ps.tag, pos=ps.position, tri=ps.tri, inactive=ps.inactive,
               stats=s.bnd_statistics().sum(0))
    s.close()
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_two_shards_equal_one_run(precision):
    case, meta, _ = load_golden("open")
    one = _run(case, meta, precision)
    parts = [_run(case, meta, precision, shard=(r, 2)) for r in range(2)]
    # active particles of the shards, by their (kept) tags
    for p in parts:
        act = p["inactive"] == 0
        for t, x, k in zip(p["tag"][act], p["pos"][act], p["tri"][act]):
            j = np.flatnonzero((one["tag"] == t) & (one["inactive"] == 0))
            assert len(j) == 1, t
            np.testing.assert_array_equal(x, one["pos"][j[0]])
            assert k == one["tri"][j[0]]
    n_act = sum(int((p["inactive"] == 0).sum()) for p in parts)
    assert n_act == int((one["inactive"] == 0).sum())
    np.testing.assert_array_equal(parts[0]["stats"] + parts[1]["stats"], one["stats"])
    assert one["stats"].sum() > 0
    new = np.concatenate([p["tag"][p["inactive"] == 1] for p in parts])
    assert len(np.unique(new)) == len(new)
