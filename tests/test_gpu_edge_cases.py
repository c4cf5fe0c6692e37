"""Edge cases of the GPU step: an empty particle set, particle counts that
leave ragged warps and blocks, and a pool whose particles all leave
through open boundaries or strand (then keep stepping with none active).
Both forms; unsorted and element-sorted calls.

Plain form: element indices, deletions and tags bit-exact against the
oracle, positions within 1e-10 relative.  Mixed form: same decisions,
FP32 increments: element indices agree for at least 95% of the particles
and positions within 1e-3 m over 30 steps of 2 s.
"""
import numpy as np
import pytest

from conftest import RTOL, assert_state_close, load_golden, run_oracle

pytestmark = pytest.mark.gpu


def _solver(case, params, precision, sort_period, seed):
    import cylag_gb300 as cg
    from conftest import fields_from_case, mesh_from_case
    fs = cg.EulerianFieldSet(mesh_from_case(case), **fields_from_case(case))
    ps = cg.LagrangianParticleSet(case["position"], dim=2)
    s = cg.Solver(fs, ps, params, precision=precision, seed=seed, sort_period=sort_period)
    return s, ps


def _keps_case(n):
    from cylag_gb300 import synth
    c = synth.keps_drift_channel(npart=max(n, 1), nx=41, ny=11, seed=7)
    case = {k: c[k] for k in ("x", "y", "triangles", "times", "elevation", "velocity_x",
                              "velocity_y", "opt_fields", "position")}
    case["opt_fields_names"] = c["opt_fields_names"]
    case["position"] = np.ascontiguousarray(c["position"][:n])
    p = dict(c["parameters"])
    p.update(time_step=2.0, final_time=400.0)
    return case, p


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_empty_particle_set(precision):
    """No particles: steps (sorted calls included) run and change nothing."""
    case, p = _keps_case(0)
    s, ps = _solver(case, p, precision, sort_period=5, seed=1)
    s.forward(nsteps=12)
    s.forward(nsteps=1)
    assert ps.npart == 0 and ps.position.shape == (0, 2)
    s.close()


@pytest.mark.parametrize("sort_period", [0, 5])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("n", [1, 31, 33, 257, 1000])
def test_ragged_counts_follow_oracle(n, precision, sort_period):
    """Counts below, at and just past a warp and a block of 256, k-eps drift
    with time interpolation and wall rebounds, against the oracle."""
    case, p = _keps_case(n)
    meta = dict(params=p, nsteps=30, seed=4, pset={})
    o = run_oracle(case, meta)
    s, ps = _solver(case, p, precision, sort_period, seed=4)
    s.forward(nsteps=30)
    if precision == "fp64":
        want = dict(position=o.pos, tri=o.tri, inactive=o.inactive)
        assert_state_close(dict(position=ps.position, tri=ps.tri, inactive=ps.inactive), want,
                           rtol=RTOL, what=f"n={n}")
        np.testing.assert_array_equal(ps.tag, o.tag)
    else:
        both = (ps.inactive == 0) & (o.inactive == 0)
        assert (ps.inactive != o.inactive).sum() <= max(1, n // 100)
        assert (ps.tri[both] == o.tri[both]).mean() >= 0.95
        same = both & (ps.tri == o.tri)
        if same.any():
            assert np.abs(ps.position[same] - o.pos[same]).max() < 1e-3
    s.close()


@pytest.mark.parametrize("sort_period", [0, 25])
def test_pool_empties_then_keeps_stepping(sort_period):
    """Open boundaries, stranding and damped rebounds (the reference's open
    channel case) for 600 steps: every particle exits or strands, with the
    reference's deletion order (tags) and exit counts; 100 more steps on the
    all-inactive pool change nothing."""
    case, meta, _ = load_golden("open")
    meta = dict(meta, params=dict(meta["params"], final_time=1400.0))
    o = run_oracle(case, meta, nsteps=600)
    assert (o.inactive == 1).all()
    s, ps = _solver(case, meta["params"], "fp64", sort_period, seed=meta["seed"])
    s.forward(nsteps=600)
    want = dict(position=o.pos, tri=o.tri, inactive=o.inactive)
    assert_state_close(dict(position=ps.position, tri=ps.tri, inactive=ps.inactive), want,
                       rtol=RTOL, what="open x600")
    np.testing.assert_array_equal(ps.tag, o.tag)
    np.testing.assert_array_equal(s.bnd_statistics(), np.stack(o.bnd_stats))
    before = (ps.position.copy(), ps.tri.copy(), ps.tag.copy())
    s.forward(nsteps=100)
    assert not s.bnd_statistics()[600:].any()
    np.testing.assert_array_equal(ps.position, before[0])
    np.testing.assert_array_equal(ps.tri, before[1])
    np.testing.assert_array_equal(ps.tag, before[2])
    s.close()
