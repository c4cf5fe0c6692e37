"""Particle sources with the GPU step.

* plain form vs the reference's runs with sources (tests/golden/src_*.npz):
  pool size, every entry's element index, tag and deletion bit-exact,
  positions and velocities within 1e-10 relative -- with and without the
  element sort, in one call or in several;
* with diffusion (per-particle streams, pcg32_seed(seed, tag) for an added
  particle), LSM1 and LSM2, 20,000+ particles: GPU vs the oracle given the
  same sources;
* particles added by hand between forward calls;
* the mixed form follows the plain one (same pool, positions to 1e-3 m).
"""
import numpy as np
import pytest

from conftest import (RTOL, assert_state_close, fields_from_case, load_source, make_sources,
                      mesh_from_case, source_names)

pytestmark = pytest.mark.gpu


def _field_set(case):
    import cylag_gb300 as cg
    f = fields_from_case(case)
    return cg.EulerianFieldSet(mesh_from_case(case), dim=f["dim"], nlayers=f["nlayers"],
                               times=f["times"], elevation=f["elevation"],
                               velocity_x=f["velocity_x"], velocity_y=f["velocity_y"],
                               velocity_z=f["velocity_z"], opt_fields=f["opt_fields"],
                               opt_fields_names=f["opt_fields_names"])


def _gpu(case, params, nsteps, spec, pset, precision="fp64", seed=0, sort_period=0,
         batch=None, rng_stream=None):
    import cylag_gb300 as cg
    ps = cg.LagrangianParticleSet(case["position"], dim=case.get("dim", 2), **pset)
    s = cg.Solver(_field_set(case), ps, params, sources=make_sources(spec, rng_stream),
                  precision=precision, seed=seed, sort_period=sort_period)
    done = 0
    while done < nsteps:
        k = nsteps - done if batch is None else min(batch, nsteps - done)
        s.forward(nsteps=k)
        done += k
    out = dict(position=ps.position, velocity=ps.velocity,
               fluid_velocity_seen=ps.fluid_velocity_seen, tri=ps.tri, inactive=ps.inactive,
               lowerlayer=ps.lowerlayer, last_position=ps.last_position, tag=ps.tag,
               last_tri=ps.last_tri, diameter=ps.diameter, npart=ps.npart, maxtag=ps.maxtag)
    s.close()
    return out


def _oracle(case, params, nsteps, spec, pset, seed=0, rng_stream=None):
    import oracle
    o = oracle.OracleSolver(mesh_from_case(case), fields_from_case(case), params,
                            case["position"], pset=pset, seed=seed, nthreads=8,
                            sources=make_sources(spec, rng_stream),
                            initial_pool_size=pset.get("initial_pool_size"),
                            min_pool_size_update=pset.get("min_pool_size_update", 1000))
    o.solve(nsteps)
    return dict(position=o.pos, velocity=o.vel, fluid_velocity_seen=o.fvs, tri=o.tri,
                inactive=o.inactive, lowerlayer=o.lowerlayer, last_position=o.last_pos,
                tag=o.tag, last_tri=o.last_tri, diameter=o.diameter, npart=o.n,
                maxtag=o.maxtag)


def _check(got, want, what, rtol=RTOL):
    assert got["npart"] == int(np.asarray(want["npart"]).reshape(-1)[-1]), what
    assert got["maxtag"] == int(want["maxtag"]), what
    assert_state_close(got, want, rtol=rtol, what=what)
    for k in ("tag", "last_tri", "diameter"):
        np.testing.assert_array_equal(got[k], want[k], err_msg=f"{what}: {k}")


@pytest.mark.parametrize("sort_period,batch", [(0, None), (5, None), (0, 7), (4, 11)])
@pytest.mark.parametrize("name", source_names())
def test_gpu_sources_match_reference(name, sort_period, batch):
    case, meta, want = load_source(name)
    got = _gpu(case, meta["params"], meta["nsteps"], meta["sources"], meta["pset"],
               sort_period=sort_period, batch=batch, rng_stream=meta.get("rng_stream"))
    _check(got, want, f"{name} sort={sort_period} batch={batch}")


def _drift(npart):
    from cylag_gb300 import synth
    c = synth.keps_drift_channel(npart=npart, nx=101, ny=26, seed=9)
    return c


SPEC_2D = [
    dict(scheduler=dict(iteration_delta=3),
         poly=[[500., 200.], [900., 200.], [900., 500.], [500., 500.]],
         kwargs=dict(xy_method=2, xy_density=0.0025)),
    dict(scheduler=dict(time_delta=7.5, ini_time=0.25),
         poly=[[3800., 800.], [4200., 800.], [4200., 1100.], [3800., 1100.]],
         kwargs=dict(grid_res=[10, 6, 1])),
]


@pytest.mark.parametrize("model", [1, 2])
def test_gpu_sources_with_diffusion_match_oracle(model):
    """20,000 particles in a pool of 20,500 growing by 700: LSM1 k-epsilon
    (Euler) or LSM2 (DI, added mass), two sources, 60 steps in batches of 16
    with the element sort every 10 steps."""
    c = _drift(20000)
    p = dict(c["parameters"], final_time=1000.0)
    pset = dict(initial_pool_size=20500, min_pool_size_update=700)
    if model == 2:
        p.update(model=2, time_scheme=5, diffusion_lsm2_option=2, time_step=1.0)
        pset["added_mass_force"] = True
    want = _oracle(c, p, 60, SPEC_2D, pset, seed=13)
    got = _gpu(c, p, 60, SPEC_2D, pset, seed=13, sort_period=10, batch=16)
    _check(got, want, f"model {model}")


def test_gpu_manual_add_between_forward_calls():
    import cylag_gb300 as cg
    import oracle
    c = _drift(3000)
    p = dict(c["parameters"], final_time=1000.0)
    rng = np.random.default_rng(4)
    extra_pos = [np.stack([rng.uniform(0, 4000, m), rng.uniform(0, 1000, m)], 1)
                 for m in (50, 1500, 7)]
    ps = cg.LagrangianParticleSet(c["position"], dim=2, min_pool_size_update=100)
    s = cg.Solver(_field_set(c), ps, p, seed=3)
    o = oracle.OracleSolver(mesh_from_case(c), fields_from_case(c), p, c["position"], seed=3,
                            nthreads=8, min_pool_size_update=100)
    for k, pos in enumerate(extra_pos):
        s.forward(nsteps=5 + k)
        o.solve(5 + k)
        ps.add(pos)
        o.add(pos)
    s.forward(nsteps=6)
    o.solve(6)
    got = dict(position=ps.position, velocity=ps.velocity, fluid_velocity_seen=ps.fluid_velocity_seen,
               tri=ps.tri, inactive=ps.inactive, lowerlayer=ps.lowerlayer,
               last_position=ps.last_position)
    want = dict(position=o.pos, velocity=o.vel, fluid_velocity_seen=o.fvs, tri=o.tri,
                inactive=o.inactive, lowerlayer=o.lowerlayer, last_position=o.last_pos)
    assert ps.npart == o.n
    assert_state_close(got, want, rtol=RTOL, what="manual add")
    np.testing.assert_array_equal(ps.tag, o.tag)
    s.close()


@pytest.mark.parametrize("name", ["open_lsm1_rk4", "field_open_lsm1", "loglaw3d_lsm2_rk4"])
def test_mixed_sources_follow_plain(name):
    case, meta, want = load_source(name)
    got = _gpu(case, meta["params"], meta["nsteps"], meta["sources"], meta["pset"],
               precision="mixed", sort_period=5, rng_stream=meta.get("rng_stream"))
    assert got["npart"] == int(want["npart"][-1])
    both = (got["inactive"] == 0) & (want["inactive"] == 0)
    assert both.sum() >= 0.97 * (want["inactive"] == 0).sum()
    assert (got["tri"][both] == want["tri"][both]).mean() > 0.97
    err = np.abs(got["position"][both] - want["position"][both]).max()
    assert err < 1e-3, err
