"""The GPU step against the oracle on the benchmarked configurations at their
full mesh sizes.

* config 1 exactly: the Couette channel (2,000 triangles), 10,000 particles,
  1,000 steps of 1 s, every particle checked;
* config 2: LSM1 k-epsilon drift on the 4 km x 1 km jittered mesh (1001x251
  vertices, 5e5 triangles), field records A, B, A 600 s apart;
* config 3: LSM2 direct integrator with k-epsilon velocity diffusion on the
  3D log-law channel (501x201 jittered vertices, 2e5 triangles, 21 sigma
  planes);
* config 4: LSM3 polydisperse settling in the Taylor-Green vortex on the
  same 3D mesh.

Configs 2-4 run 1e6 particles on the GPU and the oracle on a tag subsample
of 50,000 of them (every 20th) for 100 steps: particle t draws from
pcg32_seed(seed, t) on both sides, so the subsample is an exact check on
those particles.  Plain form: element and layer indices, active flags, the
tags of particles still active and the final PCG32 states bit-exact;
positions, velocities and fluid velocities seen within 1e-10 relative.
Mixed form (same particles): ensemble mean and variance of the displacement
(and, for LSM2/LSM3, of the velocity) within 1e-3 of the oracle's.
"""
import numpy as np
import pytest

from conftest import RTOL, assert_state_close

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-3
NGPU = 1_000_000
EVERY = 20


def _fields(c):
    return dict(dim=c.get("dim", 2), nlayers=c.get("nlayers", 1), times=c["times"],
                elevation=c["elevation"], velocity_x=c["velocity_x"],
                velocity_y=c["velocity_y"], velocity_z=c.get("velocity_z"),
                opt_fields=c.get("opt_fields"), opt_fields_names=c.get("opt_fields_names"))


def _config(name):
    from cylag_gb300 import synth
    if name == "cfg1_couette":
        c = synth.couette_channel(npart=10_000)
        c.update(dim=2, nlayers=1)
        return c, dict(c["parameters"]), 1000, 1
    if name == "cfg2_keps_drift":
        c = synth.keps_drift_channel(npart=NGPU)
        c.update(dim=2, nlayers=1)
        return c, dict(c["parameters"]), 100, EVERY
    if name == "cfg3_lsm2_loglaw":
        c = synth.lsm2_loglaw_workload(npart=NGPU)
        return c, dict(c["parameters"]), 100, EVERY
    c = synth.lsm3_taylor_green_workload(npart=NGPU)
    return c, dict(c["parameters"]), 100, EVERY


_CACHE = {}


def _case(name):
    """(case, params, nsteps, subsample indices, oracle result) per config,
    built once per session."""
    if name in _CACHE:
        return _CACHE[name]
    import oracle
    from cylag_gb300.mesh import TriangularMesh
    c, p, nsteps, every = _config(name)
    n = len(c["position"])
    idx = np.arange(0, n, every)
    mesh = TriangularMesh(c["x"], c["y"], c["triangles"])
    diam = c["diameter"][idx] if "diameter" in c else None
    o = oracle.OracleSolver(mesh, _fields(c), p, c["position"][idx], pset=c.get("pset"),
                            seed=0, tags=idx, nthreads=16, diameter=diam)
    o.solve(nsteps)
    want = dict(position=o.pos.copy(), velocity=o.vel.copy(), fluid_velocity_seen=o.fvs.copy(),
                tri=o.tri.copy(), inactive=o.inactive.copy(), lowerlayer=o.lowerlayer.copy(),
                tag=o.tag.copy(), rng_state=np.asarray(o.rng_state).view(np.uint64).copy())
    _CACHE[name] = (c, p, nsteps, idx, mesh, want)
    return _CACHE[name]


def _gpu(c, p, mesh, nsteps, precision):
    import cylag_gb300 as cg
    fs = cg.EulerianFieldSet(mesh, **_fields(c))
    ps = cg.LagrangianParticleSet(c["position"], dim=c.get("dim", 2), **c.get("pset", {}))
    if "diameter" in c:
        ps.diameter = c["diameter"]
    s = cg.Solver(fs, ps, p, precision=precision, seed=0, sort_period=25)
    s.forward(nsteps=nsteps)
    ps._sync()
    out = dict(position=ps.position, velocity=ps.velocity,
               fluid_velocity_seen=ps.fluid_velocity_seen, tri=ps.tri, inactive=ps.inactive,
               lowerlayer=ps.lowerlayer, tag=ps.tag,
               rng_state=ps._dev["rng_state"].cpu().numpy().view(np.uint64))
    s.close()
    return out


CONFIGS = ["cfg1_couette", "cfg2_keps_drift", "cfg3_lsm2_loglaw", "cfg4_lsm3_settling"]


@pytest.mark.parametrize("name", CONFIGS)
def test_plain_matches_oracle_at_config_size(name):
    c, p, nsteps, idx, mesh, want = _case(name)
    got = {k: np.asarray(v)[idx] for k, v in _gpu(c, p, mesh, nsteps, "fp64").items()}
    assert_state_close(got, want, rtol=RTOL, what=name)
    np.testing.assert_array_equal(got["rng_state"], want["rng_state"],
                                  err_msg=f"{name}: PCG32 states")
    active = want["inactive"] == 0
    np.testing.assert_array_equal(got["tag"][active], want["tag"][active],
                                  err_msg=f"{name}: tags of active particles")
    assert active.sum() > 0.9 * len(idx)


@pytest.mark.parametrize("name", CONFIGS)
def test_mixed_statistics_match_oracle_at_config_size(name):
    from cylag_gb300.stats import displacement_report
    c, p, nsteps, idx, mesh, want = _case(name)
    got = {k: np.asarray(v)[idx] for k, v in _gpu(c, p, mesh, nsteps, "mixed").items()}
    act = (got["inactive"] == 0) & (want["inactive"] == 0)
    assert (got["inactive"] != want["inactive"]).sum() <= max(2, int(1e-4 * len(idx)))
    rep = displacement_report(c["position"][idx], got["position"], want["position"], act)
    assert max(rep["var_rel_err"]) <= MIXED_TOL, rep
    assert max(rep["mean_rel_err"]) <= MIXED_TOL, rep
    if p["model"] >= 2:
        va, vb = got["velocity"][act], want["velocity"][act]
        verr = np.abs(va.var(0) - vb.var(0)) / np.maximum(vb.var(0), 1e-300)
        assert verr.max() <= MIXED_TOL, verr
    # same streams and decisions: indices agree for nearly every particle
    assert (got["tri"][act] == want["tri"][act]).mean() >= 0.999
