"""Mixed-precision form: stated error against the FP64 oracle and the plain
form, and the analytical 2Kt spread.

Tolerance (the mixed form's contract): ensemble variance of the
displacement within 1e-3 relative of the FP64 result; ensemble mean within
1e-3 of the spread; element decisions identical to the FP64 predicate.
"""
import numpy as np
import pytest

from conftest import load_golden, run_oracle
from test_gpu_parity import gpu_run

pytestmark = pytest.mark.gpu

VAR_TOL = 1e-3


def keps_case(npart, nx=101, ny=26, seed=5):
    from cylag_gb300 import synth
    c = synth.keps_drift_channel(npart=npart, nx=nx, ny=ny, seed=seed)
    case = {k: c[k] for k in ("x", "y", "triangles", "times", "elevation", "velocity_x",
                              "velocity_y", "opt_fields", "position")}
    case["opt_fields_names"] = c["opt_fields_names"]
    p = dict(c["parameters"])
    p.update(time_step=2.0, final_time=400.0)
    return case, p


def test_mixed_vs_fp64_oracle_keps():
    from cylag_gb300.stats import displacement_report
    case, p = keps_case(50_000)
    meta = dict(params=p, nsteps=150, seed=11, pset={})
    o = run_oracle(case, meta, nthreads=8)
    s, ps = gpu_run(case, meta, precision="mixed")
    act = (o.inactive == 0) & (ps.inactive == 0)
    rep = displacement_report(case["position"], ps.position, o.pos, act)
    print(rep)
    assert max(rep["var_rel_err"]) <= VAR_TOL, rep
    assert max(rep["mean_rel_err"]) <= VAR_TOL, rep
    # same per-particle streams: trajectories stay close particle by particle
    assert rep["rms_displacement_diff"] < 1e-2 * np.sqrt(max(rep["var_ref"])), rep
    s.close()


@pytest.mark.parametrize("diffusion_model", [0, 1, 2])
@pytest.mark.parametrize("rng_method", [1, 2, 3])
def test_mixed_configuration_forms_vs_fp64_oracle(diffusion_model, rng_method):
    """The element-sorted Euler steps without per-call outputs run a kernel
    compiled for the run's diffusion (none, constant, k-epsilon) and random
    number method; each of the nine against the FP64 oracle, 60 steps of
    20,000 particles in one call: ensemble variance and mean within the
    mixed form's tolerance, per-particle trajectories close."""
    from cylag_gb300.stats import displacement_report
    case, p = keps_case(20_000)
    p = dict(p, diffusion_model=diffusion_model, rng_method=rng_method,
             horizontal_diffusivity=0.05)
    meta = dict(params=p, nsteps=60, seed=7, pset={})
    o = run_oracle(case, meta, nthreads=8)
    s, ps = gpu_run(case, meta, precision="mixed")
    act = (o.inactive == 0) & (ps.inactive == 0)
    assert (o.inactive != ps.inactive).sum() <= 5
    rep = displacement_report(case["position"], ps.position, o.pos, act)
    assert max(rep["var_rel_err"]) <= VAR_TOL, rep
    assert max(rep["mean_rel_err"]) <= VAR_TOL, rep
    assert rep["rms_displacement_diff"] < 1e-2 * np.sqrt(max(rep["var_ref"])), rep
    s.close()


def test_mixed_vs_plain_same_decisions():
    """From identical positions one mixed step and one plain step give the
    same element indices when the displacement is identical (zero
    diffusion, frozen uniform flow)."""
    name = "couette"
    case, meta, _ = load_golden(name)
    meta = dict(meta)
    meta["params"] = dict(meta["params"], diffusion_model=0, time_scheme=1)
    sa, pa = gpu_run(case, meta, nsteps=50, precision="fp64")
    sb, pb = gpu_run(case, meta, nsteps=50, precision="mixed")
    np.testing.assert_array_equal(pa.tri, pb.tri)
    assert np.max(np.abs(pa.position - pb.position)) < 1e-5
    sa.close()
    sb.close()


def test_mixed_pure_diffusion_matches_2Kt():
    """Zero velocity, constant K: the spread of 200,000 particles after t
    seconds is 2Kt within 5 standard errors (walls far away)."""
    from cylag_gb300 import synth
    from cylag_gb300.stats import diffusion_report
    x, y, tri = synth.channel_mesh(2000.0, 2000.0, 41, 41, seed=2)
    n = 200_000
    pos = np.tile([[1000.0, 1000.0]], (n, 1))
    case = dict(x=x, y=y, triangles=tri, times=np.zeros(1), elevation=np.ones((1, len(x))),
                velocity_x=np.zeros((1, len(x))), velocity_y=np.zeros((1, len(x))), position=pos)
    K, dt, nsteps = 0.5, 1.0, 200
    p = dict(model=1, diffusion_model=1, horizontal_diffusivity=K, time_scheme=1,
             frozen_eulerian_fields=True, time_step=dt, final_time=dt * nsteps)
    for prec in ("mixed", "fp64"):
        s, ps = gpu_run(case, dict(params=p, nsteps=nsteps, seed=1, pset={}), precision=prec)
        rep = diffusion_report(pos, ps.position, K, dt * nsteps)
        print(prec, rep)
        assert max(abs(z) for z in rep["z"]) < 5.0, (prec, rep)
        s.close()


def test_split_working_positions_follow_fp64_positions():
    """Mixed LSM1 2D over sorted working copies keeps positions as FP32
    pairs hi + lo; without the sort (sort_period=0) the same run keeps FP64
    positions.  Same streams and decisions: element indices agree for all
    but a handful of near-edge particles, positions to 1e-4 m after 150
    steps (coordinates up to 4 km)."""
    case, p = keps_case(40_000)
    meta = dict(params=p, nsteps=150, seed=3, pset={})
    import cylag_gb300 as cg
    from conftest import fields_from_case, mesh_from_case
    out = {}
    for sp in (0, 10):
        f = fields_from_case(case)
        fs = cg.EulerianFieldSet(mesh_from_case(case), **f)
        ps = cg.LagrangianParticleSet(case["position"], dim=2)
        s = cg.Solver(fs, ps, p, precision="mixed", seed=3, sort_period=sp)
        s.forward(nsteps=150)
        out[sp] = (ps.position, ps.tri, ps.inactive)
        s.close()
    (pa, ta, ia), (pb, tb, ib) = out[0], out[10]
    both = (ia == 0) & (ib == 0)
    assert (ia != ib).sum() <= 5
    assert (ta[both] != tb[both]).sum() <= max(5, int(1e-3 * both.sum()))
    same = both & (ta == tb)
    assert np.max(np.abs(pa[same] - pb[same])) < 1e-4


@pytest.mark.parametrize("model", [2, 3])
def test_split3_working_positions_follow_fp64_positions(model):
    """Mixed LSM2/LSM3 3D direct integrators over sorted working copies keep
    positions as FP32 pairs hi + lo per coordinate and FP32 velocities;
    without the sort (sort_period=0) the same run keeps FP64 positions.  Same
    streams: element and layer indices agree for all but a handful of
    particles, positions to 1e-5 m and velocities to 1e-4 of their spread
    after 60 steps for all but 1% of them.  Those are particles whose bed
    reflection the two FP32 layer tests (FP32 heights against FP32 bed
    elevations, about 1e-6 m apart between the two position forms) decide
    differently near the bed; they move apart by a few velocity-steps, under
    0.05 m here."""
    import cylag_gb300 as cg
    from cylag_gb300 import synth
    from cylag_gb300.mesh import TriangularMesh
    if model == 2:
        c = synth.lsm2_loglaw_workload(npart=30_000, nx=41, ny=21, nplanes=6, seed=3)
    else:
        c = synth.lsm3_taylor_green_workload(npart=30_000, nx=41, ny=21, nplanes=6, seed=3)
    p = dict(c["parameters"], final_time=1e6)
    out = {}
    for sp in (0, 10):
        mesh = TriangularMesh(c["x"], c["y"], c["triangles"])
        fs = cg.EulerianFieldSet(mesh, dim=3, nlayers=c["nlayers"], times=c["times"],
                                 elevation=c["elevation"], velocity_x=c["velocity_x"],
                                 velocity_y=c["velocity_y"], velocity_z=c["velocity_z"],
                                 opt_fields=c.get("opt_fields"),
                                 opt_fields_names=c.get("opt_fields_names"))
        ps = cg.LagrangianParticleSet(c["position"], dim=3, **c.get("pset", {}))
        if "diameter" in c:
            ps.diameter = c["diameter"]
        s = cg.Solver(fs, ps, p, precision="mixed", seed=3, sort_period=sp)
        s.forward(nsteps=60)
        out[sp] = (ps.position, ps.tri, ps.lowerlayer, ps.inactive, ps.velocity)
        s.close()
    (pa, ta, la, ia, va), (pb, tb, lb, ib, vb) = out[0], out[10]
    both = (ia == 0) & (ib == 0)
    assert both.sum() > 0.5 * len(ia)
    assert (ia != ib).sum() <= max(5, int(1e-3 * len(ia)))
    same = both & (ta == tb) & (la == lb)
    assert (~same & both).sum() <= max(5, int(1e-3 * both.sum()))
    few = max(5, int(1e-2 * same.sum()))
    dpos = np.max(np.abs(pa[same] - pb[same]), axis=1)
    assert (dpos > 1e-5).sum() <= few and dpos.max() < 0.05, np.sort(dpos)[-10:]
    spread = np.std(va[both], axis=0)
    dvel = np.max(np.abs(va[same] - vb[same]) / spread, axis=1)
    assert (dvel > 1e-4).sum() <= few, np.sort(dvel)[-10:]


@pytest.mark.parametrize("sort_period", [0, 20])
@pytest.mark.parametrize("name", ["keps_ts1_rm2", "keps_ts2_rm1", "keps_ts3_rm3", "keps_ts4_rm2"])
def test_mixed_time_schemes_follow_reference(name, sort_period):
    """The mixed form through each LSM1 time scheme (Euler, RK2, RK3, RK4)
    and RNG method, k-eps drift on time-interpolated fields, against the
    compiled reference's trajectories: unsorted (FP64 working positions)
    and element-sorted (split positions) kernels.  Same streams and
    decisions, FP32 increments: element indices agree and positions stay
    within 1e-3 m over 80 steps of 5 s."""
    import cylag_gb300 as cg
    from conftest import fields_from_case, mesh_from_case
    case, meta, want = load_golden(name)
    f = fields_from_case(case)
    fs = cg.EulerianFieldSet(mesh_from_case(case), **f)
    ps = cg.LagrangianParticleSet(case["position"], dim=2, **meta.get("pset", {}))
    s = cg.Solver(fs, ps, meta["params"], precision="mixed", seed=meta["seed"],
                  sort_period=sort_period)
    s.forward(nsteps=meta["nsteps"])
    both = (ps.inactive == 0) & (want["inactive"] == 0)
    assert (ps.inactive != want["inactive"]).sum() <= 1
    assert (ps.tri[both] == want["tri"][both]).mean() >= 0.95
    same = both & (ps.tri == want["tri"])
    err = np.abs(ps.position[same] - want["position"][same]).max()
    assert err < 1e-3, err
    s.close()
