"""LSM2 and LSM3 on the GPU at sizes beyond the golden fixtures, against the
oracle run on the same inputs.

Plain form: element and layer indices and deletions bit-exact, positions,
velocities and fluid velocities seen within 1e-10 relative.  Mixed form
(FP32 node records, FP64 state): ensemble statistics within 1e-3 relative
of the oracle's.
"""
import numpy as np
import pytest

from conftest import RTOL, assert_state_close

pytestmark = pytest.mark.gpu


def _fields(c):
    return dict(dim=c["dim"], nlayers=c["nlayers"], times=c["times"], elevation=c["elevation"],
                velocity_x=c["velocity_x"], velocity_y=c["velocity_y"],
                velocity_z=c.get("velocity_z"), opt_fields=c.get("opt_fields"),
                opt_fields_names=c.get("opt_fields_names"))


def _run_gpu(c, params, nsteps, precision="fp64", seed=0, sort_period=25, batch=None):
    import cylag_gb300 as cg
    from cylag_gb300.mesh import TriangularMesh
    mesh = TriangularMesh(c["x"], c["y"], c["triangles"])
    fs = cg.EulerianFieldSet(mesh, **_fields(c))
    ps = cg.LagrangianParticleSet(c["position"], dim=c["dim"], **c.get("pset", {}))
    if "diameter" in c:
        ps.diameter = c["diameter"]
    s = cg.Solver(fs, ps, params, precision=precision, seed=seed, sort_period=sort_period)
    if batch is None:
        s.forward(nsteps=nsteps)
    else:
        for _ in range(nsteps // batch):
            s.forward(nsteps=batch)
    out = dict(position=ps.position, velocity=ps.velocity,
               fluid_velocity_seen=ps.fluid_velocity_seen, tri=ps.tri, inactive=ps.inactive,
               lowerlayer=ps.lowerlayer, last_position=ps.last_position, tag=ps.tag)
    s.close()
    return out


def _run_oracle(c, params, nsteps, seed=0):
    import oracle
    from cylag_gb300.mesh import TriangularMesh
    mesh = TriangularMesh(c["x"], c["y"], c["triangles"])
    o = oracle.OracleSolver(mesh, _fields(c), params, c["position"], pset=c.get("pset"),
                            seed=seed, nthreads=8, diameter=c.get("diameter"))
    o.solve(nsteps)
    return dict(position=o.pos, velocity=o.vel, fluid_velocity_seen=o.fvs, tri=o.tri,
                inactive=o.inactive, lowerlayer=o.lowerlayer, last_position=o.last_pos,
                tag=o.tag)


def _lsm2_3d(npart):
    from cylag_gb300 import synth
    c = synth.lsm2_loglaw_workload(npart=npart, nx=81, ny=41, nplanes=11, seed=2)
    return c, dict(c["parameters"], final_time=1e6)


def _lsm3_3d(npart):
    from cylag_gb300 import synth
    c = synth.lsm3_taylor_green_workload(npart=npart, nx=81, ny=41, nplanes=11, seed=4)
    return c, dict(c["parameters"], final_time=1e6)


def _lsm2_2d(npart, **over):
    from cylag_gb300 import synth
    c = synth.keps_drift_channel(npart=npart, nx=101, ny=26, seed=6)
    c.update(dim=2, nlayers=1, pset={"added_mass_force": True})
    p = dict(c["parameters"], model=2, time_scheme=5, diffusion_lsm2_option=2,
             time_step=1.0, final_time=1000.0)
    p.update(over)
    return c, p


@pytest.mark.parametrize("make", [_lsm2_3d, _lsm3_3d], ids=["lsm2_3d_di_keps", "lsm3_3d_di_settling"])
def test_plain_3d_matches_oracle(make):
    c, p = make(6000)
    want = _run_oracle(c, p, 80)
    got = _run_gpu(c, p, 80)
    assert_state_close(got, want, rtol=RTOL, what=make.__name__)
    np.testing.assert_array_equal(got["tag"], want["tag"])


@pytest.mark.parametrize("over", [dict(), dict(time_scheme=1, diffusion_lsm2_option=3,
                                               time_step=0.25),
                                  dict(diffusion_model=0, time_scheme=4, time_step=2.0)],
                         ids=["di_opt2", "em_opt3", "rk4_nodiff"])
def test_plain_2d_lsm2_sorted_matches_oracle(over):
    """20,000 particles, 100 steps in one call: the element-sorted working
    state (re-sorted every 25 steps) carries LSM2's velocities through the
    slot indirection; results equal the unsorted oracle's."""
    c, p = _lsm2_2d(20000, **over)
    if p["time_scheme"] == 1:
        c["pset"] = dict(c["pset"], drag_coefficient_model=0, drag_coefficient=0.01)
    want = _run_oracle(c, p, 100)
    got = _run_gpu(c, p, 100, sort_period=25)
    assert_state_close(got, want, rtol=RTOL, what=str(over))
    np.testing.assert_array_equal(got["tag"], want["tag"])


def test_plain_lsm3_2d_stepwise_equals_batched():
    """LSM3 (2D, k-epsilon, added mass): 60 one-step calls and one 60-step
    call give the same state."""
    c, p = _lsm2_2d(3000, model=3, diffusion_model=2, time_scheme=5)
    a = _run_gpu(c, p, 60, batch=1)
    b = _run_gpu(c, p, 60)
    assert_state_close(a, b, rtol=0.0, exact=True, what="lsm3 stepwise")


@pytest.mark.parametrize("make", [_lsm2_3d, _lsm3_3d], ids=["lsm2_3d_di_keps", "lsm3_3d_di_settling"])
def test_mixed_3d_statistics(make):
    """FP32 node records: ensemble mean and variance of the displacement and
    of the velocity within 1e-3 relative of the FP64 oracle's."""
    c, p = make(20000)
    want = _run_oracle(c, p, 60)
    got = _run_gpu(c, p, 60, precision="mixed")
    act = (want["inactive"] == 0) & (got["inactive"] == 0)
    assert act.mean() > 0.95
    x0 = c["position"][act]
    for k in ("position", "velocity"):
        ga, wa = got[k][act], want[k][act]
        if k == "position":
            ga, wa = ga - x0, wa - x0
        dv = np.abs(ga.var(0) - wa.var(0)) / wa.var(0)
        assert dv.max() < 1e-3, (k, dv)
        dm = np.abs(ga.mean(0) - wa.mean(0)) / np.sqrt(wa.var(0))
        assert dm.max() < 1e-3, (k, dm)


def _form_case(kind):
    """Configurations that select the other compiled forms of the element-
    sorted mixed 3D step (drag law, diffusion, edge option, added mass)."""
    if kind.startswith("lsm3"):
        c, p = _lsm3_3d(20000)
        pset = dict(c.get("pset", {}))
        if kind == "lsm3_drag0_edge1":
            pset["drag_coefficient_model"] = 0
            p = dict(p, lsm3_edge_opt=1)
        elif kind == "lsm3_added_mass":
            pset["added_mass_force"] = True
        elif kind == "lsm3_keps":
            c, p = _lsm2_3d(20000)
            p = dict(p, model=3, diffusion_model=2)
            pset = dict(c.get("pset", {}))
        c = dict(c, pset=pset)
        return c, p
    c, p = _lsm2_3d(20000)
    pset = dict(c.get("pset", {}))
    if kind == "lsm2_const_drag0":
        p = dict(p, diffusion_model=1, horizontal_diffusivity=0.01, vertical_diffusivity=1e-3)
        pset["drag_coefficient_model"] = 0
    elif kind == "lsm2_keps2_added_mass":
        p = dict(p, diffusion_model=2)
        pset["added_mass_force"] = True
    elif kind == "lsm2_keps3_drag0":
        pset["drag_coefficient_model"] = 0
    return dict(c, pset=pset), p


@pytest.mark.parametrize("kind", ["lsm3_drag0_edge1", "lsm3_added_mass", "lsm3_keps",
                                  "lsm2_const_drag0", "lsm2_keps2_added_mass",
                                  "lsm2_keps3_drag0"])
def test_mixed_3d_forms_statistics(kind):
    """The element-sorted mixed 3D direct integrators step with a kernel
    compiled for the run's configuration; configurations other than the
    bench workloads' against the FP64 oracle.  A few trajectories part
    where an FP32 decision (a sampler's wedge test, a wall or bed
    crossing) goes the other way: at most 0.5% of the particles end more
    than 1 mm from the oracle's (about 0.2% in the k-epsilon LSM3 case,
    with the general kernel as with the form); over the others, the
    ensemble mean and variance of the displacement and of the velocity
    agree within 1e-3 relative.  A component that the oracle keeps exactly
    constant (no vertical forcing, neutrally buoyant particles) stays within
    1e-6 of it (m, m/s)."""
    c, p = _form_case(kind)
    want = _run_oracle(c, p, 60)
    got = _run_gpu(c, p, 60, precision="mixed")
    act = (want["inactive"] == 0) & (got["inactive"] == 0)
    assert act.mean() > 0.95
    apart = np.abs(got["position"] - want["position"]).max(1) > 1e-3
    assert (act & apart).sum() <= 0.005 * act.sum(), (kind, (act & apart).sum())
    act &= ~apart
    x0 = c["position"][act]
    for k in ("position", "velocity"):
        ga, wa = got[k][act], want[k][act]
        if k == "position":
            ga, wa = ga - x0, wa - x0
        flat = wa.var(0) == 0.
        assert np.abs(ga[:, flat] - wa[:, flat]).max(initial=0.) < 1e-6, (kind, k, flat)
        var = np.where(flat, 1., wa.var(0))
        dv = np.where(flat, 0., np.abs(ga.var(0) - wa.var(0)) / var)
        assert dv.max() < 1e-3, (kind, k, dv)
        dm = np.where(flat, 0., np.abs(ga.mean(0) - wa.mean(0)) / np.sqrt(var))
        assert dm.max() < 1e-3, (kind, k, dm)

