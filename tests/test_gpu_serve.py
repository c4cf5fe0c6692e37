"""The serving pool: many runs stepped together, each result the same as
the run alone.

* a run served in a mix of others (admitted at other steps, other models,
  other sizes) gives exactly the state it gives alone in the pool, in both
  forms;
* in the plain form that state is the standalone Solver's (element indices
  and tags bit-exact, positions and velocities within 1e-10 relative);
* admission is by memory: a run that does not fit waits until a release
  frees a range, and a cancelled run leaves the others untouched.
"""
import numpy as np
import pytest

from conftest import RTOL, assert_state_close

pytestmark = pytest.mark.gpu


def _channel():
    import cylag_gb300 as cg
    from cylag_gb300 import synth
    from cylag_gb300.mesh import TriangularMesh
    c = synth.couette_channel(npart=10)
    mesh = TriangularMesh(c["x"], c["y"], c["triangles"])
    return cg.EulerianFieldSet(mesh, dim=2, nlayers=1, times=c["times"],
                               elevation=c["elevation"], velocity_x=c["velocity_x"],
                               velocity_y=c["velocity_y"])


def _requests():
    from cylag_gb300.serve import LSM1_PARAMS, LSM2_PARAMS, Request, disc
    out = []
    spec = [(700, 60, 1), (2500, 45, 2), (33, 80, 1), (4096, 30, 2), (1, 50, 1), (1500, 70, 1),
            (900, 55, 2)]
    for k, (n, h, model) in enumerate(spec):
        rng = np.random.default_rng(100 + k)
        pos = disc(rng, n, rng.uniform(100, 900), rng.uniform(10, 90), rng.uniform(5, 50))
        p = dict(LSM1_PARAMS if model == 1 else LSM2_PARAMS, final_time=float(h))
        if k == 5:
            p.update(time_scheme=4, diffusion_model=0)          # LSM1 RK4, no diffusion
        if k == 6:
            p.update(diffusion_lsm2_option=2, horizontal_diffusivity=0.002)  # LSM2 on U
        out.append(Request(k, pos, h, p, seed=1000 + 7 * k))
    return out


def _alone(fs, precision, req):
    from cylag_gb300.serve import DispersionServer
    srv = DispersionServer(fs, precision=precision, capacity=1 << 14, max_runs=8)
    assert srv.admit(req)
    srv.step(req.horizon)
    (res,) = srv.collect()
    srv.close()
    return res


def _mix(fs, precision, reqs):
    """Admissions staggered over the steps; results by request id."""
    from cylag_gb300.serve import DispersionServer
    srv = DispersionServer(fs, precision=precision, capacity=1 << 15, max_runs=16)
    done = {}
    waiting = list(reqs)
    while waiting or srv.runs:
        if waiting and srv.admit(waiting[0]):   # one admission per few steps
            waiting.pop(0)
        left = [srv.steps_left(r) for r in srv.runs]
        todo = [x for x in left if x > 0]
        if todo:
            srv.step(min(5, min(todo)))
        for r in srv.collect():
            done[r.rid] = r
    srv.close()
    return done


def _state(r):
    return dict(position=r.position, velocity=r.velocity, fluid_velocity_seen=r.fluid_velocity_seen,
                tri=r.tri, inactive=r.inactive)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_same_alone_and_in_the_mix(precision):
    fs = _channel()
    reqs = _requests()
    mix = _mix(fs, precision, reqs)
    assert sorted(mix) == [r.rid for r in reqs]
    for req in reqs:
        alone = _alone(fs, precision, req)
        assert_state_close(_state(mix[req.rid]), _state(alone), rtol=0.0, exact=True,
                           what=f"{precision} request {req.rid}")
        np.testing.assert_array_equal(mix[req.rid].tag, alone.tag)


def test_served_run_equals_standalone_solver():
    """Plain form: each served run is the standalone Solver's run."""
    import cylag_gb300 as cg
    fs = _channel()
    reqs = _requests()
    mix = _mix(fs, "fp64", reqs)
    for req in reqs:
        ps = cg.LagrangianParticleSet(req.position, dim=2)
        s = cg.Solver(fs, ps, req.parameters, precision="fp64", seed=req.seed, sort_period=0)
        s.forward(nsteps=req.horizon)
        want = dict(position=ps.position, velocity=ps.velocity,
                    fluid_velocity_seen=ps.fluid_velocity_seen, tri=ps.tri, inactive=ps.inactive)
        assert_state_close(_state(mix[req.rid]), want, rtol=RTOL, what=f"request {req.rid}")
        np.testing.assert_array_equal(mix[req.rid].tag, ps.tag)
        s.close()


def test_admission_waits_for_memory_and_cancel_is_isolated():
    from cylag_gb300.serve import DispersionServer
    fs = _channel()
    reqs = _requests()
    big, small = reqs[3], reqs[0]          # 4096 and 700 particles
    srv = DispersionServer(fs, precision="fp64", capacity=4096 + 32 * 10, max_runs=4)
    assert srv.admit(small)
    assert not srv.admit(big)               # 4096 + 704 > pool
    srv.step(10)
    (run_small,) = srv.runs
    assert srv.steps_left(run_small) == small.horizon - 10
    # cancel the small run: the big one now fits and is unaffected
    srv.cancel(run_small)
    assert srv.admit(big)
    srv.step(big.horizon)
    (r_big,) = srv.collect()
    srv.close()
    alone = _alone(fs, "fp64", big)
    assert_state_close(_state(r_big), _state(alone), rtol=0.0, exact=True, what="after cancel")


def test_serve_schedule_runs_every_request():
    """A short Poisson schedule (time-compressed): every request completes,
    latencies are positive, and a request's result does not depend on the
    schedule (spot check against the run alone)."""
    from cylag_gb300.serve import DispersionServer, poisson_mix
    fs = _channel()
    reqs = poisson_mix(rate=50.0, duration=0.5, seed=3, nmax=2e4, hmax=300)
    srv = DispersionServer(fs, precision="mixed", capacity=1 << 17, max_runs=64)
    res = srv.serve(reqs, realtime=True, chunk=16)
    srv.close()
    assert sorted(r.rid for r in res) == [r.rid for r in reqs]
    assert all(r.latency > 0 for r in res)
    by = {r.rid: r for r in res}
    for req in reqs[:3]:
        alone = _alone(fs, "mixed", req)
        assert_state_close(_state(by[req.rid]), _state(alone), rtol=0.0, exact=True,
                           what=f"schedule request {req.rid}")


def test_watchdog_cancels_a_run_past_its_deadline_and_leaves_the_others():
    """On the device pool: a request with a zero deadline is cancelled by
    the watchdog at the first loop after its admission (an error result, no
    state); the other runs of the mix give exactly their results alone."""
    import dataclasses
    from cylag_gb300.serve import DispersionServer
    fs = _channel()
    reqs = _requests()[:4]
    reqs[1] = dataclasses.replace(reqs[1], deadline=0.0)
    srv = DispersionServer(fs, precision="mixed", capacity=1 << 15, max_runs=16)
    res = {r.rid: r for r in srv.serve(reqs, realtime=False, chunk=8)}
    srv.close()
    assert sorted(res) == [0, 1, 2, 3]
    assert res[1].error and len(res[1].position) == 0
    for k in (0, 2, 3):
        assert res[k].error is None
        want = _alone(fs, "mixed", reqs[k])
        np.testing.assert_array_equal(res[k].position, want.position)
        np.testing.assert_array_equal(res[k].tri, want.tri)
