"""The allocation-free step entry point (cg_run_step_noalloc).

Some callers cannot allocate device memory while they step -- code under a
framework's memory pool that owns all device memory, real-time loops that
must not block in the allocator, hosts that cap device memory at start-up.
For them the library has one entry point whose scratch (the queue of
particles leaving their triangle) is a fixed device array inside the
library instead of cudaMalloc'd memory.

This test calls it through the C ABI and checks, on two calls in a row,
that it leaves the particle state exactly where the regular entry point
(cg_run_step) leaves it: element indices and deletions identical, positions
and velocities within the tolerance of the parity tests.  It also checks
that runs larger than the array are refused with a clear error.  Collected
last (file name) so that a failure here does not hide any other result.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import RTOL, assert_state_close

pytestmark = pytest.mark.gpu


def _case(npart):
    from cylag_gb300 import synth
    c = synth.keps_drift_channel(npart=npart, nx=101, ny=26, seed=9)
    case = {k: c[k] for k in ("x", "y", "triangles", "times", "elevation", "velocity_x",
                              "velocity_y", "opt_fields", "position")}
    case["opt_fields_names"] = c["opt_fields_names"]
    p = dict(c["parameters"])
    p.update(time_step=2.0, final_time=400.0)
    return case, p


def _solver(case, p, precision):
    import cylag_gb300 as cg
    from conftest import fields_from_case, mesh_from_case
    f = fields_from_case(case)
    fs = cg.EulerianFieldSet(mesh_from_case(case), dim=2, nlayers=1, times=f["times"],
                             elevation=f["elevation"], velocity_x=f["velocity_x"],
                             velocity_y=f["velocity_y"], opt_fields=f["opt_fields"],
                             opt_fields_names=f["opt_fields_names"])
    ps = cg.LagrangianParticleSet(case["position"], dim=2)
    return cg.Solver(fs, ps, p, precision=precision, seed=4, sort_period=0), ps


def _state(ps):
    return dict(position=ps.position, velocity=ps.velocity, tri=ps.tri, inactive=ps.inactive,
                last_position=ps.last_position)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_noalloc_step_matches_cg_run_step(precision):
    from cylag_gb300 import _lib
    case, p = _case(30_000)
    sa, pa = _solver(case, p, precision)
    sb, pb = _solver(case, p, precision)
    L = _lib.load()
    for call in range(2):
        sa.forward(nsteps=40)                       # existing entry point
        rc = L.cg_run_step_noalloc(sb._run, 40)     # allocation-free entry point
        _lib.check(sb._ctx, rc)
        want = _state(pa)
        assert_state_close(_state(pb), want, rtol=RTOL, what=f"{precision} call {call + 1}")
        np.testing.assert_array_equal(pb.tag, pa.tag)
    sa.close()
    sb.close()


def test_noalloc_refuses_runs_beyond_its_scratch():
    from cylag_gb300 import _lib
    n = _lib.CG_NOALLOC_MAX_PARTICLES + 1
    case, p = _case(n)
    s, ps = _solver(case, p, "mixed")
    L = _lib.load()
    rc = L.cg_run_step_noalloc(s._run, 1)
    assert rc == _lib.CG_EINVAL
    buf = C.create_string_buffer(512)
    L.cg_last_error(s._ctx, buf, 512)
    assert b"at most" in buf.value and str(_lib.CG_NOALLOC_MAX_PARTICLES).encode() in buf.value
    # the refused call changed nothing: the regular entry point still works
    s.forward(nsteps=1)
    s.close()
