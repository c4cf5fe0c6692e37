"""The allocation-free step entry point (cg_run_step_noalloc).

Some callers cannot allocate device memory while they step -- code under a
framework's memory pool that owns all device memory, real-time loops that
must not block in the allocator, hosts that cap device memory at start-up.
For them the library has one entry point whose scratch (the queue of
particles leaving their triangle) is a fixed device array inside the
library instead of cudaMalloc'd memory.

These tests call it through the C ABI and check, on two calls in a row,
that it leaves the particle state exactly where the regular entry point
(cg_run_step) leaves it: element indices and deletions identical, positions
and velocities within the tolerance of the parity tests -- for the 2D LSM1
step (walk queue in the fixed array) and for a 3D LSM2 run (walk inline, no
queue).  They also check that runs larger than the array, and runs with
control sections or stranding output on (which only cg_run_step records),
are refused with a clear error that leaves the run usable.  Collected last
(file name) so that a failure here does not hide any other result.
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
        ms, launches = sb.last_kernel_ms()
        assert ms == 0.0 and launches > 0     # this call's own count, no stale timing
        want = _state(pa)
        assert_state_close(_state(pb), want, rtol=RTOL, what=f"{precision} call {call + 1}")
        np.testing.assert_array_equal(pb.tag, pa.tag)
    sa.close()
    sb.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_noalloc_step_matches_cg_run_step_lsm2_3d(precision):
    """3D LSM2 (direct integrator, k-epsilon velocity diffusion): the path
    without a walk queue.  The FP64 run is element-sorted, so its working
    copies are also written back between the calls; the mixed run is not
    (sorted, the mixed form keeps its positions as FP32 pairs, whose
    arithmetic differs from the FP64 positions the caller's arrays hold)."""
    import cylag_gb300 as cg
    from cylag_gb300 import _lib, synth
    from cylag_gb300.mesh import TriangularMesh
    c = synth.lsm2_loglaw_workload(npart=20_000, nx=41, ny=21, nplanes=6, seed=3)
    p = dict(c["parameters"], final_time=1e6)
    runs = []
    for sort_period in ((10, 0) if precision == "fp64" else (0, 0)):
        mesh = TriangularMesh(c["x"], c["y"], c["triangles"])
        fs = cg.EulerianFieldSet(mesh, dim=3, nlayers=c["nlayers"], times=c["times"],
                                 elevation=c["elevation"], velocity_x=c["velocity_x"],
                                 velocity_y=c["velocity_y"], velocity_z=c["velocity_z"],
                                 opt_fields=c["opt_fields"],
                                 opt_fields_names=c["opt_fields_names"])
        ps = cg.LagrangianParticleSet(c["position"], dim=3, **c["pset"])
        runs.append((cg.Solver(fs, ps, p, precision=precision, seed=6,
                               sort_period=sort_period), ps))
    (sa, pa), (sb, pb) = runs
    L = _lib.load()
    for call in range(2):
        sa.forward(nsteps=25)
        _lib.check(sb._ctx, L.cg_run_step_noalloc(sb._run, 25))
        got = dict(_state(pb), lowerlayer=pb.lowerlayer,
                   fluid_velocity_seen=pb.fluid_velocity_seen)
        want = dict(_state(pa), lowerlayer=pa.lowerlayer,
                    fluid_velocity_seen=pa.fluid_velocity_seen)
        assert_state_close(got, want, rtol=RTOL, what=f"lsm2 3d {precision} call {call + 1}")
        np.testing.assert_array_equal(pb.tag, pa.tag)
    sa.close()
    sb.close()


@pytest.mark.parametrize("what", ["sections", "stranding"])
def test_noalloc_refuses_section_and_stranding_runs(what):
    """Control-section counts and stranding records are kept in per-call
    buffers that only cg_run_step fills: the allocation-free entry point
    refuses such runs (CG_EINVAL, a message naming them) and changes
    nothing, so cg_run_step still steps the run afterwards."""
    from cylag_gb300 import _lib
    case, p = _case(2_000)
    s, ps = _solver(case, p, "mixed")
    L = _lib.load()
    if what == "sections":
        seg = np.array([[1000.0, 0.0, 1000.0, 1000.0]])
        _lib.check(s._ctx, L.cg_run_set_sections(s._run, 1, seg.ctypes.data))
    else:
        _lib.check(s._ctx, L.cg_run_set_stranding_output(s._run, 1))
    t0 = C.c_double()
    L.cg_run_time(s._run, C.byref(t0), None)
    rc = L.cg_run_step_noalloc(s._run, 3)
    assert rc == _lib.CG_EINVAL
    buf = C.create_string_buffer(512)
    L.cg_last_error(s._ctx, buf, 512)
    assert b"control sections or stranding" in buf.value
    t1 = C.c_double()
    L.cg_run_time(s._run, C.byref(t1), None)
    assert t1.value == t0.value
    _lib.check(s._ctx, L.cg_run_step(s._run, 2, None))
    s.close()


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
