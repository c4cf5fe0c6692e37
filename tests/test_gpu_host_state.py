"""cg_run_step_host: the particle state kept in (pinned) host memory and
streamed through the GPU in chunks, with the copies of one chunk overlapping
the step of another.  Results are bit-identical to copying the whole state
in, calling cg_run_step(run, 1) and copying it out, per step -- ragged last
chunks, exit statistics, control-section counts and stranding records
included."""
import ctypes as C

import numpy as np
import pytest

from conftest import fields_from_case, load_golden, mesh_from_case

pytestmark = pytest.mark.gpu


def _solver(case, params, precision, seed, sections=None):
    import cylag_gb300 as cg
    from cylag_gb300.extra import ControlSection
    f = fields_from_case(case)
    fs = cg.EulerianFieldSet(mesh_from_case(case), **f)
    ps = cg.LagrangianParticleSet(case["position"], dim=f["dim"])
    cs = None if sections is None else [ControlSection(np.array(q)) for q in sections]
    s = cg.Solver(fs, ps, params, control_sections=cs, precision=precision, seed=seed,
                  sort_period=0)
    return s, ps


def _pinned(ps, keys):
    import torch
    d = ps._dev
    h = {k: torch.empty_like(d[k], device="cpu").pin_memory() for k in keys}
    for k in keys:
        h[k].copy_(d[k])
    return h


def _arrays(h):
    from cylag_gb300 import _lib
    p = lambda k: h[k].data_ptr() if k in h else None
    return _lib.HostArrays(p("position"), p("velocity"), p("fluid_velocity_seen"), p("tri"),
                           p("lowerlayer"), p("tag"), p("rng_state"))


KEYS = ["position", "tri", "tag", "rng_state"]


def _by_device_steps(s, ps, h, nsteps, nopen):
    """copy in, cg_run_step(run, 1), copy out, per step"""
    import torch
    from cylag_gb300 import _lib
    d = ps._dev
    stats = []
    for _ in range(nsteps):
        for k in KEYS:
            d[k].copy_(h[k])
        torch.cuda.synchronize()
        st = np.zeros((1, max(1, nopen)), np.int32)
        _lib.check(s._ctx, s.L.cg_run_step(s._run, 1, st.ctypes.data))
        for k in KEYS:
            h[k].copy_(d[k])
        torch.cuda.synchronize()
        stats.append(st[0, :nopen].copy())
    return np.array(stats)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("npart,chunk,calls", [(50_000, 7001, [5, 1, 14]), (50_000, 0, [20]),
                                               (1_100_000, 0, [3, 2])])
def test_host_state_step_equals_device_steps(precision, npart, chunk, calls):
    """chunk 0 at 1.1e6 particles: the ramp of chunk sizes"""
    from test_gpu_mixed import keps_case
    from cylag_gb300 import _lib
    case, p = keps_case(npart)
    sa, pa = _solver(case, p, precision, 4)
    sb, pb = _solver(case, p, precision, 4)
    ha = _pinned(pa, KEYS)
    hb = _pinned(pb, KEYS)
    n = sum(calls)
    _by_device_steps(sa, pa, ha, n, 0)
    arr = _arrays(hb)
    for k in calls:
        _lib.check(sb._ctx, sb.L.cg_run_step_host(sb._run, k, C.byref(arr), C.byref(arr), chunk,
                                                  None))
    for k in KEYS:
        np.testing.assert_array_equal(ha[k].numpy(), hb[k].numpy(), err_msg=k)
    sa.close()
    sb.close()


def test_host_state_statistics_sections_stranding():
    """open channel with exits, stranding on walls and control sections:
    per-step exit and section counts and the stranded positions equal the
    device-state run's."""
    from cylag_gb300 import _lib
    case, meta, _ = load_golden("open_lsm1", prefix="sec")
    params = dict(meta["params"], output_rep="/tmp/cylag_host_state_test")
    nopen = int(case["nopen"])
    res = []
    for mode in ("device", "host"):
        s, ps = _solver(case, params, "fp64", meta["seed"], meta["sections"])
        h = _pinned(ps, KEYS)
        stats, csec, strand = [], [], []
        for _ in range(40):
            if mode == "device":
                st = _by_device_steps(s, ps, h, 1, nopen)[0]
            else:
                st = np.zeros((1, nopen), np.int32)
                arr = _arrays(h)
                _lib.check(s._ctx, s.L.cg_run_step_host(s._run, 1, C.byref(arr), C.byref(arr),
                                                        17, st.ctypes.data))
                st = st[0]
            stats.append(st)
            cs = np.zeros(len(meta["sections"]), np.int32)
            k = C.c_int32()
            s.L.cg_run_section_stats(s._run, cs.ctypes.data, C.byref(k))
            csec.append(cs)
            cnt = C.c_int32()
            s.L.cg_run_stranded(s._run, None, C.byref(cnt))
            xyz = np.zeros((cnt.value, 3))
            s.L.cg_run_stranded(s._run, xyz.ctypes.data, C.byref(cnt))
            strand.append(xyz)
        res.append((np.array(stats), np.array(csec), np.concatenate(strand),
                    {k: h[k].numpy().copy() for k in KEYS}))
        s.close()
    (a_st, a_cs, a_sd, a_h), (b_st, b_cs, b_sd, b_h) = res
    np.testing.assert_array_equal(a_st, b_st)
    np.testing.assert_array_equal(a_cs, b_cs)
    np.testing.assert_array_equal(a_sd, b_sd)
    assert a_st.sum() > 0 and a_cs.sum() > 0 and len(a_sd) > 0
    for k in KEYS:
        np.testing.assert_array_equal(a_h[k], b_h[k], err_msg=k)


@pytest.mark.parametrize("model", [2, 3])
def test_host_state_lsm23_3d(model):
    """3D LSM2/LSM3 with the velocity (and fluid velocity seen) and layer
    index kept in host memory: equal to the device-state steps."""
    import cylag_gb300 as cg
    import torch
    from cylag_gb300 import _lib, synth
    from cylag_gb300.mesh import TriangularMesh
    mk = synth.lsm2_loglaw_workload if model == 2 else synth.lsm3_taylor_green_workload
    c = mk(npart=20000, nx=81, ny=41, nplanes=11, seed=2)
    p = dict(c["parameters"], final_time=1e6)
    keys = ["position", "tri", "tag", "rng_state", "lowerlayer", "velocity"]
    if model == 3:
        keys.append("fluid_velocity_seen")
    res = []
    for mode in ("device", "host"):
        mesh = TriangularMesh(c["x"], c["y"], c["triangles"])
        fs = cg.EulerianFieldSet(mesh, dim=3, nlayers=c["nlayers"], times=c["times"],
                                 elevation=c["elevation"], velocity_x=c["velocity_x"],
                                 velocity_y=c["velocity_y"], velocity_z=c["velocity_z"],
                                 opt_fields=c.get("opt_fields"),
                                 opt_fields_names=c.get("opt_fields_names"))
        ps = cg.LagrangianParticleSet(c["position"], dim=3, **c.get("pset", {}))
        if "diameter" in c:
            ps.diameter = c["diameter"]
        s = cg.Solver(fs, ps, p, precision="mixed", seed=5, sort_period=0)
        d = ps._dev
        h = {k: torch.empty_like(d[k], device="cpu").pin_memory() for k in keys}
        for k in keys:
            h[k].copy_(d[k])
        for _ in range(12):
            if mode == "device":
                for k in keys:
                    d[k].copy_(h[k])
                torch.cuda.synchronize()
                _lib.check(s._ctx, s.L.cg_run_step(s._run, 1, None))
                for k in keys:
                    h[k].copy_(d[k])
                torch.cuda.synchronize()
            else:
                arr = _arrays(h)
                _lib.check(s._ctx, s.L.cg_run_step_host(s._run, 1, C.byref(arr), C.byref(arr),
                                                        3001, None))
        res.append({k: h[k].numpy().copy() for k in keys})
        s.close()
    for k in keys:
        np.testing.assert_array_equal(res[0][k], res[1][k], err_msg=k)
