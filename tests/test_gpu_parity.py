"""GPU particle step vs the reference (golden fixtures) and vs the oracle.

Plain form (FP64, -fmad=false): element indices, layer indices and
deletions bit-exact; positions and velocities within 1e-10 relative
(CUDA's exp/log/pow may differ from the host libm in the last place).
"""
import numpy as np
import pytest

from conftest import (RTOL, assert_state_close, fields_from_case, golden_names, load_golden,
                      mesh_from_case, run_oracle)

pytestmark = pytest.mark.gpu


def gpu_run(case, meta, nsteps=None, batch=None, precision="fp64", seed=None):
    import cylag_gb300 as cg
    mesh = mesh_from_case(case)
    f = fields_from_case(case)
    fs = cg.EulerianFieldSet(mesh, dim=f["dim"], nlayers=f["nlayers"], times=f["times"],
                             elevation=f["elevation"], velocity_x=f["velocity_x"],
                             velocity_y=f["velocity_y"], velocity_z=f["velocity_z"],
                             opt_fields=f["opt_fields"], opt_fields_names=f["opt_fields_names"],
                             friction_model=case.get("friction_model", 1),
                             friction_coefficient=case.get("friction_coefficient", 40.))
    ps = cg.LagrangianParticleSet(case["position"], dim=case.get("dim", 2), **meta.get("pset", {}))
    s = cg.Solver(fs, ps, meta["params"], precision=precision,
                  seed=meta["seed"] if seed is None else seed)
    n = meta["nsteps"] if nsteps is None else nsteps
    if batch is None:
        s.forward(nsteps=n)
    else:
        done = 0
        while done < n:
            k = min(batch, n - done)
            s.forward(nsteps=k)
            done += k
    return s, ps


def state(ps):
    out = dict(position=ps.position, velocity=ps.velocity,
               fluid_velocity_seen=ps.fluid_velocity_seen, tri=ps.tri,
               inactive=ps.inactive, lowerlayer=ps.lowerlayer, last_position=ps.last_position)
    if ps.compute_depth:
        out["depth"] = ps.depth
    return out


@pytest.mark.parametrize("name", golden_names())
def test_gpu_matches_reference_golden(name):
    case, meta, want = load_golden(name)
    s, ps = gpu_run(case, meta)
    assert_state_close(state(ps), want, rtol=RTOL, what=name)
    if meta["params"].get("bnd_statistics"):
        np.testing.assert_array_equal(s.bnd_statistics(), want["bnd_stats"])
    s.close()


@pytest.mark.parametrize("name", ["couette", "keps_ts2_rm1", "open", "3d_keps",
                                  "p3d_unsteady_keps3_ts4", "depth_3d_lsm2"])
def test_gpu_matches_oracle_stepwise(name):
    """Single-step calls (every public array refreshed each step) equal one
    batched call, and both equal the oracle run on this machine."""
    case, meta, _ = load_golden(name)
    o = run_oracle(case, meta)
    want = dict(position=o.pos, velocity=o.vel, fluid_velocity_seen=o.fvs, tri=o.tri,
                inactive=o.inactive, lowerlayer=o.lowerlayer, last_position=o.last_pos)
    if o.depth is not None:
        want["depth"] = o.depth
    s1, p1 = gpu_run(case, meta, batch=7)
    assert_state_close(state(p1), want, rtol=RTOL, what=name + " batch=7")
    np.testing.assert_array_equal(p1.tag, o.tag)
    s1.close()


def test_gpu_keps_larger_vs_oracle():
    """20,000 particles on a 101x26 jittered mesh, 100 steps of k-epsilon drift
    with time interpolation: indices bit-exact, positions to 1e-10."""
    from cylag_gb300 import synth
    c = synth.keps_drift_channel(npart=20000, nx=101, ny=26, seed=5)
    case = {k: c[k] for k in ("x", "y", "triangles", "times", "elevation", "velocity_x",
                              "velocity_y", "opt_fields", "position")}
    case["opt_fields_names"] = c["opt_fields_names"]
    p = dict(c["parameters"])
    p.update(time_step=2.0, final_time=400.0)
    meta = dict(params=p, nsteps=100, seed=3, pset={})
    o = run_oracle(case, meta, nthreads=8)
    want = dict(position=o.pos, tri=o.tri, inactive=o.inactive)
    s, ps = gpu_run(case, meta)
    assert_state_close(dict(position=ps.position, tri=ps.tri, inactive=ps.inactive), want,
                       rtol=RTOL, what="keps20k")
    s.close()


def test_gpu_run_from_telemac_files(tmp_path):
    """The open-channel fixture's mesh, boundary and fields written as a
    TELEMAC-2D result file (FP64) and a .cli file, read back through
    EulerianFieldSet.from_telemac2d: same trajectories as the reference's,
    exit counts per open boundary (numbered in .cli order)."""
    import cylag_gb300 as cg
    from cylag_gb300.telemac import write_selafin
    case, meta, want = load_golden("open")
    bp = case["boundary_points"]
    lines = []
    for vid, lab in bp:
        code = "2 2 2" if lab == 0 else "5 4 4"
        lines.append(f"{code} 0.0 0.0 0.0 0.0 2 0.0 0.0 0.0 {vid + 1} 0")
    (tmp_path / "open.cli").write_text("\n".join(lines) + "\n")
    nv = len(case["x"])
    vals = [[case["elevation"][0], case["velocity_x"][0], case["velocity_y"][0]]]
    write_selafin(tmp_path / "open.slf", case["x"], case["y"], case["triangles"], [0.0], vals,
                  ["FREE SURFACE", "VELOCITY U", "VELOCITY V"], double=True)
    fs = cg.EulerianFieldSet.from_telemac2d(str(tmp_path / "open.slf"),
                                            bnd_file=str(tmp_path / "open.cli"))
    assert fs.triangular_mesh.nopen == 2 and fs.npoints == nv
    ps = cg.LagrangianParticleSet(case["position"], dim=2, **meta.get("pset", {}))
    s = cg.Solver(fs, ps, meta["params"], seed=meta["seed"])
    s.forward(nsteps=meta["nsteps"])
    assert_state_close(state(ps), want, rtol=RTOL, what="from telemac")
    # .cli order numbers the right side 1 and the left side 2
    order = [2, 1] if bp[[i for i in range(len(bp)) if bp[i, 1]][0], 1] == 2 else [1, 2]
    got = s.bnd_statistics()
    np.testing.assert_array_equal(got[:, [o - 1 for o in order]], want["bnd_stats"])
    s.close()


def test_gpu_run_from_hdf5_files(tmp_path):
    """The open-channel fixture's field set saved as CyLag HDF5 mesh and
    field-set files (save_hdf5) and read back (from_hdf5): the reference's
    trajectories and exit counts.  The reloaded mesh is a second
    TriangularMesh built from the file's arrays, not the one that wrote it."""
    import cylag_gb300 as cg
    case, meta, want = load_golden("open")
    fs0 = cg.EulerianFieldSet(mesh_from_case(case), **fields_from_case(case))
    fs0.save_hdf5(str(tmp_path / "f.h5"), str(tmp_path / "m.h5"))
    fs = cg.EulerianFieldSet.from_hdf5(str(tmp_path / "f.h5"), str(tmp_path / "m.h5"))
    assert fs.triangular_mesh is not fs0.triangular_mesh and fs.triangular_mesh.nopen == 2
    ps = cg.LagrangianParticleSet(case["position"], dim=2, **meta.get("pset", {}))
    s = cg.Solver(fs, ps, meta["params"], seed=meta["seed"])
    s.forward(nsteps=meta["nsteps"])
    assert_state_close(state(ps), want, rtol=RTOL, what="from hdf5")
    np.testing.assert_array_equal(s.bnd_statistics(), want["bnd_stats"])
    s.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_sorted_state_kept_across_calls(precision):
    """An element-sorted run keeps its working copies between forward()
    calls (re-sorted every sort_period steps counted across calls).  100
    single-step calls, 100 steps in calls of 7 with the arrays read after
    every call (each read writes the copies back and the next step gathers
    them again), and one 100-step call leave the same state bit for bit:
    positions, elements, tags, PCG32 states and the per-call outputs (the
    velocity, fluid velocity seen and last velocity come from two working
    velocity arrays that the re-sorts move only in part)."""
    import cylag_gb300 as cg
    from cylag_gb300 import synth
    c = synth.keps_drift_channel(npart=20000, nx=101, ny=26, seed=5)
    case = {k: c[k] for k in ("x", "y", "triangles", "times", "elevation", "velocity_x",
                              "velocity_y", "opt_fields", "position")}
    case["opt_fields_names"] = c["opt_fields_names"]
    p = dict(c["parameters"], time_step=2.0, final_time=400.0)
    out = []
    for mode in ("one", "single", "read7"):
        f = fields_from_case(case)
        fs = cg.EulerianFieldSet(mesh_from_case(case), **f)
        ps = cg.LagrangianParticleSet(case["position"], dim=2)
        s = cg.Solver(fs, ps, p, precision=precision, seed=3, sort_period=10)
        if mode == "one":
            s.forward(nsteps=100)
        elif mode == "single":
            for _ in range(100):
                s.forward()
        else:
            done = 0
            while done < 100:
                k = min(7, 100 - done)
                s.forward(nsteps=k)
                done += k
                _ = ps.position
        ps._sync()
        out.append({k: ps._dev[k].cpu().numpy() for k in ("position", "tri", "tag", "rng_state",
                                                           "last_position", "velocity",
                                                           "fluid_velocity_seen", "last_velocity",
                                                           "last_tri")})
        s.close()
    for mode, o in zip(("single", "read7"), out[1:]):
        for k in out[0]:
            np.testing.assert_array_equal(o[k], out[0][k], err_msg=f"{precision} {mode}: {k}")


def test_device_samplers_match_reference_streams():
    """The device's PCG32 and its uniform, ziggurat and polar samplers
    (cg_rng_draws) against the streams the compiled reference drew from
    pcg32_seed(seed, stream): uniform draws and method-1 pairs bit-exact
    (integer arithmetic and exact FP64 scaling); ziggurat and polar draws
    within 1e-14 relative (exp and log of CUDA's library against the host's;
    an acceptance test decided the other way would desynchronize the stream
    and fail by far more)."""
    import ctypes as C
    from conftest import GOLDEN
    from cylag_gb300 import _lib
    L = _lib.load()
    ctx = C.c_void_p()
    _lib.check(None, L.cg_ctx_create(0, 0, C.byref(ctx)))
    z = np.load(GOLDEN / "rng.npz")

    def draws(seed, stream, kind, n, method=2):
        out = np.zeros(n * (2 if kind == 3 else 1))
        _lib.check(ctx, L.cg_rng_draws(ctx, seed, stream, kind, method, n, out.ctypes.data))
        return out

    def close(a, b, what):
        err = np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))
        assert err <= 1e-14, f"{what}: max rel err {err:.3e}"

    for j, (seed, stream) in enumerate(z["pairs"].tolist()):
        np.testing.assert_array_equal(draws(seed, stream, 0, 512), z[f"uniform_{j}"])
        close(draws(seed, stream, 1, 512), z[f"zig_{j}"], f"ziggurat {j}")
        close(draws(seed, stream, 2, 256), z[f"polar_{j}"], f"polar {j}")
        close(draws(seed, stream, 3, 128, method=3), z[f"pair3_{j}"], f"pair3 {j}")
        np.testing.assert_array_equal(draws(seed, stream, 3, 128, method=1), z[f"pair1_{j}"])
    L.cg_ctx_destroy(ctx)
