"""Generate the golden fixtures of tests/golden/ from the compiled reference.

Runs the unmodified reference CyLag (built by oracle/build_ref.py into
oracle/_ref) and records its outputs for small seeded inputs:

* ``rng.npz``: PCG32 uniform, ziggurat and polar draws
  (cylag/lsm/random_utils.pyx) for several (seed, stream) pairs, plus a
  SHA-256 of 200,000 ziggurat draws (pins the ziggurat tables);
* ``mesh_open.npz``: every TriangularMesh array of a channel with two open
  boundaries (cylag/geom/triangular_mesh.pyx);
* ``traj_*.npz``: inputs (mesh, fields, particles, parameters) and the final
  particle state after N steps of Solver.forward.

Per-particle streams: the reference draws from one global PCG32 in
particle order.  Each particle is therefore run through its own Solver with
``pcg32_seed(seed, tag)`` set just before; particles do not interact, so
this is the reference's own code path under the per-particle stream
convention, with no source change.

Usage (needs the reference build; run in the development container):
    python oracle/build_ref.py && python tests/golden/make_golden.py [group ...]
with groups rng, mesh, lsm1, lsm23 (default: all).
"""
from __future__ import annotations

import hashlib
import json
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT))
OUT = Path(__file__).resolve().parent

import refpath  # noqa: E402

from cylag_gb300 import synth  # noqa: E402


def _cylag():
    return refpath.use_reference()


def rng_fixture():
    cy = _cylag()
    R = cy.random_utils
    out = {}
    pairs = [(0, 0), (0, 1), (0, 12345), (42, 7), (7, 2**40 + 3)]
    for j, (seed, stream) in enumerate(pairs):
        R.pcg32_seed(seed, stream)
        out[f"uniform_{j}"] = np.array([R.random_uniform() for _ in range(512)])
        R.pcg32_seed(seed, stream)
        out[f"zig_{j}"] = np.array([R.random_gaussian_ziggurat() for _ in range(512)])
        R.pcg32_seed(seed, stream)
        out[f"polar_{j}"] = np.array([R.random_gaussian() for _ in range(256)])
        R.pcg32_seed(seed, stream)
        out[f"pair3_{j}"] = np.array([R.generate_random_pair(3) for _ in range(128)]).reshape(-1)
        R.pcg32_seed(seed, stream)
        out[f"pair1_{j}"] = np.array([R.generate_random_pair(1) for _ in range(128)]).reshape(-1)
        R.pcg32_seed(seed, stream)
        R.pcg32_advance(1000)
        out[f"adv_{j}"] = np.array([R.random_uniform() for _ in range(16)])
    R.pcg32_seed(0, 99)
    big = np.array([R.random_gaussian_ziggurat() for _ in range(200_000)])
    out["zig_big_sha256"] = np.frombuffer(hashlib.sha256(big.tobytes()).digest(), dtype=np.uint8)
    out["pairs"] = np.array(pairs, dtype=np.uint64)
    np.savez_compressed(OUT / "rng.npz", **out)


def open_channel(nx=21, ny=6, lx=400.0, ly=100.0, seed=0):
    """Channel whose left side is open boundary 1 and right side open
    boundary 2 (boundary points listed counter-clockwise, as a .cli file
    lists them; cylag/geom/triangular_mesh.pyx:536-548)."""
    x, y, tri = synth.channel_mesh(lx, ly, nx, ny, seed=seed)
    idx = lambda i, j: j * nx + i
    ring = ([idx(i, 0) for i in range(nx)] + [idx(nx - 1, j) for j in range(1, ny)] +
            [idx(i, ny - 1) for i in range(nx - 2, -1, -1)] + [idx(0, j) for j in range(ny - 2, 0, -1)])
    lab = np.zeros(len(ring), dtype=np.int32)
    for k, v in enumerate(ring):
        i, j = v % nx, v // nx
        if i == 0 and 0 < j < ny - 1:
            lab[k] = 1
        elif i == nx - 1 and 0 < j < ny - 1:
            lab[k] = 2
    bp = np.stack([np.array(ring, dtype=np.int32), lab], axis=1)
    return x, y, tri, bp, 2


def mesh_fixture():
    cy = _cylag()
    x, y, tri, bp, nopen = open_channel()
    m = cy.TriangularMesh(x, y, tri, boundary_points=bp, nopen=nopen)
    out = dict(x=x, y=y, triangles=tri, boundary_points=bp, nopen=nopen)
    for a in ("edges", "triedge_map", "edgetri_map", "edges_labels", "vertex_labels",
              "gradx", "grady", "det", "signed_area", "vertex_adjacency"):
        out[a] = np.asarray(getattr(m, a)).copy()
    np.savez_compressed(OUT / "mesh_open.npz", **out)


def run_reference(case, params, nsteps, seed=0, pset_kw=None, sections=None):
    """Run every particle through its own reference Solver with
    pcg32_seed(seed, tag) and return the stacked final state.  With
    ``sections`` (polylines), also the control-section counts summed over
    the particles ([nsteps, ncsec]); with stranding output on, the stranded
    positions in the order one Solver over all particles appends them (by
    step, then particle index)."""
    cy = _cylag()
    R = cy.random_utils
    pset_kw = dict(pset_kw or {})
    dim = case.get("dim", 2)
    mesh = cy.TriangularMesh(case["x"], case["y"], case["triangles"],
                             boundary_points=case.get("boundary_points"),
                             nopen=case.get("nopen", 0))
    fdim = case.get("fdim", dim)
    fset = cy.EulerianFieldSet(
        mesh, dim=fdim, nlayers=case.get("nlayers", 1), times=case["times"],
        elevation=case["elevation"], velocity_x=case["velocity_x"], velocity_y=case["velocity_y"],
        velocity_z=case.get("velocity_z"), opt_fields=case.get("opt_fields"),
        opt_fields_names=case.get("opt_fields_names"),
        friction_model=case.get("friction_model", 1),
        friction_coefficient=case.get("friction_coefficient", 40.))
    tmp = tempfile.mkdtemp(prefix="cylag_golden_")
    params = dict(params)
    params["output_rep"] = tmp
    keys = ("position", "velocity", "fluid_velocity_seen", "last_position", "last_velocity")
    res = {k: [] for k in keys + ("tri", "last_tri", "lowerlayer", "inactive")}
    if pset_kw.get("compute_depth"):
        res["depth"] = []
    nopen = case.get("nopen", 0)
    stats = np.zeros((nsteps, max(1, nopen)), dtype=np.int64)
    ncsec = len(sections or [])
    csec = np.zeros((nsteps, max(1, ncsec)), dtype=np.int64)
    stranded = []
    for i, p in enumerate(case["position"]):
        R.pcg32_seed(seed, i)
        ps = cy.LagrangianParticleSet(np.array(p, dtype=np.float64)[None, :], dim=dim, **pset_kw)
        if "diameter" in case:
            ps.diameter[0] = case["diameter"][i]
            ps.volume[0] = np.pi * case["diameter"][i] ** 3 / 6.
        cs = None if sections is None else [cy.ControlSection(np.array(q, dtype=np.float64))
                                            for q in sections]
        s = cy.Solver(fset, ps, params, control_sections=cs)
        for it in range(nsteps):
            before = ps.stranded_count
            s.forward(s.simutime.time_step)
            for k in range(before, ps.stranded_count):
                stranded.append((it, i, *np.asarray(ps.stranded_positions)[k]))
        if ncsec:
            csec[:, :ncsec] += np.asarray(s._csec_stats_data)[:nsteps, :ncsec]
        for k in keys:
            res[k].append(np.asarray(getattr(ps, k))[0].copy())
        res["tri"].append(ps.tri[0])
        res["last_tri"].append(ps.last_tri[0])
        res["lowerlayer"].append(ps.lowerlayer[0])
        res["inactive"].append(ps.inactive[0])
        if "depth" in res:
            res["depth"].append(np.asarray(ps.depth)[0])
        if params.get("bnd_statistics"):
            stats += np.asarray(s._bnd_stats_data)[:nsteps]
    out = {k: np.array(v) for k, v in res.items()}
    out["bnd_stats"] = stats[:, :nopen]
    if ncsec:
        out["csec_stats"] = csec[:, :ncsec]
    if params.get("stranding_output"):
        stranded.sort(key=lambda r: (r[0], r[1]))
        out["stranded"] = np.array([r[2:] for r in stranded], dtype=np.float64).reshape(-1, 3)
    return out


def save_traj(name, case, params, nsteps, seed=0, pset_kw=None, sections=None, prefix="traj"):
    res = run_reference(case, params, nsteps, seed, pset_kw, sections)
    inputs = {k: v for k, v in case.items() if isinstance(v, np.ndarray)}
    meta = {k: v for k, v in case.items() if not isinstance(v, np.ndarray)}
    np.savez_compressed(
        OUT / f"{prefix}_{name}.npz",
        meta=json.dumps({"params": params, "nsteps": nsteps, "seed": seed,
                         "pset": pset_kw or {}, "case": meta, "sections": sections}),
        **{f"in_{k}": v for k, v in inputs.items()},
        **{f"out_{k}": v for k, v in res.items()})
    na = int((res["inactive"] == 0).sum())
    extra = ""
    if "csec_stats" in res:
        extra += f", crossings {res['csec_stats'].sum(0).tolist()}"
    if "stranded" in res:
        extra += f", {len(res['stranded'])} stranded"
    print(f"{prefix}_{name}: {len(case['position'])} particles x {nsteps} steps, {na} active{extra}")


def traj_fixtures():
    # LSM1 2D, Couette channel (101x11, 2,000 triangles), constant K, walls
    c = synth.couette_channel(npart=64)
    case = {k: c[k] for k in ("x", "y", "triangles", "times", "elevation", "velocity_x",
                              "velocity_y", "position")}
    p = dict(c["parameters"])
    p["final_time"] = 300.0
    save_traj("couette", case, p, 300)

    # LSM1 2D, k-epsilon drift, time interpolation over 3 records
    c = synth.keps_drift_channel(npart=48, nx=41, ny=11)
    case = {k: c[k] for k in ("x", "y", "triangles", "times", "elevation", "velocity_x",
                              "velocity_y", "opt_fields", "position")}
    case["opt_fields_names"] = c["opt_fields_names"]
    for ts, rm in ((1, 2), (2, 1), (3, 3), (4, 2)):
        p = dict(c["parameters"])
        p.update(time_step=5.0, final_time=500.0, time_scheme=ts, rng_method=rm)
        save_traj(f"keps_ts{ts}_rm{rm}", case, p, 80)

    # LSM1 2D, open boundaries (exit statistics), stranding, damped rebound
    x, y, tri, bp, nopen = open_channel()
    u = 0.4 + 0.0 * x
    v = 0.05 * np.sin(2 * np.pi * x / 400.0)
    rng = np.random.default_rng(11)
    pos = np.stack([rng.uniform(5.0, 395.0, 64), rng.uniform(0.5, 99.5, 64)], 1)
    case = dict(x=x, y=y, triangles=tri, boundary_points=bp, nopen=nopen, times=np.zeros(1),
                elevation=np.ones((1, len(x))), velocity_x=u[None, :], velocity_y=v[None, :],
                position=pos)
    p = dict(model=1, diffusion_model=1, horizontal_diffusivity=0.5, time_scheme=1,
             frozen_eulerian_fields=True, time_step=2.0, final_time=400.0,
             bnd_statistics=True, stranding_probability=0.2, rebound_damping_coef=0.3)
    save_traj("open", case, p, 200)

    # LSM1 3D sigma layers, k-epsilon 3D drift, Euler
    c = synth.loglaw_case(nx=21, ny=11, lx=400.0, ly=200.0, nplanes=6, npart=48)
    case = {k: c[k] for k in ("x", "y", "triangles", "times", "elevation", "velocity_x",
                              "velocity_y", "velocity_z", "opt_fields", "position")}
    case.update(dim=3, nlayers=6, opt_fields_names=c["opt_fields_names"])
    p = dict(model=1, diffusion_model=3, time_scheme=1, frozen_eulerian_fields=True,
             time_step=1.0, final_time=60.0, vertical_diffusivity=1e-3)
    save_traj("3d_keps", case, p, 60)
    # LSM1 3D, RK4, constant K, settling (Ruby-Zanke range), bed/surface reflection
    p = dict(model=1, diffusion_model=1, time_scheme=4, frozen_eulerian_fields=True,
             time_step=2.0, final_time=120.0, horizontal_diffusivity=0.05,
             vertical_diffusivity=2e-3)
    save_traj("3d_rk4_settling", case, p, 60,
              pset_kw=dict(particle_density=2650., particle_diameter=3e-4,
                           buoyancy_velocity_model=1))


def _keps2d(npart=40):
    c = synth.keps_drift_channel(npart=npart, nx=41, ny=11)
    case = {k: c[k] for k in ("x", "y", "triangles", "times", "elevation", "velocity_x",
                              "velocity_y", "opt_fields", "position")}
    case["opt_fields_names"] = c["opt_fields_names"]
    return case


def _loglaw3d(npart=40, unsteady=False):
    c = synth.loglaw_case(nx=21, ny=11, lx=400.0, ly=200.0, nplanes=6, npart=npart)
    case = {k: c[k] for k in ("x", "y", "triangles", "times", "elevation", "velocity_x",
                              "velocity_y", "velocity_z", "opt_fields", "position")}
    case.update(dim=3, nlayers=6, opt_fields_names=c["opt_fields_names"])
    if unsteady:
        # two records 300 s apart, the second current 25% stronger with a
        # small vertical component: exercises the Eulerian time derivative of
        # the added-mass acceleration
        case["times"] = np.array([0.0, 300.0])
        case["elevation"] = np.concatenate([case["elevation"]] * 2)
        w = 1e-3 * np.sin(2 * np.pi * c["x"] / 400.0)
        w = np.tile(w, 6)
        case["velocity_x"] = np.concatenate([case["velocity_x"], 1.25 * case["velocity_x"]])
        case["velocity_y"] = np.concatenate([case["velocity_y"], 1.25 * case["velocity_y"]])
        case["velocity_z"] = np.concatenate([case["velocity_z"], w[None, :]])
        case["opt_fields"] = np.concatenate([case["opt_fields"]] * 2, axis=1)
    return case


def lsm23_fixtures():
    """LSM2 (particle velocity) and LSM3 (velocity seen) cases, 2D and 3D.
    The reference accepts the Runge-Kutta schemes (2-4) for LSM2 only
    without diffusion, and only Euler-Maruyama (1) or the direct
    integrator (5) otherwise (cylag/core/parameters.pyx:219-238)."""
    c2 = _keps2d()
    base2 = dict(frozen_eulerian_fields=False, time_step=2.0, final_time=500.0,
                 schmidt_number=0.72)
    lsm2_2d = [
        # name, parameters, particle-set keywords
        ("lsm2_ts1_am", dict(model=2, time_scheme=1, diffusion_model=1,
                             horizontal_diffusivity=0.5),
         dict(added_mass_force=True)),
        ("lsm2_ts2_cd0", dict(model=2, time_scheme=2, diffusion_model=0),
         dict(drag_coefficient_model=0, drag_coefficient=0.8)),
        ("lsm2_ts3_am_cd2", dict(model=2, time_scheme=3, diffusion_model=0),
         dict(added_mass_force=True, drag_coefficient_model=2)),
        ("lsm2_ts4", dict(model=2, time_scheme=4, diffusion_model=0), {}),
        ("lsm2_ts5_ode_keps_rm2", dict(model=2, time_scheme=5, diffusion_model=2, rng_method=2),
         {}),
        # explicit velocity updates are stable for a1*dt < 2: smaller steps
        ("lsm2_em_opt2", dict(model=2, time_scheme=1, diffusion_model=1, diffusion_lsm2_option=2,
                              horizontal_diffusivity=0.01, time_step=0.25), {}),
        # the k-epsilon velocity noise grows with the drag rate, which grows
        # with the slip for Cd*|slip| drag: a small constant Cd keeps it bounded
        ("lsm2_em_opt3_keps", dict(model=2, time_scheme=1, diffusion_model=2,
                                   diffusion_lsm2_option=3, time_step=1.0),
         dict(added_mass_force=True, drag_coefficient_model=0, drag_coefficient=0.01)),
        ("lsm2_di_opt2_am", dict(model=2, time_scheme=5, diffusion_model=1,
                                 diffusion_lsm2_option=2, horizontal_diffusivity=0.01),
         dict(added_mass_force=True)),
        ("lsm2_di_opt3_keps3_small", dict(model=2, time_scheme=5, diffusion_model=3,
                                          diffusion_lsm2_option=3),
         dict(particle_diameter=1e-3, particle_density=1050.)),
        ("lsm3_em_const", dict(model=3, time_scheme=1, diffusion_model=1, time_step=0.25,
                               horizontal_diffusivity=0.5, diffusion_lsm3_tl_horizontal=20.),
         dict(particle_diameter=0.05)),
        ("lsm3_em_keps_am", dict(model=3, time_scheme=1, diffusion_model=2, time_step=0.25),
         dict(added_mass_force=True, particle_diameter=0.05)),
        ("lsm3_di_keps3_am", dict(model=3, time_scheme=5, diffusion_model=3),
         dict(added_mass_force=True)),
        ("lsm3_di_edge1_const", dict(model=3, time_scheme=5, diffusion_model=1, lsm3_edge_opt=1,
                                     horizontal_diffusivity=0.5,
                                     diffusion_lsm3_tl_horizontal=5.), {}),
        ("lsm3_di_edge1_keps_small", dict(model=3, time_scheme=5, diffusion_model=2,
                                          lsm3_edge_opt=1),
         dict(particle_diameter=1e-3, particle_density=1050.)),
    ]
    for name, prm, pkw in lsm2_2d:
        p = dict(base2)
        p.update(prm)
        save_traj(name, c2, p, 60 if p["time_step"] >= 1.0 else 100, seed=5, pset_kw=pkw)

    # particles released within 2 m of the walls: Runge-Kutta stages that
    # leave the domain stop the step early and leave the element index at -1
    # for the final localization (cylag/lsm/update_state_lsm2.pyx:291-333)
    cw = dict(c2)
    rng = np.random.default_rng(21)
    side = rng.integers(0, 4, 40)
    t = rng.uniform(0.0, 1.0, 40)
    d = rng.uniform(0.05, 2.0, 40)
    px = np.where(side == 0, d, np.where(side == 1, 4000.0 - d, 5.0 + t * 3990.0))
    py = np.where(side == 2, d, np.where(side == 3, 1000.0 - d, 5.0 + t * 990.0))
    cw["position"] = np.stack([px, py], 1)
    for ts in (2, 3, 4):
        p = dict(base2)
        p.update(model=2, time_scheme=ts, diffusion_model=0, time_step=2.0)
        save_traj(f"lsm2_ts{ts}_walls", cw, p, 60, seed=6)

    c3 = _loglaw3d()
    c3u = _loglaw3d(unsteady=True)
    base3 = dict(time_step=1.0, final_time=100.0, vertical_diffusivity=1e-3,
                 horizontal_diffusivity=0.05)
    lsm23_3d = [
        ("lsm2_3d_rk4_settling", c3, dict(model=2, time_scheme=4, diffusion_model=0,
                                          frozen_eulerian_fields=True, time_step=0.1),
         dict(particle_density=1200.)),
        ("lsm2_3d_di_opt3_keps_am", c3u, dict(model=2, time_scheme=5, diffusion_model=2,
                                              diffusion_lsm2_option=3,
                                              frozen_eulerian_fields=False),
         dict(added_mass_force=True)),
        ("lsm2_3d_em_opt2_keps3", c3, dict(model=2, time_scheme=1, diffusion_model=3,
                                           diffusion_lsm2_option=2, time_step=0.5,
                                           frozen_eulerian_fields=True),
         dict(drag_coefficient_model=0, drag_coefficient=0.01)),
        # explicit seen-velocity updates need dt < T_L: constant T_L here (the
        # k-epsilon T_L of the log-law case vanishes at the bed)
        ("lsm3_3d_em_const", c3, dict(model=3, time_scheme=1, diffusion_model=1,
                                      diffusion_lsm3_tl_horizontal=10.,
                                      diffusion_lsm3_tl_vertical=5.,
                                      frozen_eulerian_fields=True, time_step=0.5),
         dict(particle_diameter=0.05)),
        ("lsm3_3d_di_keps_am", c3u, dict(model=3, time_scheme=5, diffusion_model=2,
                                         diffusion_lsm3_tl_vertical=10.,
                                         frozen_eulerian_fields=False),
         dict(added_mass_force=True, particle_density=1100.)),
        ("lsm3_3d_di_edge1_const", c3, dict(model=3, time_scheme=5, diffusion_model=1,
                                            lsm3_edge_opt=1, diffusion_lsm3_tl_horizontal=10.,
                                            diffusion_lsm3_tl_vertical=5.,
                                            frozen_eulerian_fields=True), {}),
    ]
    for name, case, prm, pkw in lsm23_3d:
        p = dict(base3)
        p.update(prm)
        save_traj(name, case, p, 50 if p["time_step"] >= 0.5 else 100, seed=8, pset_kw=pkw)


# ---------------------------------------------------------------------------
# particle sources: one reference Solver for the whole pool (no diffusion,
# so no draws), sources releasing into a pool that reuses deleted entries and
# grows by min_pool_size_update
# ---------------------------------------------------------------------------
def make_sources(cy, spec):
    """Sources from their JSON description, with the reference's classes."""
    out = []
    for d in spec:
        sch = cy.schedules(**d["scheduler"])
        if d.get("kind") == "field":
            out.append(cy.ParticleSourceFromField(sch, **d["kwargs"]))
            continue
        kw = dict(d.get("kwargs", {}))
        if "grid_res" in kw:
            kw["grid_res"] = np.array(kw["grid_res"], dtype=np.int32)
        out.append(cy.ParticleSource(sch, np.array(d["poly"], dtype=np.float64), **kw))
    return out


def run_reference_sources(case, params, nsteps, spec, pset_kw, rng_stream=None):
    cy = _cylag()
    dim = case.get("dim", 2)
    mesh = cy.TriangularMesh(case["x"], case["y"], case["triangles"],
                             boundary_points=case.get("boundary_points"),
                             nopen=case.get("nopen", 0))
    fset = cy.EulerianFieldSet(
        mesh, dim=dim, nlayers=case.get("nlayers", 1), times=case["times"],
        elevation=case["elevation"], velocity_x=case["velocity_x"], velocity_y=case["velocity_y"],
        velocity_z=case.get("velocity_z"), opt_fields=case.get("opt_fields"),
        opt_fields_names=case.get("opt_fields_names"))
    params = dict(params, output_rep=tempfile.mkdtemp(prefix="cylag_golden_"))
    ps = cy.LagrangianParticleSet(case["position"], dim=dim, **pset_kw)
    s = cy.Solver(fset, ps, params, sources=make_sources(cy, spec))
    if rng_stream is not None:
        # the field sources' disc positions are the only draws of these runs
        cy.random_utils.pcg32_seed(*rng_stream)
    npart = []
    for _ in range(nsteps):
        s.forward(s.simutime.time_step)
        npart.append(ps.npart)
    out = {k: np.asarray(getattr(ps, k)).copy() for k in
           ("position", "velocity", "fluid_velocity_seen", "last_position", "last_velocity",
            "tri", "last_tri", "lowerlayer", "inactive", "tag", "diameter")}
    out["npart"] = np.array(npart, dtype=np.int64)
    out["maxtag"] = np.array(ps.maxtag)
    return out


def save_sources(name, case, params, nsteps, spec, pset_kw, rng_stream=None):
    res = run_reference_sources(case, params, nsteps, spec, pset_kw, rng_stream)
    inputs = {k: v for k, v in case.items() if isinstance(v, np.ndarray)}
    meta = {k: v for k, v in case.items() if not isinstance(v, np.ndarray)}
    np.savez_compressed(
        OUT / f"src_{name}.npz",
        meta=json.dumps({"params": params, "nsteps": nsteps, "sources": spec,
                         "pset": pset_kw, "case": meta, "rng_stream": rng_stream}),
        **{f"in_{k}": v for k, v in inputs.items()},
        **{f"out_{k}": v for k, v in res.items()})
    na = int((res["inactive"] == 0).sum())
    print(f"src_{name}: pool {res['npart'][0]}..{res['npart'][-1]}, {na} active after "
          f"{nsteps} steps, maxtag {int(res['maxtag'])}")


def source_fixtures():
    # 2D open channel, two field records (time interpolation), LSM1 RK4
    # without diffusion: exits free entries, three sources refill them
    x, y, tri, bp, nopen = open_channel()
    u0 = 0.4 + 0.3 * y / 100.0
    v0 = 0.05 * np.sin(2 * np.pi * x / 400.0)
    rng = np.random.default_rng(21)
    pos = np.stack([rng.uniform(250.0, 395.0, 20), rng.uniform(2.0, 98.0, 20)], 1)
    case = dict(x=x, y=y, triangles=tri, boundary_points=bp, nopen=nopen,
                times=np.array([0.0, 200.0]), elevation=np.ones((2, len(x))),
                velocity_x=np.stack([u0, 1.3 * u0]), velocity_y=np.stack([v0, -v0]),
                position=pos)
    p = dict(model=1, diffusion_model=0, time_scheme=4, frozen_eulerian_fields=False,
             time_step=2.0, final_time=200.0, bnd_statistics=True)
    spec = [
        # 6 particles every 4 iterations
        dict(scheduler=dict(iteration_delta=4),
             poly=[[10., 10.], [60., 10.], [60., 40.], [10., 40.]],
             kwargs=dict(grid_res=[3, 2, 1])),
        # triangle by density; 41.0 and 41.5 fall in the same step: one release
        dict(scheduler=dict(times=[3.0, 17.0, 41.0, 41.5]),
             poly=[[100., 60.], [180., 70.], [120., 95.]],
             kwargs=dict(xy_method=2, xy_density=0.01)),
        # half outside the mesh: those particles are deleted at initialization
        dict(scheduler=dict(count=5),
             poly=[[300., 80.], [340., 80.], [340., 130.], [300., 130.]],
             kwargs=dict(grid_res=[2, 5, 1])),
    ]
    save_sources("open_lsm1_rk4", case, p, 90, spec,
                 dict(initial_pool_size=24, min_pool_size_update=7))
    # same with Euler and a release every 6 s by time_delta, npart-based grid
    p1 = dict(p, time_scheme=1)
    spec1 = [dict(scheduler=dict(time_delta=6.0, ini_time=1.0),
                  poly=[[20., 20.], [90., 25.], [80., 80.], [30., 70.]],
                  kwargs=dict(xy_method=1, xy_npart=9)),
             spec[2]]
    save_sources("open_lsm1_euler", case, p1, 90, spec1,
                 dict(initial_pool_size=20, min_pool_size_update=5))

    # releases where a field meets a criterion: three field records (the
    # record changes at t = 60 s), a density field in kg/m2 and a source
    # field; interior nodes only; disc positions from the global stream,
    # seeded (5, 77) once the solver exists
    nv = len(x)
    srng = np.random.default_rng(31)
    src_field = np.zeros((3, nv))
    for r in range(3):
        src_field[r, srng.choice(nv, 6, replace=False)] = 1.0
    dens = np.stack([0.01 + 0.008 * (1 + np.sin(2 * np.pi * x / 150.0))] * 3)
    casef = dict(case, times=np.array([0.0, 60.0, 200.0]), elevation=np.ones((3, nv)),
                 velocity_x=np.stack([u0, 1.2 * u0, 1.3 * u0]),
                 velocity_y=np.stack([v0, 0.5 * v0, -v0]),
                 opt_fields=np.stack([dens, src_field]),
                 opt_fields_names=["DENSITY", "SOURCE"], position=pos[:8])
    specf = [
        dict(kind="field", scheduler=dict(iteration_delta=2),
             kwargs=dict(field_id_criteria=5, field_id_density=4, criteria="val_gt",
                         threshold=0.5, virtual_mass=2.0, single_release=True)),
        dict(kind="field", scheduler=dict(times=[10.0, 70.0, 71.0]),
             kwargs=dict(field_id_criteria=5, field_id_density=4, criteria="var_geq",
                         threshold=0.5)),
    ]
    save_sources("field_open_lsm1", casef, dict(p, time_scheme=2), 60, specf,
                 dict(initial_pool_size=8, min_pool_size_update=16), rng_stream=[5, 77])

    # 3D log-law, LSM2 RK4 without diffusion, settling particles, a 3D
    # source every 5 iterations
    c = synth.loglaw_case(nx=21, ny=11, lx=400.0, ly=200.0, nplanes=6, npart=30)
    case3 = {k: c[k] for k in ("x", "y", "triangles", "times", "elevation", "velocity_x",
                               "velocity_y", "velocity_z", "opt_fields", "position")}
    case3.update(dim=3, nlayers=6, opt_fields_names=c["opt_fields_names"])
    hmin = float(c["bathymetry"].min())
    p3 = dict(model=2, time_scheme=4, diffusion_model=0, frozen_eulerian_fields=True,
              time_step=0.1, final_time=100.0)
    spec3 = [dict(scheduler=dict(iteration_delta=5),
                  poly=[[50., 50.], [150., 50.], [150., 120.], [50., 120.]],
                  kwargs=dict(grid_res=[3, 2, 2], zmin=-0.9 * hmin, zmax=-0.1 * hmin))]
    save_sources("loglaw3d_lsm2_rk4", case3, p3, 40, spec3,
                 dict(min_pool_size_update=10, particle_density=1200.))


# ---------------------------------------------------------------------------
# control sections and stranding output
# ---------------------------------------------------------------------------
def section_fixtures():
    # 2D open channel, LSM1 diffusion, walls with stranding, open exits
    x, y, tri, bp, nopen = open_channel()
    u = 0.4 + 0.0 * x
    v = 0.05 * np.sin(2 * np.pi * x / 400.0)
    rng = np.random.default_rng(12)
    pos = np.stack([rng.uniform(5.0, 395.0, 80), rng.uniform(0.5, 99.5, 80)], 1)
    case = dict(x=x, y=y, triangles=tri, boundary_points=bp, nopen=nopen, times=np.zeros(1),
                elevation=np.ones((1, len(x))), velocity_x=u[None, :], velocity_y=v[None, :],
                position=pos)
    p = dict(model=1, diffusion_model=1, horizontal_diffusivity=0.8, time_scheme=1,
             frozen_eulerian_fields=True, time_step=2.0, final_time=400.0,
             bnd_statistics=True, stranding_probability=0.3, stranding_output=True)
    sections = [
        [[200.0, -10.0], [200.0, 110.0]],                  # across the channel
        [[100.0, 20.0], [300.0, 80.0], [350.0, 0.0]],      # first segment only counts
        [[50.0, 50.0], [380.0, 50.0]],                     # along the flow
        [[0.0, 0.0], [0.0, 100.0]],                        # the inlet line (and the origin)
    ]
    save_traj("open_lsm1", case, p, 150, seed=3, sections=sections, prefix="sec")
    # RK4 without diffusion: deterministic crossings
    p2 = dict(p, diffusion_model=0, time_scheme=4, stranding_probability=0.5)
    save_traj("open_lsm1_rk4", case, p2, 150, seed=3, sections=sections, prefix="sec")

    # 3D sigma layers, LSM2 DI with k-epsilon: walls strand, sections in (x, y)
    c3 = _loglaw3d(npart=60)
    p3 = dict(model=2, time_scheme=5, diffusion_model=3, diffusion_lsm2_option=2,
              frozen_eulerian_fields=True, time_step=1.0, final_time=100.0,
              stranding_probability=0.4, stranding_output=True)
    sec3 = [[[0.0, 100.0], [400.0, 100.0]], [[150.0, -5.0], [250.0, 205.0]]]
    save_traj("loglaw3d_lsm2", c3, p3, 60, seed=8, sections=sec3, prefix="sec")


def _p3d_channel(npart=48, unsteady=False, keps=False, seed=21):
    """Pseudo-3D case: 2D fields (free surface, depth-averaged current,
    BOTTOM) on a 400 m x 100 m walled channel (41x11 vertices, random
    diagonals), 3D particles.  The bed slopes down along x and across the
    channel, the free surface carries a standing wave; unsteady: records 0,
    200, 400 s with the wave rising and the current strengthening (dzs/dt
    and the Eulerian fields change between steps).  keps: nodal k and eps
    (K = 0.02 + 0.03 (1 + sin(2 pi x / 200)) / 2) for the k-epsilon
    diffusion models."""
    x, y, tri = synth.channel_mesh(400.0, 100.0, 41, 11, seed=seed)
    zb = -4.0 - 2.0 * (x / 400.0) - 0.5 * (y / 100.0)
    times = np.array([0.0, 200.0, 400.0]) if unsteady else np.zeros(1)
    amp = [1.0, 1.4, 1.8] if unsteady else [1.0]
    zs = np.stack([0.3 * a * np.sin(2 * np.pi * x / 400.0) for a in amp])
    u = np.stack([(0.25 + 0.05 * a) + 0.05 * np.cos(2 * np.pi * y / 100.0) for a in amp])
    v = np.stack([0.04 * a * np.sin(2 * np.pi * x / 200.0) for a in amp])
    names = ["BOTTOM"]
    opt = [np.stack([zb] * len(times))]
    if keps:
        K = 0.02 + 0.03 * 0.5 * (1.0 + np.sin(2 * np.pi * x / 200.0))
        k, eps = synth.keps_from_K(K)
        names += ["TURBULENT ENERG.", "DISSIPATION"]
        opt += [np.stack([k] * len(times)), np.stack([eps] * len(times))]
    rng = np.random.default_rng(seed + 1)
    px = rng.uniform(20.0, 380.0, npart)
    py = rng.uniform(2.0, 98.0, npart)
    zbp = -4.0 - 2.0 * (px / 400.0) - 0.5 * (py / 100.0)
    zsp = 0.3 * np.sin(2 * np.pi * px / 400.0)
    pz = zbp + (zsp - zbp) * rng.uniform(0.02, 0.98, npart)
    return dict(x=x, y=y, triangles=tri, dim=3, fdim=2, nlayers=1, times=times,
                elevation=zs, velocity_x=u, velocity_y=v, opt_fields=np.stack(opt),
                opt_fields_names=names, position=np.stack([px, py, pz], 1))


def p3d_fixtures():
    """Pseudo-3D LSM1 (2D fields, 3D particles; the log-law horizontal
    factor and the vertical velocity of eulerian_field_set.pyx:1887-1955
    inside every time scheme) and compute_depth (solver.pyx:526-538)."""
    base = dict(model=1, frozen_eulerian_fields=True, time_step=5.0, final_time=1000.0)
    c = _p3d_channel()
    # advection only, every time scheme and the four friction laws
    for ts, fm, fc in ((1, 1, 40.), (2, 0, 60.), (3, 2, 0.025), (4, 3, 0.05)):
        cc = dict(c, friction_model=fm, friction_coefficient=fc)
        save_traj(f"p3d_ts{ts}_fm{fm}", cc, dict(base, diffusion_model=0, time_scheme=ts), 80,
                  pset_kw=dict(compute_depth=True))
    # constant diffusion, settling, bed and surface reflection, walls
    save_traj("p3d_rk2_diff_settling", c,
              dict(base, diffusion_model=1, time_scheme=2, horizontal_diffusivity=0.05,
                   vertical_diffusivity=5e-3, rebound_damping_coef=0.2), 80, seed=2,
              pset_kw=dict(particle_density=2650., particle_diameter=2e-4,
                           buoyancy_velocity_model=1, compute_depth=True))
    # unsteady fields (dzs/dt, time interpolation), k-epsilon diffusion
    cu = _p3d_channel(unsteady=True, keps=True)
    for dm, ts in ((2, 1), (3, 4)):
        save_traj(f"p3d_unsteady_keps{dm}_ts{ts}", cu,
                  dict(model=1, frozen_eulerian_fields=False, time_step=4.0, final_time=400.0,
                       diffusion_model=dm, time_scheme=ts, vertical_diffusivity=1e-3), 90,
                  seed=5, pset_kw=dict(compute_depth=True))
    # compute_depth on 3D sigma-layer fields: LSM1 k-eps, LSM2 DI, LSM3 DI
    c3 = _loglaw3d(npart=40)
    save_traj("depth_3d_lsm1", c3, dict(model=1, diffusion_model=3, time_scheme=1,
                                        frozen_eulerian_fields=True, time_step=1.0,
                                        final_time=60.0, vertical_diffusivity=1e-3), 60,
              pset_kw=dict(compute_depth=True))
    save_traj("depth_3d_lsm2", c3, dict(model=2, time_scheme=5, diffusion_model=3,
                                        diffusion_lsm2_option=2, frozen_eulerian_fields=True,
                                        time_step=1.0, final_time=60.0), 60, seed=4,
              pset_kw=dict(compute_depth=True, particle_density=1000., particle_diameter=1e-4))
    save_traj("depth_3d_lsm3", c3, dict(model=3, time_scheme=5, diffusion_model=1,
                                        horizontal_diffusivity=0.01, vertical_diffusivity=1e-3,
                                        frozen_eulerian_fields=True, time_step=1.0,
                                        final_time=60.0), 60, seed=6,
              pset_kw=dict(compute_depth=True, particle_density=2650.,
                           particle_diameter=1e-4))


GROUPS = {"rng": rng_fixture, "mesh": mesh_fixture, "lsm1": traj_fixtures,
          "lsm23": lsm23_fixtures, "sources": source_fixtures, "sections": section_fixtures,
          "p3d": p3d_fixtures}

if __name__ == "__main__":
    for g in (sys.argv[1:] or list(GROUPS)):
        GROUPS[g]()
