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
    python oracle/build_ref.py && python tests/golden/make_golden.py
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
              "gradx", "grady", "det", "signed_area"):
        out[a] = np.asarray(getattr(m, a)).copy()
    np.savez_compressed(OUT / "mesh_open.npz", **out)


def run_reference(case, params, nsteps, seed=0, pset_kw=None):
    """Run every particle through its own reference Solver with
    pcg32_seed(seed, tag) and return the stacked final state."""
    cy = _cylag()
    R = cy.random_utils
    pset_kw = dict(pset_kw or {})
    dim = case.get("dim", 2)
    mesh = cy.TriangularMesh(case["x"], case["y"], case["triangles"],
                             boundary_points=case.get("boundary_points"),
                             nopen=case.get("nopen", 0))
    fset = cy.EulerianFieldSet(
        mesh, dim=dim, nlayers=case.get("nlayers", 1), times=case["times"],
        elevation=case["elevation"], velocity_x=case["velocity_x"], velocity_y=case["velocity_y"],
        velocity_z=case.get("velocity_z"), opt_fields=case.get("opt_fields"),
        opt_fields_names=case.get("opt_fields_names"))
    tmp = tempfile.mkdtemp(prefix="cylag_golden_")
    params = dict(params)
    params["output_rep"] = tmp
    keys = ("position", "velocity", "fluid_velocity_seen", "last_position", "last_velocity")
    res = {k: [] for k in keys + ("tri", "last_tri", "lowerlayer", "inactive")}
    nopen = case.get("nopen", 0)
    stats = np.zeros((nsteps, max(1, nopen)), dtype=np.int64)
    for i, p in enumerate(case["position"]):
        R.pcg32_seed(seed, i)
        ps = cy.LagrangianParticleSet(np.array(p, dtype=np.float64)[None, :], dim=dim, **pset_kw)
        if "diameter" in case:
            ps.diameter[0] = case["diameter"][i]
            ps.volume[0] = np.pi * case["diameter"][i] ** 3 / 6.
        s = cy.Solver(fset, ps, params)
        for _ in range(nsteps):
            s.forward(s.simutime.time_step)
        for k in keys:
            res[k].append(np.asarray(getattr(ps, k))[0].copy())
        res["tri"].append(ps.tri[0])
        res["last_tri"].append(ps.last_tri[0])
        res["lowerlayer"].append(ps.lowerlayer[0])
        res["inactive"].append(ps.inactive[0])
        if params.get("bnd_statistics"):
            stats += np.asarray(s._bnd_stats_data)[:nsteps]
    out = {k: np.array(v) for k, v in res.items()}
    out["bnd_stats"] = stats[:, :nopen]
    return out


def save_traj(name, case, params, nsteps, seed=0, pset_kw=None):
    res = run_reference(case, params, nsteps, seed, pset_kw)
    inputs = {k: v for k, v in case.items() if isinstance(v, np.ndarray)}
    meta = {k: v for k, v in case.items() if not isinstance(v, np.ndarray)}
    np.savez_compressed(
        OUT / f"traj_{name}.npz",
        meta=json.dumps({"params": params, "nsteps": nsteps, "seed": seed,
                         "pset": pset_kw or {}, "case": meta}),
        **{f"in_{k}": v for k, v in inputs.items()},
        **{f"out_{k}": v for k, v in res.items()})
    na = int((res["inactive"] == 0).sum())
    print(f"traj_{name}: {len(case['position'])} particles x {nsteps} steps, {na} active")


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


if __name__ == "__main__":
    rng_fixture()
    mesh_fixture()
    traj_fixtures()
