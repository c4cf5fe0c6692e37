"""Shared test helpers.

Markers: ``gpu`` (needs a CUDA device; run on a GB300).  Everything else runs
on a CPU-only machine.  The oracle (oracle/) is test infrastructure: tests
use it only as the checker.
"""
from __future__ import annotations

import json
import platform
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
for p in (str(ROOT), str(ROOT / "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

# The reference rounds like gcc on x86-64 without FMA; the oracle built here
# reproduces it exactly.  On other hosts libm (exp/log/pow) may differ in the
# last place, so floating results are compared to a tight relative bound.
X86 = platform.machine() in ("x86_64", "AMD64")
RTOL = 1e-10


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


def golden_names():
    return sorted(p.stem[len("traj_"):] for p in GOLDEN.glob("traj_*.npz"))


def section_names():
    return sorted(p.stem[len("sec_"):] for p in GOLDEN.glob("sec_*.npz"))


def load_golden(name, prefix="traj"):
    z = np.load(GOLDEN / f"{prefix}_{name}.npz", allow_pickle=False)
    meta = json.loads(str(z["meta"]))
    case = dict(meta["case"])
    for k in z.files:
        if k.startswith("in_"):
            case[k[3:]] = z[k]
    out = {k[4:]: z[k] for k in z.files if k.startswith("out_")}
    return case, meta, out


def source_names():
    return sorted(p.stem[len("src_"):] for p in GOLDEN.glob("src_*.npz"))


def load_source(name):
    """A fixture of a reference run with particle sources: (case, meta, out);
    meta["sources"] describes the sources (see make_sources)."""
    z = np.load(GOLDEN / f"src_{name}.npz", allow_pickle=False)
    meta = json.loads(str(z["meta"]))
    case = dict(meta["case"])
    for k in z.files:
        if k.startswith("in_"):
            case[k[3:]] = z[k]
    out = {k[4:]: z[k] for k in z.files if k.startswith("out_")}
    return case, meta, out


def make_sources(spec, rng_stream=None):
    """ParticleSource objects (cylag_gb300.extra) from a fixture's JSON
    description: {"scheduler": schedules() keywords, "poly": [[x, y], ...],
    "kwargs": ParticleSource keywords}, or {"kind": "field", "scheduler",
    "kwargs": ParticleSourceFromField keywords} whose disc positions draw
    from pcg32_seed(*rng_stream) (one stream shared by the field sources, as
    the reference's global stream is)."""
    from cylag_gb300 import extra
    out = []
    shared = extra.HostPCG32(*(rng_stream if rng_stream is not None else (0, 0)))
    for d in spec:
        if d.get("kind") == "field":
            out.append(extra.ParticleSourceFromField(extra.schedules(**d["scheduler"]),
                                                     rng=shared, **d["kwargs"]))
            continue
        kw = dict(d.get("kwargs", {}))
        if "grid_res" in kw:
            kw["grid_res"] = np.array(kw["grid_res"], dtype=np.int32)
        out.append(extra.ParticleSource(extra.schedules(**d["scheduler"]),
                                        np.array(d["poly"], dtype=np.float64), **kw))
    return out


def mesh_from_case(case):
    from cylag_gb300.mesh import TriangularMesh
    return TriangularMesh(case["x"], case["y"], case["triangles"],
                          boundary_points=case.get("boundary_points"),
                          nopen=case.get("nopen", 0))


def fields_from_case(case):
    """The field-set arguments of a fixture case (``fdim``: the field set's
    dimension when it differs from the particles', pseudo-3D)."""
    return dict(dim=case.get("fdim", case.get("dim", 2)), nlayers=case.get("nlayers", 1),
                times=case["times"],
                elevation=case["elevation"], velocity_x=case["velocity_x"],
                velocity_y=case["velocity_y"], velocity_z=case.get("velocity_z"),
                opt_fields=case.get("opt_fields"), opt_fields_names=case.get("opt_fields_names"))


def run_oracle(case, meta, nthreads=1, nsteps=None, seed=None):
    import oracle
    o = oracle.OracleSolver(mesh_from_case(case), fields_from_case(case), meta["params"],
                            case["position"], pset=meta.get("pset"),
                            seed=meta["seed"] if seed is None else seed, nthreads=nthreads,
                            control_sections=[np.array(q) for q in meta.get("sections") or []],
                            friction_model=case.get("friction_model", 1),
                            friction_coefficient=case.get("friction_coefficient", 40.))
    o.solve(meta["nsteps"] if nsteps is None else nsteps)
    return o


def assert_state_close(got, want, rtol=RTOL, exact=False, what=""):
    """Integer state bit-exact; floating state within rtol (exact if asked)."""
    for k in ("tri", "inactive", "lowerlayer"):
        if k in want and k in got:
            np.testing.assert_array_equal(np.asarray(got[k]), want[k], err_msg=f"{what}: {k}")
    active = np.asarray(want["inactive"]) == 0
    for k in ("position", "velocity", "fluid_velocity_seen", "last_position", "depth"):
        if k not in want or k not in got:
            continue
        g, w = np.asarray(got[k])[active], np.asarray(want[k])[active]
        if exact:
            np.testing.assert_array_equal(g, w, err_msg=f"{what}: {k}")
        else:
            scale = np.maximum(np.abs(w), 1.0)
            err = np.max(np.abs(g - w) / scale) if g.size else 0.0
            assert err <= rtol, f"{what}: {k} max rel err {err:.3e} > {rtol:.1e}"


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle
