"""Particle snapshot files: the native writers (cg_snapshot_txt /
cg_snapshot_vtk, no GPU needed) against the reference's own writers on the
same particle arrays, byte for byte, when the compiled reference is present;
and the Python-repr float formatting on awkward values."""
import numpy as np
import pytest


def _ref():
    import refpath
    if not refpath.available():
        pytest.skip("compiled reference not built here")
    return refpath.use_reference()


AWKWARD = [1e16, 1e-5, 1e-4, 0.0001234, -0.0, 123.0, 1 / 3, 2.5e-300, -7.0e22, 1234567890123456.0,
           12345678901234567.0, 0.1, 100.0, 5e-324, 1.7976931348623157e308, -1.5, 3.0e-7, 99999.99]


def _arrays(dim, n, seed):
    rng = np.random.default_rng(seed)
    pos = rng.normal(0, 1e3, (n, dim)) * 10.0 ** rng.integers(-6, 8, (n, 1))
    vel = rng.normal(0, 1, (n, dim))
    fvs = rng.normal(0, 1, (n, dim))
    flat = pos.reshape(-1)
    flat[: len(AWKWARD)] = AWKWARD
    vel.reshape(-1)[: len(AWKWARD)] = AWKWARD[::-1]
    inactive = (rng.uniform(size=n) < 0.3).astype(np.int32)
    tag = rng.permutation(n * 3)[:n].astype(np.int32)
    return pos, vel, fvs, inactive, tag


@pytest.mark.parametrize("dim,model,depth", [(2, 1, False), (2, 2, False), (3, 1, False),
                                             (3, 3, False), (3, 1, True), (3, 2, True)])
def test_snapshot_files_match_reference_writers(tmp_path, dim, model, depth):
    """... with the compute_depth column (3D) in both formats."""
    cy = _ref()
    import importlib
    WT = importlib.import_module("cylag.io.writer_txt")
    WV = importlib.import_module("cylag.io.writer_vtk")
    from cylag_gb300 import output
    n = 50000 if dim == 2 else 30000   # above the parallel-format threshold
    pos, vel, fvs, inactive, tag = _arrays(dim, n, dim * 10 + model)
    ps = cy.LagrangianParticleSet(pos.copy(), velocity=vel.copy(), fluid_velocity_seen=fvs.copy(),
                                  dim=dim, compute_depth=depth)
    dep = None
    if depth:
        dep = np.random.default_rng(5).uniform(-1.0, 30.0, n)
        dep[: len(AWKWARD)] = AWKWARD
        np.asarray(ps.depth)[:] = dep
    np.asarray(ps.inactive)[:] = inactive
    np.asarray(ps.tag)[:] = tag
    ps.npart_active = int((inactive == 0).sum())
    ref, ours = tmp_path / "ref", tmp_path / "ours"
    ref.mkdir()
    ours.mkdir()
    t, it = 1234.5, 77
    wt = WT.write_txt_2d if dim == 2 else WT.write_txt_3d
    wv = WV.write_vtk_2d if dim == 2 else WV.write_vtk_3d
    wt(ps, t, it, 1, -1, str(ref), "particles", model)
    wv(ps, t, it, 1, -1, str(ref), "particles", model)
    tri = np.where(inactive == 0, 0, -1).astype(np.int32)
    output.write_snapshot((tri, tag, pos, vel, fvs if model >= 2 else None, None, dep), dim,
                          model, t, it, str(ours), "particles", "all")
    for name in ("particles.txt", f"particles_{it}.vtk"):
        a, b = (ref / name).read_bytes(), (ours / name).read_bytes()
        assert a == b, (name, _first_diff(a, b))


def _first_diff(a, b):
    k = next((i for i, (x, y) in enumerate(zip(a, b)) if x != y), min(len(a), len(b)))
    return a[max(0, k - 80):k + 80], b[max(0, k - 80):k + 80]


def test_snapshot_repr_formatting(tmp_path):
    """VTK positions use Python's repr of a double."""
    from cylag_gb300 import output
    vals = np.array(AWKWARD + list(np.random.default_rng(0).normal(0, 1, 200) *
                                   10.0 ** np.random.default_rng(1).integers(-20, 20, 200)))
    n = len(vals)
    pos = np.stack([vals, vals[::-1]], 1)
    output.write_snapshot((np.zeros(n, np.int32), np.arange(n, dtype=np.int32), pos,
                           np.zeros((n, 2)), None, None), 2, 1, 0.5, 3, str(tmp_path), "p", "vtk")
    lines = (tmp_path / "p_3.vtk").read_text().splitlines()
    k = lines.index(f"POINTS {n} FLOAT")
    for j in range(n):
        assert lines[k + 1 + j] == f"{float(pos[j, 0])!r} {float(pos[j, 1])!r} 0.0"
