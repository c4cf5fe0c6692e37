"""Host-side logic that needs no GPU: parameters, mesh preprocessing,
point-location grid, the C ABI surface, the Python API's failure modes."""
import ctypes as C
import re

import numpy as np
import pytest

from conftest import GOLDEN, ROOT


# ---------------------------------------------------------------------------
# parameters (cylag/core/parameters.pyx:116-351)
# ---------------------------------------------------------------------------
def test_parameters_defaults_and_time_scheme():
    from cylag_gb300.parameters import Parameters
    assert Parameters({}).time_scheme == 4                      # LSM1, no diffusion
    assert Parameters({"diffusion_model": 1}).time_scheme == 1  # LSM1 + diffusion
    assert Parameters({"model": 2}).time_scheme == 5
    assert Parameters({"model": 3, "diffusion_model": 1}).time_scheme == 5
    assert Parameters({"model": 1, "time_scheme": 2}).time_scheme == 2
    p = Parameters({"frozen_eulerian_fields": True, "initial_time": 5.})
    assert p.initial_time == 0.


def test_parameters_errors():
    from cylag_gb300.parameters import Parameters
    with pytest.raises(TypeError):
        Parameters({"not_a_key": 1})
    with pytest.raises(TypeError):
        Parameters({"time_step": 1})        # int where the default is float
    for bad in ({"model": 4}, {"rng_method": 0}, {"model": 3, "diffusion_model": 0},
                {"model": 2, "diffusion_model": 1, "time_scheme": 2},
                {"rebound_damping_coef": 1.5}, {"stranding_probability": -0.1}):
        with pytest.raises(ValueError):
            Parameters(bad).check_values()


def test_parameters_match_reference():
    import refpath
    if not refpath.available():
        pytest.skip("reference build not present")
    cy = refpath.use_reference()
    from cylag_gb300.parameters import Parameters
    for d in ({}, {"model": 2}, {"model": 1, "diffusion_model": 2},
              {"frozen_eulerian_fields": True, "initial_time": 3.}):
        a, b = Parameters(d), cy.Parameters(d)
        for k in ("time_scheme", "initial_time", "rng_method", "max_wall_rebounds",
                  "rebound_damping_coef", "schmidt_number", "lsm3_edge_opt"):
            assert getattr(a, k) == getattr(b, k), (d, k)


# ---------------------------------------------------------------------------
# mesh (cylag/geom/triangular_mesh.pyx)
# ---------------------------------------------------------------------------
def test_mesh_arrays_match_reference_golden():
    from cylag_gb300.mesh import TriangularMesh
    z = np.load(GOLDEN / "mesh_open.npz")
    m = TriangularMesh(z["x"], z["y"], z["triangles"], boundary_points=z["boundary_points"],
                       nopen=int(z["nopen"]))
    for a in ("edges", "triedge_map", "edgetri_map", "edges_labels", "vertex_labels",
              "gradx", "grady", "det", "signed_area"):
        np.testing.assert_array_equal(getattr(m, a), z[a], err_msg=a)


def test_mesh_rejects_bad_input():
    from cylag_gb300.mesh import TriangularMesh
    x = np.array([0., 1., 0., 2.])
    y = np.array([0., 0., 1., 0.])
    with pytest.raises(ValueError):
        TriangularMesh(x, y, np.array([[0, 1, 3]], dtype=np.int32))   # zero area
    with pytest.raises(ValueError):
        TriangularMesh(x, y, np.array([[0, 1, 7]], dtype=np.int32))   # index out of range
    with pytest.raises(ValueError):
        TriangularMesh(np.array([0., np.nan, 0.]), y[:3], np.array([[0, 1, 2]], dtype=np.int32))


def test_locator_grid_finds_lowest_index_triangle(oracle_lib):
    """The bucket grid returns what an exhaustive lowest-index search returns,
    for centroids, vertices (ties) and points outside."""
    import ctypes as C
    from cylag_gb300 import synth
    from cylag_gb300.mesh import TriangularMesh
    x, y, tri = synth.channel_mesh(400.0, 100.0, 41, 11, seed=3, jitter=0.3)
    m = TriangularMesh(x, y, tri)
    g = m.locator_grid()
    ptr = lambda a: a.ctypes.data
    mesh = oracle_lib.Mesh(m.nv, m.nt, m.ne, ptr(m.x), ptr(m.y), ptr(m.triangles), ptr(m.gradx),
                           ptr(m.grady), ptr(m.det), ptr(m.edges), ptr(m.triedge_map),
                           ptr(m.edgetri_map), ptr(m.edges_labels), g[0], g[1], g[2], g[3], g[4],
                           ptr(g[5]), ptr(g[6]))
    L = oracle_lib.lib()
    cen = np.stack([x[tri].mean(1), y[tri].mean(1)], 1)
    rng = np.random.default_rng(0)
    pts = np.concatenate([cen, np.stack([x, y], 1), rng.uniform(-50, 450, (2000, 2))])
    for px, py in pts:
        a = L.cgo_locate(C.byref(mesh), px, py)
        b = L.cgo_locate_exhaustive(C.byref(mesh), px, py)
        assert a == b, (px, py, a, b)


# ---------------------------------------------------------------------------
# the C ABI
# ---------------------------------------------------------------------------
def header_functions():
    text = (ROOT / "include" / "cylag_gpu.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|uint64_t)\s+(cg_\w+)\s*\(", text, flags=re.M)))


def test_library_exports_every_declared_symbol():
    from cylag_gb300 import _lib
    if not _lib.library_path().exists():
        from cylag_gb300 import build
        build.build()
    L = C.CDLL(str(_lib.library_path()))
    names = header_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(L, n), n
    declared = {n for n, _, _ in _lib.SIGNATURES}
    assert set(names) <= declared, set(names) - declared


def test_library_fails_cleanly_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from cylag_gb300 import _lib
    L = _lib.load()
    ctx = C.c_void_p()
    assert L.cg_ctx_create(0, 0, C.byref(ctx)) == _lib.CG_ECUDA
    assert not ctx.value
    # null arguments are rejected, not dereferenced
    assert L.cg_run_step(None, 1, None) == _lib.CG_EINVAL
    assert L.cg_ctx_destroy(None) == _lib.CG_EINVAL


def test_solver_refuses_to_run_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import cylag_gb300 as cg
    from conftest import fields_from_case, load_golden, mesh_from_case
    case, meta, _ = load_golden("couette")
    f = fields_from_case(case)
    fs = cg.EulerianFieldSet(mesh_from_case(case), dim=2, times=f["times"],
                             elevation=f["elevation"], velocity_x=f["velocity_x"],
                             velocity_y=f["velocity_y"])
    ps = cg.LagrangianParticleSet(case["position"], dim=2)
    with pytest.raises((RuntimeError, cg._lib.CylagGpuError)):
        cg.Solver(fs, ps, meta["params"])


def test_particle_set_host_arrays_before_attach():
    import cylag_gb300 as cg
    pos = np.array([[1., 2.], [3., 4.]])
    ps = cg.LagrangianParticleSet(pos, dim=2, initial_pool_size=5)
    assert ps.npart == 5 and ps.npart_active == 2
    np.testing.assert_array_equal(ps.position[:2], pos)
    np.testing.assert_array_equal(ps.inactive, [0, 0, 1, 1, 1])
    with pytest.raises(ValueError):
        cg.LagrangianParticleSet(np.zeros((3, 3)), dim=2)
    with pytest.raises(ValueError):
        cg.LagrangianParticleSet(pos, dim=2, initial_pool_size=1)


def test_field_set_validation():
    import cylag_gb300 as cg
    from cylag_gb300 import synth
    from cylag_gb300.mesh import TriangularMesh
    x, y, tri = synth.channel_mesh(10., 10., 3, 3)
    m = TriangularMesh(x, y, tri)
    nv = len(x)
    with pytest.raises(ValueError):
        cg.EulerianFieldSet(m, times=np.array([0., 0.]), elevation=np.ones((2, nv)),
                            velocity_x=np.ones((2, nv)), velocity_y=np.ones((2, nv)))
    with pytest.raises(ValueError):
        cg.EulerianFieldSet(m, times=np.zeros(1), elevation=np.ones((1, nv + 1)),
                            velocity_x=np.ones((1, nv)), velocity_y=np.ones((1, nv)))
    fs = cg.EulerianFieldSet(m, times=np.zeros(1), elevation=np.ones((1, nv)),
                             velocity_x=np.ones((1, nv)), velocity_y=np.ones((1, nv)),
                             opt_fields=np.ones((2, 1, nv)),
                             opt_fields_names=["DISSIPATION", "TURBULENT ENERG."])
    assert fs.fid_dissip == 4 and fs.fid_turbeng == 5


# ---------------------------------------------------------------------------
# host helpers of the step: retagging, record search, error reports
# ---------------------------------------------------------------------------
def test_retag_follows_deletion_order():
    """Markers -1 (deleted at initialization, before the call's steps) and
    -2-it (deleted in iteration it) become maxtag+1, ... in deletion order,
    index order within one iteration (lagrangian_particle_set.pyx:786-788)."""
    from cylag_gb300.core import retag
    tag = np.array([0, -7, 2, -2, -1, 5, -2, -7, -1], dtype=np.int32)
    got, mx = retag(tag, 10)
    #             init (-1): idx 4, 8 -> 11, 12; it 0 (-2): idx 3, 6 -> 13, 14;
    #             it 5 (-7): idx 1, 7 -> 15, 16
    np.testing.assert_array_equal(got, [0, 15, 2, 13, 11, 5, 14, 16, 12])
    assert mx == 16
    same, mx2 = retag(np.array([3, 4], np.int32), 4)
    np.testing.assert_array_equal(same, [3, 4])
    assert mx2 == 4


def test_lower_index_intervals():
    """zlocalizer.pyx:125-151: the record interval holding a time."""
    from cylag_gb300.core import lower_index
    t = np.array([0.0, 600.0, 1200.0, 1800.0])
    assert lower_index(t, -5.0) == 0
    assert lower_index(t, 0.0) == 0
    assert lower_index(t, 599.9) == 0
    assert lower_index(t, 600.0) == 1
    assert lower_index(t, 1799.0, last=1) == 2
    assert lower_index(t, 1800.0) == 2 and lower_index(t, 5000.0) == 2
    assert lower_index(np.array([0.0]), 10.0) == 0


def test_error_reports_known_answers():
    from cylag_gb300.stats import diffusion_report, displacement_report
    x0 = np.zeros((4, 2))
    xb = np.array([[1.0, 0.0], [-1.0, 0.0], [0.0, 2.0], [0.0, -2.0]])
    xa = xb * 1.1
    rep = displacement_report(x0, xa, xb)
    assert rep["n"] == 4
    np.testing.assert_allclose(rep["var_rel_err"], [0.21, 0.21])   # (1.1^2 - 1)
    np.testing.assert_allclose(rep["mean_rel_err"], [0.0, 0.0], atol=1e-15)
    np.testing.assert_allclose(rep["rms_displacement_diff"], np.sqrt((0.01 + 0.01 + 0.04 + 0.04) / 4))
    rng = np.random.default_rng(1)
    K, t, n = 0.5, 100.0, 200_000
    x = rng.normal(0.0, np.sqrt(2 * K * t), (n, 2))
    d = diffusion_report(np.zeros((n, 2)), x, K, t)
    assert d["var_exact"] == 100.0 and max(abs(z) for z in d["z"]) < 5


def test_particle_set_delete_like_the_reference():
    """lagrangian_particle_set.pyx:712-788: delete() deactivates the listed
    active particles in the order listed (once each), zeroes their state and
    retags them maxtag+1, ...; delete_single is the one-particle case."""
    import cylag_gb300 as cg
    pos = np.arange(12, dtype=np.float64).reshape(6, 2) + 1.0
    ps = cg.LagrangianParticleSet(pos, dim=2)
    assert ps.maxtag == 5 and ps.npart_active == 6
    ps.delete(np.array([4, 1, 4, 0], dtype=np.int32))
    np.testing.assert_array_equal(ps.tag, [8, 7, 2, 3, 6, 5])
    assert ps.maxtag == 8 and ps.npart_active == 3
    np.testing.assert_array_equal(ps.inactive, [1, 1, 0, 0, 1, 0])
    assert not ps.position[[0, 1, 4]].any() and (ps.position[[2, 3, 5]] == pos[[2, 3, 5]]).all()
    np.testing.assert_array_equal(ps.last_tri[[0, 1, 4]], -1)
    ps.delete_single(2)
    ps.delete_single(2)          # already inactive: nothing happens
    ps.delete([])
    assert ps.tag[2] == 9 and ps.maxtag == 9 and ps.npart_active == 2


def test_particle_set_depth_like_the_reference():
    """compute_depth: the reference refuses it for 2D sets (ValueError) and
    leaves depth None without it; a 3D set starts with zero depths
    (lagrangian_particle_set.pyx:212-219), grows them with the pool and
    zeroes a deleted particle's."""
    import cylag_gb300 as cg
    ps = cg.LagrangianParticleSet(np.zeros((3, 2)) + 1.0, dim=2)
    assert ps.depth is None
    with pytest.raises(ValueError):
        cg.LagrangianParticleSet(np.zeros((3, 2)) + 1.0, dim=2, compute_depth=True)
    ps3 = cg.LagrangianParticleSet(np.zeros((3, 3)) + 1.0, dim=3, compute_depth=True,
                                   min_pool_size_update=4)
    np.testing.assert_array_equal(ps3.depth, np.zeros(3))
    ps3._host["depth"][:] = [1.0, 2.0, 3.0]
    ps3.delete([1])
    np.testing.assert_array_equal(ps3.depth, [1.0, 0.0, 3.0])
    ps3.add(np.array([[5.0, 5.0, -1.0], [6.0, 6.0, -1.0]]))
    assert ps3.depth.shape == (7,) and ps3.depth[3:].tolist() == [0.0] * 4


# ---------------------------------------------------------------------------
# pre- and post-processing helpers (eulerian_field_set.pyx:606-1886)
# ---------------------------------------------------------------------------
def _inside_all(mesh, x, y):
    """Brute force: every triangle under the reference's point-in-triangle
    test (utils.pyx:332-385)."""
    t = mesh.triangles
    a = np.stack([mesh.x[t[:, 0]], mesh.y[t[:, 0]]])
    b = np.stack([mesh.x[t[:, 1]], mesh.y[t[:, 1]]])
    c = np.stack([mesh.x[t[:, 2]], mesh.y[t[:, 2]]])

    def rot(v, eo, ei):
        wx, wy = x - v[0], y - v[1]
        t1 = eo[0] * wy - wx * eo[1]
        t2 = ei[0] * wy - wx * ei[1]
        return (t1 == 0) | (t2 == 0) | (np.signbit(t1) == np.signbit(t2))

    return np.flatnonzero(rot(a, b - a, a - c) & rot(b, c - b, b - a) & rot(c, a - c, c - b))


def test_find_triangle_is_the_lowest_index_containing_triangle():
    from cylag_gb300 import synth
    from cylag_gb300.mesh import TriangularMesh
    x, y, tri = synth.channel_mesh(100.0, 40.0, 21, 9, seed=3, jitter=0.3)
    mesh = TriangularMesh(x, y, tri)
    rng = np.random.default_rng(4)
    pts = np.concatenate([np.stack([rng.uniform(-5, 105, 400), rng.uniform(-5, 45, 400)], 1),
                          np.stack([x[:40], y[:40]], 1)])        # vertices: shared by several
    for px, py in pts:
        allk = _inside_all(mesh, px, py)
        assert mesh.find_triangle(px, py) == (allk[0] if len(allk) else -1)


def _linear_fieldset(dim=2, nl=1):
    import cylag_gb300 as cg
    from cylag_gb300 import synth
    from cylag_gb300.mesh import TriangularMesh
    x, y, tri = synth.channel_mesh(100.0, 40.0, 21, 9, seed=3, jitter=0.3)
    mesh = TriangularMesh(x, y, tri)
    n = len(x)
    lin = 2.0 * x - 3.0 * y + 5.0
    if dim == 2:
        rec = lambda s: (s * lin)[None, :]
        zs = np.zeros((2, n))
        return cg.EulerianFieldSet(mesh, dim=2, nlayers=1, times=np.array([0.0, 10.0]),
                                   elevation=zs, velocity_x=np.concatenate([rec(1), rec(2)]),
                                   velocity_y=np.concatenate([rec(-1), rec(-1)])), lin
    planes = np.concatenate([-10.0 + 2.5 * l + 0.0 * x for l in range(nl)])
    lin3 = np.concatenate([lin] * nl)
    return cg.EulerianFieldSet(mesh, dim=3, nlayers=nl, times=np.array([0.0]),
                               elevation=planes[None, :], velocity_x=lin3[None, :],
                               velocity_y=planes[None, :], velocity_z=np.zeros((1, nl * n))), lin


def test_field_interpolation_helpers_2d():
    fs, lin = _linear_fieldset()
    names, ids = fs.get_field_list()
    assert names[:3] == ["ELEVATION", "VELOCITY U", "VELOCITY V"] and ids[:3] == [0, 1, 2]
    # time interpolation between records: 0.75 * rec0 + 0.25 * rec1 at t = 2.5
    np.testing.assert_allclose(fs.get_field(1, 2.5), 1.25 * lin, rtol=1e-14)
    rng = np.random.default_rng(5)
    for px, py in np.stack([rng.uniform(1, 99, 50), rng.uniform(1, 39, 50)], 1):
        want = 2.0 * px - 3.0 * py + 5.0
        got = fs.interpolate_field(1, np.array([px, py]), 2.5)
        assert abs(got - 1.25 * want) <= 1e-10 * max(1.0, abs(want))
        u, v = fs.interpolate_velocity(np.array([px, py]), 10.0)
        assert abs(u - 2.0 * want) <= 1e-10 * max(1.0, abs(want))
        assert abs(v + want) <= 1e-10 * max(1.0, abs(want))
    with pytest.raises(ValueError):
        fs.interpolate_field(1, np.array([500.0, 500.0]), 0.0)
    with pytest.raises(ValueError):
        fs.get_field(3, 0.0)
    assert fs.record == 0   # the set's own record is left alone


def test_field_interpolation_helpers_3d():
    fs, lin = _linear_fieldset(dim=3, nl=5)
    np.testing.assert_allclose(fs.get_field(0, 0.0, layer=2), -5.0)
    rng = np.random.default_rng(6)
    for px, py, pz in np.stack([rng.uniform(1, 99, 40), rng.uniform(1, 39, 40),
                                rng.uniform(-10, 0, 40)], 1):
        pt = np.array([px, py, pz])
        # VELOCITY V holds the layer elevations: linear in z between them
        assert abs(fs.interpolate_field(2, pt, 0.0) - pz) <= 1e-9
        u, v, w = fs.interpolate_velocity(pt, 0.0)
        assert abs(u - (2.0 * px - 3.0 * py + 5.0)) <= 1e-9 and abs(v - pz) <= 1e-9 and w == 0.0


def test_mesh_from_a_triangulation_object():
    """triangular_mesh.pyx:182-201: TriangularMesh.from_matplotlib takes any
    object with x, y, triangles and edges; same arrays as the constructor."""
    from types import SimpleNamespace
    from cylag_gb300 import synth
    from cylag_gb300.mesh import TriangularMesh
    x, y, tri = synth.channel_mesh(50.0, 20.0, 11, 5, seed=1, jitter=0.2)
    ref = TriangularMesh(x, y, tri)
    got = TriangularMesh.from_matplotlib(SimpleNamespace(x=x, y=y, triangles=tri, edges=ref.edges))
    for k in ("edges", "triedge_map", "edgetri_map", "edges_labels", "gradx", "grady", "det"):
        np.testing.assert_array_equal(getattr(got, k), getattr(ref, k), err_msg=k)


def test_field_set_check_dim():
    fs, _ = _linear_fieldset()
    fs.check_dim(np.zeros((2, fs.npoints)))
    with pytest.raises(ValueError):
        fs.check_dim(np.zeros((1, fs.npoints)))


def test_particle_set_drag_and_buoyancy_like_the_reference(capsys):
    """lagrangian_particle_set.pyx:790-890 on the host: the three drag laws
    (double powers as complex powers, as the compiled reference evaluates
    them) and the settling-velocity laws across their diameter ranges."""
    import cylag_gb300 as cg
    nu, g = 1.3e-6, 9.80665
    cp = lambda x, y: (complex(x) ** y).real
    for model in (0, 1, 2):
        ps = cg.LagrangianParticleSet(np.ones((2, 2)), dim=2, drag_coefficient_model=model,
                                      drag_coefficient=0.5)
        for U, dp in ((1e-3, 1e-4), (0.2, 1e-3), (2.0, 5e-3), (50.0, 0.05)):
            Re = max(1e-16, U * dp / nu)
            if model == 0:
                want = 0.5
            elif model == 1:
                want = (24. / Re) * (1. + 0.15 * cp(Re, 0.687)) if Re <= 1000. else 0.44
            else:
                p1 = (24. / Re) ** 10 + cp(21. * cp(Re, -0.67), 10.) + cp(4. * cp(Re, -0.33), 10.) \
                    + 0.4 ** 10
                p2 = 1. / (cp(0.148 * cp(Re, 0.11), -10.) + 0.5 ** -10)
                p3 = cp(1.57 * cp(Re, -1.625) * 1e8, 10.)
                p4 = 1. / (cp(6e-17 * cp(Re, 2.63), -10.) + 0.2 ** -10)
                want = (1. / (1. / (p1 + p2) + 1. / p3) + p4) ** 0.1
            got = ps.drag_coefficient(U, dp)
            assert abs(got - want) <= 1e-13 * abs(want), (model, U, dp, got, want)
    ps = cg.LagrangianParticleSet(np.ones((2, 2)), dim=2, particle_density=2650.,
                                  buoyancy_velocity_model=1, drag_coefficient=0.44)
    s = 2.65
    assert np.isclose(ps.buoyancy_velocity(5e-5, 0, 1000.), -(s - 1) * g * 5e-5 ** 2 / (18 * nu))
    assert np.isclose(ps.buoyancy_velocity(5e-4, 0, 1000.),
                      -(10 * nu / 5e-4) * (np.sqrt(1 + (s - 1) * g * 5e-4 ** 3 / (100 * nu ** 2)) - 1))
    assert np.isclose(ps.buoyancy_velocity(2e-3, 0, 1000.), -np.sqrt((s - 1) * 4 * 2e-3 * g / (3 * 0.44)))
    assert np.isclose(ps.buoyancy_velocity(2e-3, 1, 1000.), -1.1 * np.sqrt((s - 1) * g * 2e-3))
    light = cg.LagrangianParticleSet(np.ones((2, 2)), dim=2, particle_density=900.,
                                     buoyancy_velocity_model=1)
    assert light.buoyancy_velocity(5e-5, 0, 1000.) > 0
    const = cg.LagrangianParticleSet(np.ones((2, 2)), dim=2, buoyancy_velocity=-0.01)
    assert const.buoyancy_velocity(1e-3, 0, 1000.) == -0.01
    const.show_status(1)
    assert "Particle n° 1" in capsys.readouterr().out
