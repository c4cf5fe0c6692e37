"""Particle sources on the host side, checked without a GPU.

* the oracle with sources (pool growth by min_pool_size_update, reuse of
  deleted entries in index order, new tags, initialization of the added
  particles in the step that releases them, the one-step wait of entries of
  a pool grown in that step) reproduces the reference's runs recorded in
  tests/golden/src_*.npz: every pool entry, its tag and the pool size;
* the schedulers, the release grids and the field-criterion releases
  (cylag_gb300.extra) give the reference's answers, step by step, when the
  compiled reference is present.
"""
import numpy as np
import pytest

from conftest import (X86, assert_state_close, fields_from_case, load_source, make_sources,
                      mesh_from_case, source_names)


def host_field_set(case):
    """The host-side EulerianFieldSet that sources query (no device use)."""
    import cylag_gb300 as cg
    f = fields_from_case(case)
    return cg.EulerianFieldSet(mesh_from_case(case), **f)


def _oracle_run(case, meta, nthreads=1):
    import oracle
    pk = dict(meta["pset"])
    o = oracle.OracleSolver(mesh_from_case(case), fields_from_case(case), meta["params"],
                            case["position"], pset=pk, seed=0, nthreads=nthreads,
                            sources=make_sources(meta["sources"], meta.get("rng_stream")),
                            initial_pool_size=pk.get("initial_pool_size"),
                            min_pool_size_update=pk.get("min_pool_size_update", 1000),
                            field_set=host_field_set(case))
    sizes = []
    for _ in range(meta["nsteps"]):
        o.forward()
        sizes.append(o.n)
    return o, np.array(sizes)


@pytest.mark.parametrize("name", source_names())
def test_oracle_with_sources_matches_reference(oracle_lib, name):
    case, meta, want = load_source(name)
    o, sizes = _oracle_run(case, meta)
    np.testing.assert_array_equal(sizes, want["npart"])
    assert o.maxtag == int(want["maxtag"])
    got = dict(position=o.pos, velocity=o.vel, fluid_velocity_seen=o.fvs, tri=o.tri,
               inactive=o.inactive, lowerlayer=o.lowerlayer, last_position=o.last_pos)
    assert_state_close(got, want, exact=X86, what=name)
    np.testing.assert_array_equal(o.tag, want["tag"])
    np.testing.assert_array_equal(o.last_tri, want["last_tri"])
    np.testing.assert_array_equal(o.diameter, want["diameter"])


def _ref():
    import refpath
    if not refpath.available():
        pytest.skip("compiled reference not built here")
    return refpath.use_reference()


class _Clock:
    def __init__(self, t0, dt, tf):
        self.time, self.time_step, self.iteration, self.final_time = t0, dt, 0, tf

    def advance(self):
        self.time += self.time_step
        self.iteration += 1


@pytest.mark.parametrize("kw", [dict(time_delta=2.5, ini_time=1.0), dict(iteration_delta=3),
                                dict(times=[0.0, 0.5, 4.0, 4.2, 9.99, 30.]),
                                dict(iterations=[0, 2, 3, 17]), dict(count=4),
                                dict(always=True)])
def test_schedulers_fire_like_the_reference(kw):
    cy = _ref()
    from cylag_gb300 import extra
    a, b = extra.schedules(**kw), cy.schedules(**kw)
    ca = _Clock(0.0, 0.7, 20.0)
    cb = cy.SimuTime(False, initial_time=0.0, final_time=20.0, time_step=0.7)
    for _ in range(28):
        assert bool(a.now(ca)) == bool(b.now(cb)), (kw, ca.iteration)
        ca.advance()
        cb.increment()


def test_schedules_argument_errors():
    from cylag_gb300 import extra
    with pytest.raises(ValueError):
        extra.schedules()
    with pytest.raises(ValueError):
        extra.schedules(times=[1.0], count=3)
    with pytest.raises(ValueError, match="No argument found"):
        extra.schedules(never=True)


@pytest.mark.parametrize("poly,kw", [
    ([[10., 10.], [60., 10.], [60., 40.], [10., 40.]], dict(grid_res=[3, 2, 1])),
    ([[100., 60.], [180., 70.], [120., 95.]], dict(xy_method=2, xy_density=0.01)),
    ([[20., 20.], [90., 25.], [80., 80.], [30., 70.]], dict(xy_method=1, xy_npart=9)),
    ([[0., 0.], [7., 1.], [9., 6.], [4., 9.3], [-1., 5.]], dict(xy_method=1, xy_npart=200)),
])
def test_release_grids_match_the_reference(poly, kw):
    cy = _ref()
    from cylag_gb300 import extra
    P = np.array(poly)
    k = dict(kw)
    if "grid_res" in k:
        k["grid_res"] = np.array(k["grid_res"], dtype=np.int32)
    assert extra.polygon_area(P[:, 0], P[:, 1]) == cy.polygon_area(P[:, 0].copy(), P[:, 1].copy())
    for dim in (2, 3):
        kk = dict(k, zmin=-3.0, zmax=-0.5, z_method=1, z_npart=3) if dim == 3 else k
        a = extra.ParticleSource(extra.schedules(always=True), P, **kk)
        b = cy.ParticleSource(cy.schedules(always=True), P, **kk)
        np.testing.assert_array_equal(a.init_positions(None, dim),
                                      np.asarray(b.init_positions(None, dim)))


def test_vertex_adjacency_matches_reference():
    from conftest import GOLDEN
    z = np.load(GOLDEN / "mesh_open.npz")
    from cylag_gb300.mesh import TriangularMesh
    m = TriangularMesh(z["x"], z["y"], z["triangles"], boundary_points=z["boundary_points"],
                       nopen=int(z["nopen"]))
    np.testing.assert_array_equal(m.vertex_adjacency, z["vertex_adjacency"])


def test_host_pcg32_matches_reference_streams():
    from conftest import GOLDEN
    from cylag_gb300.extra import HostPCG32
    z = np.load(GOLDEN / "rng.npz")
    for j, (seed, stream) in enumerate(z["pairs"]):
        g = HostPCG32(int(seed), int(stream))
        np.testing.assert_array_equal([g.uniform() for _ in range(512)], z[f"uniform_{j}"])
