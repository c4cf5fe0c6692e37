"""CyLag's HDF5 mesh and field-set files (cylag/geom/triangular_mesh.pyx:204-290,
cylag/core/eulerian_field_set.pyx:486-604) through cylag_gb300.hdf5, which
reads and writes the HDF5 subset those files use without h5py.

Pinned on the reference's own mesh file, tests/data/geo_flume.h5 of the
reference tree (its test_04_geom_mesh_io.py writes it with
``save_mesh_hdf5`` from r2d_flume.slf and geo_flume.cli): every array read
from it equals the mesh this package builds from the same TELEMAC files.
The file's edges are numbered as the matplotlib version that wrote it
numbered them ((max, min) pairs in order); the connectivity is compared
through that renumbering.
"""
import numpy as np
import pytest

from cylag_gb300 import hdf5


def _reference_data():
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
    import build_ref
    d = build_ref.default_src() / "tests" / "data"
    if not (d / "geo_flume.h5").is_file():
        pytest.skip("reference test data not present here")
    return d


def test_reference_mesh_file_matches_mesh_from_telemac_files():
    import cylag_gb300 as cg
    d = _reference_data()
    f = hdf5.read(d / "geo_flume.h5")
    fs = cg.EulerianFieldSet.from_telemac2d(str(d / "r2d_flume.slf"),
                                            bnd_file=str(d / "geo_flume.cli"))
    m = fs.triangular_mesh
    for k in ("x", "y", "triangles", "vertex_adjacency", "boundary_points", "boundary_edges",
              "vertex_labels", "signed_area", "gradx", "grady", "det", "triangle_centroids"):
        np.testing.assert_array_equal(f[k], np.asarray(getattr(m, k)), err_msg=k)
        assert f[k].dtype == np.asarray(getattr(m, k)).dtype, k
    assert int(f["nopen"][0]) == m.nopen
    # the same edges, numbered (max, min) in order in the file
    me = np.asarray(m.edges)
    key = {tuple(e): i for i, e in enumerate(me.tolist())}
    perm = np.array([key[tuple(sorted(e))] for e in f["edges"].tolist()])
    assert len(set(perm.tolist())) == len(me) == len(f["edges"])
    np.testing.assert_array_equal(me[perm][:, ::-1], f["edges"])
    np.testing.assert_array_equal(perm[f["triedge_map"]], np.asarray(m.triedge_map))
    np.testing.assert_array_equal(np.asarray(m.edgetri_map)[perm], f["edgetri_map"])
    np.testing.assert_array_equal(np.asarray(m.edges_labels)[perm], f["edges_labels"])


def test_mesh_from_reference_file_round_trips():
    from cylag_gb300.mesh import TriangularMesh
    d = _reference_data()
    f = hdf5.read(d / "geo_flume.h5")
    m = TriangularMesh.from_hdf5(str(d / "geo_flume.h5"))
    np.testing.assert_array_equal(np.asarray(m.edges), f["edges"])   # the file's numbering kept
    assert m.nopen == 2


def test_mesh_save_and_load(tmp_path):
    from cylag_gb300 import synth
    from cylag_gb300.mesh import TriangularMesh
    c = synth.couette_channel(npart=10)
    m = TriangularMesh(c["x"], c["y"], c["triangles"])
    m.save_mesh_hdf5(str(tmp_path / "m.h5"))
    f = hdf5.read(tmp_path / "m.h5")
    for k in TriangularMesh._HDF5_ARRAYS:
        np.testing.assert_array_equal(f[k], np.asarray(getattr(m, k)), err_msg=k)
        assert f[k].dtype == np.asarray(getattr(m, k)).dtype, k
    assert f["nopen"].dtype == np.int64 and int(f["nopen"][0]) == m.nopen
    back = TriangularMesh.from_hdf5(str(tmp_path / "m.h5"))
    for k in TriangularMesh._HDF5_ARRAYS:
        np.testing.assert_array_equal(np.asarray(getattr(back, k)), np.asarray(getattr(m, k)))


@pytest.mark.parametrize("dim", [2, 3])
def test_field_set_save_and_load(tmp_path, dim):
    import cylag_gb300 as cg
    from cylag_gb300 import synth
    from cylag_gb300.mesh import TriangularMesh
    if dim == 2:
        c = synth.keps_drift_channel(npart=10, nx=21, ny=11)
        c.update(dim=2, nlayers=1)
    else:
        c = synth.lsm2_loglaw_workload(npart=10, nx=21, ny=11, nplanes=4)
    mesh = TriangularMesh(c["x"], c["y"], c["triangles"])
    fs = cg.EulerianFieldSet(mesh, dim=c["dim"], nlayers=c["nlayers"], times=c["times"],
                             elevation=c["elevation"], velocity_x=c["velocity_x"],
                             velocity_y=c["velocity_y"], velocity_z=c.get("velocity_z"),
                             opt_fields=c.get("opt_fields"),
                             opt_fields_names=c.get("opt_fields_names"))
    fs.save_hdf5(str(tmp_path / "f.h5"), str(tmp_path / "m.h5"))
    raw = hdf5.read(tmp_path / "f.h5")
    assert raw["dim"].tolist() == [dim] and raw["nplan"].tolist() == [fs.nlayers]
    assert [n.decode() for n in raw["opt_fields_names"]] == list(fs.opt_fields_names)
    g = cg.EulerianFieldSet.from_hdf5(str(tmp_path / "f.h5"), str(tmp_path / "m.h5"))
    assert (g.dim, g.nlayers, g.nopt) == (fs.dim, fs.nlayers, fs.nopt)
    assert list(g.opt_fields_names) == list(fs.opt_fields_names)
    for k in ("times", "elevation", "velocity_x", "velocity_y", "opt_fields") + (
            ("velocity_z",) if dim == 3 else ()):
        np.testing.assert_array_equal(getattr(g, k), getattr(fs, k), err_msg=k)
    g2 = cg.EulerianFieldSet.from_hdf5(str(tmp_path / "f.h5"), str(tmp_path / "m.h5"),
                                       optional_fields=["A", "B"])
    assert g2.opt_fields_names == ["A", "B"]


def test_reader_refuses_what_it_does_not_read(tmp_path):
    p = tmp_path / "x.h5"
    p.write_bytes(b"not hdf5")
    with pytest.raises(ValueError, match="not an HDF5 file"):
        hdf5.read(p)
    hdf5.write(p, {"a": np.arange(3)})
    b = bytearray(p.read_bytes())
    b[8] = 2   # superblock version 2
    p.write_bytes(bytes(b))
    with pytest.raises(ValueError, match="superblock version 2"):
        hdf5.read(p)
