"""TELEMAC inputs without TELEMAC: the Selafin reader against files written
in the published layout (2D and 3D, FP32 and FP64 values), field sets built
from them, and the .cli reader against the reference's read_cli."""
import numpy as np
import pytest


def _channel():
    from cylag_gb300 import synth
    return synth.channel_mesh(400.0, 100.0, 21, 6, seed=1)


@pytest.mark.parametrize("double", [False, True])
def test_selafin_2d_round_trip_and_field_set(tmp_path, double):
    import cylag_gb300 as cg
    from cylag_gb300.telemac import SelafinFile, write_selafin
    x, y, tri = _channel()
    rng = np.random.default_rng(0)
    times = np.array([100.0, 700.0, 1300.0])
    names = ["VELOCITY U", "VELOCITY V", "FREE SURFACE", "TURBULENT ENERG.", "DISSIPATION"]
    vals = [[rng.normal(0, 1, len(x)) for _ in names] for _ in times]
    f = tmp_path / "r2d.slf"
    write_selafin(f, x, y, tri, times, vals, names, double=double)
    r = SelafinFile(f)
    assert r.varnames == names and r.nplan == 1 and r.ntimestep == 3
    np.testing.assert_array_equal(r.ikle2, tri)
    cast = (lambda a: a) if double else (lambda a: np.asarray(a, np.float32).astype(np.float64))
    np.testing.assert_array_equal(r.x, cast(x))
    np.testing.assert_array_equal(r.times, times)
    np.testing.assert_array_equal(r.get_data_value("FREE SURFACE", 2), cast(vals[2][2]))
    fs = cg.EulerianFieldSet.from_telemac2d(
        str(f), optional_fields=["TURBULENT ENERG.", "DISSIPATION"])
    assert fs.dim == 2 and fs.ntimes == 3 and fs.fid_turbeng == 4 and fs.fid_dissip == 5
    np.testing.assert_array_equal(fs.times, times - times[0])
    np.testing.assert_array_equal(fs.velocity_y[1], cast(vals[1][1]))
    np.testing.assert_array_equal(fs.elevation[0], cast(vals[0][2]))


def test_selafin_3d_layers(tmp_path):
    import cylag_gb300 as cg
    from cylag_gb300.telemac import SelafinFile, write_selafin
    x, y, tri = _channel()
    nplan, n2 = 4, len(x)
    zb = -5.0 - 0.01 * x
    z = np.concatenate([zb + (0.0 - zb) * p / (nplan - 1) for p in range(nplan)])
    u = np.linspace(0.1, 0.4, nplan * n2)
    vals = [[z, u, 0.5 * u, 0.0 * u] for _ in range(2)]
    f = tmp_path / "r3d.slf"
    names = ["ELEVATION Z", "VELOCITY U", "VELOCITY V", "VELOCITY W"]
    write_selafin(f, x, y, tri, [0.0, 60.0], vals, names, nplan=nplan, double=True)
    r = SelafinFile(f)
    assert r.nplan == nplan and r.npoin2 == n2 and r.npoin3 == nplan * n2
    np.testing.assert_array_equal(r.ikle2, tri)
    fs = cg.EulerianFieldSet.from_telemac3d(str(f))
    assert fs.dim == 3 and fs.nlayers == nplan
    np.testing.assert_array_equal(fs.elevation[1], z)
    np.testing.assert_array_equal(fs.velocity_x[0], u)


def test_read_cli_matches_reference(tmp_path):
    import refpath
    if not refpath.available():
        pytest.skip("compiled reference not built here")
    cy = refpath.use_reference()
    import importlib
    R = importlib.import_module("cylag.geom.read_cli")
    from cylag_gb300.telemac import read_cli
    # an open boundary cut by the start/end of the list, a wall, another
    # open boundary, walls
    labels = [5, 5, 2, 2, 2, 4, 4, 2, 2, 5]
    lines = []
    for k, lab in enumerate(labels):
        code = "2 2 2" if lab == 2 else f"{lab} {lab} {lab}"
        lines.append(f"{code} 0.0 0.0 0.0 0.0 2 0.0 0.0 0.0 {100 + 3 * k} {k + 1}")
    f = tmp_path / "b.cli"
    f.write_text("\n".join(lines) + "\n\n")
    a, na = read_cli(str(f))
    b, nb = R.read_cli(str(f))
    np.testing.assert_array_equal(a, np.asarray(b))
    assert na == nb
