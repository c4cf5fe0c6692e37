"""Control sections and stranding output, checked without a GPU.

* the oracle reproduces the reference's per-step control-section counts
  (first segment of each polyline; a particle deleted in the step counts
  for a section through the origin), the stranded positions in the
  reference's order and the final state (tests/golden/sec_*.npz);
* the statistics files are byte-identical to the reference writers' when
  the compiled reference is present.
"""
import numpy as np
import pytest

from conftest import X86, assert_state_close, load_golden, run_oracle, section_names


@pytest.mark.parametrize("name", section_names())
def test_oracle_sections_and_stranding_match_reference(oracle_lib, name):
    case, meta, want = load_golden(name, prefix="sec")
    o = run_oracle(case, meta, nthreads=4)
    got = dict(position=o.pos, velocity=o.vel, fluid_velocity_seen=o.fvs, tri=o.tri,
               inactive=o.inactive, lowerlayer=o.lowerlayer, last_position=o.last_pos)
    assert_state_close(got, want, exact=X86, what=name)
    np.testing.assert_array_equal(np.stack(o.section_stats), want["csec_stats"])
    st = np.array(o.stranded).reshape(-1, 3)
    assert st.shape == want["stranded"].shape
    if X86:
        np.testing.assert_array_equal(st, want["stranded"])
    else:
        np.testing.assert_allclose(st, want["stranded"], rtol=1e-10, atol=1e-10)


def test_control_section_tests_first_segment_only():
    from cylag_gb300.extra import ControlSection, section_segments
    cs = ControlSection(np.array([[0., 0.], [1., 0.], [1., 1.]]))
    assert cs.nseg == 1
    assert cs.cross([0.5, -1.], [0.5, 1.]) == 1
    assert cs.cross([2., 0.5], [0., 0.5]) == 0       # crosses only the second segment
    seg = section_segments([cs, ControlSection(np.zeros((3, 1)))])
    np.testing.assert_array_equal(seg[0], [0., 0., 1., 0.])
    assert np.isnan(seg[1]).all()


def _ref():
    import refpath
    if not refpath.available():
        pytest.skip("compiled reference not built here")
    return refpath.use_reference()


def test_statistics_files_match_reference_writers(tmp_path):
    _ref()
    import importlib
    W = importlib.import_module("cylag.io.write_statistics")
    WP = importlib.import_module("cylag.io.write_particles")
    from cylag_gb300 import statistics as S
    times = np.array([0.0, 0.5, 1.25, 3.0])
    data = np.array([[0, 3], [12, 0], [7, 123456], [0, 1]], dtype=np.int32)
    xyz = np.array([[1.5, -2.25, 0.0], [1e-9, 3e7, -4.125]])
    for root, mod in ((tmp_path / "ref", W), (tmp_path / "ours", S)):
        mod.prepare_secstats_output(True, 2, str(root), "bnd_stats", True, 2, "cs_stats")
        mod.write_secstats_buffer(times, data, 4, 2, str(root), "bnd_stats")
        mod.write_secstats_buffer(times[:2], data[:2], 2, 2, str(root), "cs_stats")
    WP.write_stranded_particles_txt_2d(1, -1, str(tmp_path / "ref"), "stranded", xyz, 2)
    S.write_stranded_particles_txt_2d(str(tmp_path / "ours"), "stranded", xyz, 2)
    names = sorted(p.name for p in (tmp_path / "ref").iterdir())
    assert names == sorted(p.name for p in (tmp_path / "ours").iterdir())
    for n in names:
        assert (tmp_path / "ref" / n).read_bytes() == (tmp_path / "ours" / n).read_bytes(), n
