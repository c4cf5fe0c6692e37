"""Control sections and stranding output in the GPU step, against the
reference (tests/golden/sec_*.npz): per-step section counts and exit counts
bit-exact, stranded positions in the reference's order (1e-10), final state
as in the other parity tests; with and without the element sort, in one
call or several; the statistics files written by solve()."""
import numpy as np
import pytest

from conftest import (RTOL, assert_state_close, fields_from_case, load_golden, mesh_from_case,
                      section_names)

pytestmark = pytest.mark.gpu


def _run(case, meta, tmp_path, precision="fp64", sort_period=0, batch=None, solve=False):
    import cylag_gb300 as cg
    from cylag_gb300.extra import ControlSection
    f = fields_from_case(case)
    fs = cg.EulerianFieldSet(mesh_from_case(case), **f)
    ps = cg.LagrangianParticleSet(case["position"], dim=f["dim"], **meta.get("pset", {}))
    params = dict(meta["params"], output_rep=str(tmp_path))
    cs = [ControlSection(np.array(q)) for q in meta["sections"]]
    s = cg.Solver(fs, ps, params, control_sections=cs, precision=precision, seed=meta["seed"],
                  sort_period=sort_period)
    n = meta["nsteps"]
    if solve:
        s.forward(nsteps=n)
        s.flush_statistics()
    else:
        done = 0
        while done < n:
            k = n - done if batch is None else min(batch, n - done)
            s.forward(nsteps=k)
            done += k
    st = dict(position=ps.position, velocity=ps.velocity,
              fluid_velocity_seen=ps.fluid_velocity_seen, tri=ps.tri, inactive=ps.inactive,
              lowerlayer=ps.lowerlayer, last_position=ps.last_position)
    out = dict(state=st, csec=s.section_statistics(), bnd=s.bnd_statistics(),
               stranded=ps.stranded_positions[:ps.stranded_count].copy())
    s.close()
    return out


@pytest.mark.parametrize("sort_period,batch", [(0, None), (10, None), (0, 13), (7, 40)])
@pytest.mark.parametrize("name", section_names())
def test_gpu_sections_and_stranding_match_reference(name, sort_period, batch, tmp_path):
    case, meta, want = load_golden(name, prefix="sec")
    got = _run(case, meta, tmp_path, sort_period=sort_period, batch=batch)
    what = f"{name} sort={sort_period} batch={batch}"
    assert_state_close(got["state"], want, rtol=RTOL, what=what)
    np.testing.assert_array_equal(got["csec"], want["csec_stats"], err_msg=what)
    if meta["params"].get("bnd_statistics"):
        np.testing.assert_array_equal(got["bnd"], want["bnd_stats"], err_msg=what)
    assert got["stranded"].shape == want["stranded"].shape, what
    np.testing.assert_allclose(got["stranded"], want["stranded"], rtol=RTOL, atol=RTOL)


def test_statistics_files_written(tmp_path):
    name = "open_lsm1"
    case, meta, want = load_golden(name, prefix="sec")
    _run(case, meta, tmp_path, solve=True)
    times = meta["params"]["time_step"] * np.arange(meta["nsteps"])
    for c in range(want["csec_stats"].shape[1]):
        lines = (tmp_path / f"cs_stats_{c + 1}.txt").read_text().splitlines()
        assert lines[0] == "cylag control section file"
        rows = np.array([[float(v) for v in ln.split(",")] for ln in lines[2:]])
        np.testing.assert_array_equal(rows[:, 0], times)
        np.testing.assert_array_equal(rows[:, 1], want["csec_stats"][:, c])
    st = np.loadtxt(tmp_path / "stranded_particles.txt", delimiter=",", skiprows=2, ndmin=2)
    np.testing.assert_allclose(st, want["stranded"], rtol=RTOL, atol=RTOL)


def test_mixed_sections_follow_plain(tmp_path):
    case, meta, want = load_golden("open_lsm1_rk4", prefix="sec")
    got = _run(case, meta, tmp_path, precision="mixed", sort_period=10)
    tot, ref = got["csec"].sum(0), want["csec_stats"].sum(0)
    assert np.all(np.abs(tot - ref) <= np.maximum(2, 0.05 * ref)), (tot, ref)


def _read_txt_blocks(path):
    lines = path.read_text().splitlines()
    assert lines[0] == "cylag particles result file"
    blocks, k = [], 2
    while k < len(lines):
        head = lines[k]
        t = float(head.split("Time =")[1].split(",")[0])
        it = int(head.split("Iter =")[1].split(",")[0])
        n = int(head.split("Npart =")[1])
        rows = np.array([[float(v) for v in ln.split(",")[:-1]] for ln in lines[k + 1:k + 1 + n]])
        blocks.append((t, it, rows.reshape(n, -1)))
        k += 1 + n
    return blocks


def test_solver_snapshots(tmp_path):
    """output_file: the initial snapshot and one every output_printout_period
    iterations, in one forward call that the snapshots split; the last
    block is the final state (tags, positions to 1e-10 of the reference)."""
    import cylag_gb300 as cg
    from conftest import golden_names  # noqa: F401
    case, meta, want = load_golden("couette")
    f = fields_from_case(case)
    fs = cg.EulerianFieldSet(mesh_from_case(case), **f)
    ps = cg.LagrangianParticleSet(case["position"], dim=2)
    params = dict(meta["params"], output_file=True, output_file_format="all",
                  output_printout_period=50, output_rep=str(tmp_path))
    s = cg.Solver(fs, ps, params, seed=meta["seed"], sort_period=20)
    s.forward(nsteps=meta["nsteps"])
    s.flush_statistics()
    s._snapshots.wait()
    blocks = _read_txt_blocks(tmp_path / "particles.txt")
    its = [b[1] for b in blocks]
    assert its == list(range(0, meta["nsteps"] + 1, 50))
    t, it, rows = blocks[-1]
    assert it == meta["nsteps"]
    act = want["inactive"] == 0
    np.testing.assert_array_equal(rows[:, 0].astype(int), ps.tag[act])
    np.testing.assert_allclose(rows[:, 1:3], want["position"][act], rtol=RTOL, atol=1e-9)
    for k in its:
        assert (tmp_path / f"particles_{k}.vtk").exists()
    s.close()
