"""Checkpoint and resume (Solver.save_checkpoint / load_checkpoint over
cg_run_clock / cg_run_resume): a run checkpointed after N1 steps and resumed
in a new Solver -- built with another seed, so the streams must come from the
checkpoint -- takes the same N2 following steps as the uninterrupted run.
The cases have time-varying fields (the resumed run rebuilds the previous
field record for the Eulerian derivative of the added-mass acceleration)
and re-sorts at other steps than the uninterrupted run.  The plain form bit
for bit; the mixed form too (its FP32-pair working positions round-trip
through the FP64 arrays exactly but at rounding ties)."""
import numpy as np
import pytest

from conftest import fields_from_case, load_golden, mesh_from_case

pytestmark = pytest.mark.gpu

KEYS = ("position", "velocity", "fluid_velocity_seen", "tri", "lowerlayer", "inactive")


def _solver(case, meta, precision, seed):
    import cylag_gb300 as cg
    fs = cg.EulerianFieldSet(mesh_from_case(case), **fields_from_case(case))
    ps = cg.LagrangianParticleSet(case["position"], dim=case.get("dim", 2),
                                  **meta.get("pset", {}))
    return cg.Solver(fs, ps, meta["params"], precision=precision, seed=seed, sort_period=7), ps


def _state(ps):
    out = {k: np.array(getattr(ps, k)) for k in KEYS}
    out["tag"] = np.array(ps.tag)
    out["rng_state"] = ps._dev["rng_state"].cpu().numpy()
    return out


@pytest.mark.parametrize("name", ["keps_ts1_rm2", "lsm2_3d_di_opt3_keps_am",
                                  "lsm3_3d_di_keps_am"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_resume_continues_the_run(tmp_path, name, precision):
    case, meta, _ = load_golden(name)
    n1, n2 = 11, 16
    sa, pa = _solver(case, meta, precision, seed=meta["seed"])
    sa.forward(nsteps=n1)
    sa.save_checkpoint(str(tmp_path / "ck.npz"))
    sa.forward(nsteps=n2)
    want = _state(pa)
    sb, pb = _solver(case, meta, precision, seed=meta["seed"] + 12345)
    sb.load_checkpoint(str(tmp_path / "ck.npz"))
    assert sb.simutime.iteration == n1
    sb.forward(nsteps=n2)
    got = _state(pb)
    for k in want:
        np.testing.assert_array_equal(got[k], want[k], err_msg=f"{name} {precision}: {k}")
    assert sb.simutime.iteration == sa.simutime.iteration
    sa.close()
    sb.close()
