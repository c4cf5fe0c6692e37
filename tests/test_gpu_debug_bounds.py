"""The bounds-checked build (CYLAG_DEBUG_BOUNDS=1 loads
libcylag_gpu_debug.so: every gather index from the mesh tables or the
particle state range-checked in the kernels, out-of-range ones flagged as
CG_ERR_BOUNDS and redirected in bounds, nothing traps).  On well-formed runs
it must change nothing: the same fixtures, stepped through both builds,
give bit-identical states and no error flag (a flag would make the step
call fail)."""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, load_golden

pytestmark = pytest.mark.gpu

NAMES = ["open", "3d_keps", "lsm2_3d_di_opt3_keps_am", "p3d_unsteady_keps3_ts4"]

_CHILD = """
import sys, numpy as np
sys.path[:0] = [sys.argv[2], sys.argv[2] + "/tests", sys.argv[2] + "/oracle"]
from test_gpu_parity import gpu_run, state
from conftest import load_golden
out = {}
for name in sys.argv[3:]:
    for prec in ("fp64", "mixed"):
        case, meta, _ = load_golden(name)
        s, ps = gpu_run(case, meta, precision=prec, batch=9)
        st = state(ps)
        for k in ("position", "tri", "inactive"):
            out[f"{name}:{prec}:{k}"] = np.asarray(st[k])
        s.close()
np.savez(sys.argv[1], **out)
"""


def _names():
    from conftest import golden_names
    have = set(golden_names())
    return [n for n in NAMES if n in have]


def test_bounds_checked_build_changes_nothing(tmp_path):
    names = _names()
    outs = {}
    for mode in ("normal", "checked"):
        env = dict(os.environ)
        env.pop("CYLAG_DEBUG_BOUNDS", None)
        if mode == "checked":
            env["CYLAG_DEBUG_BOUNDS"] = "1"
        f = tmp_path / f"{mode}.npz"
        r = subprocess.run([sys.executable, "-c", _CHILD, str(f), str(ROOT), *names], env=env,
                           capture_output=True, text=True, timeout=1200)
        assert r.returncode == 0, r.stderr[-3000:]
        outs[mode] = np.load(f)
    a, b = outs["normal"], outs["checked"]
    assert sorted(a.files) == sorted(b.files) and len(a.files) == 6 * len(names)
    for k in a.files:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
