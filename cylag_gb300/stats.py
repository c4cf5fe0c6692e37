"""Error report of a run against a reference run (the FP64 oracle or the
plain form): the quantities the mixed-precision form states.

* per-particle displacement RMS difference;
* ensemble mean and variance of the displacement, and their relative
  differences;
* for pure diffusion, the deviation of the spread from 2 K t.

Inputs are numpy arrays; ensemble reductions are done in FP64 with pairwise
(numpy) summation.
"""
from __future__ import annotations

import numpy as np


def displacement_report(x0, xa, xb, active=None):
    """x0: start positions [n, d]; xa, xb: end positions of the run under test
    and of the reference run; active: mask of particles active in both."""
    x0 = np.asarray(x0, dtype=np.float64)
    da = np.asarray(xa, dtype=np.float64) - x0
    db = np.asarray(xb, dtype=np.float64) - x0
    if active is not None:
        da, db = da[active], db[active]
    n = da.shape[0]
    rms = float(np.sqrt(np.mean(np.sum((da - db) ** 2, axis=1)))) if n else 0.0
    ma, mb = da.mean(axis=0), db.mean(axis=0)
    va, vb = da.var(axis=0), db.var(axis=0)
    scale_m = np.maximum(np.sqrt(vb), 1e-300)
    return {
        "n": int(n),
        "rms_displacement_diff": rms,
        "mean": ma.tolist(), "mean_ref": mb.tolist(),
        # mean difference in units of the reference spread
        "mean_rel_err": (np.abs(ma - mb) / scale_m).tolist(),
        "var": va.tolist(), "var_ref": vb.tolist(),
        "var_rel_err": (np.abs(va - vb) / np.maximum(vb, 1e-300)).tolist(),
    }


def diffusion_report(x0, x, K, t, active=None):
    """Spread of a pure-diffusion run vs the analytic 2 K t per axis."""
    d = np.asarray(x, dtype=np.float64) - np.asarray(x0, dtype=np.float64)
    if active is not None:
        d = d[active]
    var = d.var(axis=0)
    exact = 2.0 * K * t
    n = d.shape[0]
    # standard error of a sample variance of Gaussian data: var * sqrt(2/(n-1))
    se = exact * np.sqrt(2.0 / max(n - 1, 1))
    return {"n": int(n), "var": var.tolist(), "var_exact": float(exact),
            "rel_dev": ((var - exact) / exact).tolist(), "z": ((var - exact) / se).tolist()}
