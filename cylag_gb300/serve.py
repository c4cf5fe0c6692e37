"""Serving many dispersion runs on one GPU (continuous batching).

A ``DispersionServer`` keeps one mesh and its frozen field records resident
in HBM and a pool of particle state; requests (a release set of particles,
a horizon in steps, LSM parameters and a PCG32 seed) are admitted as pool
memory frees up, every admitted run advances in the same launch each step
(one CUDA-graph replay per step, ``cg_server_step``), and a run's result is
copied back as soon as its horizon is reached.  Each request's result is the
result of the reference ``Solver`` for that release set alone
(cylag/core/solver.pyx:413-585 applied ``horizon`` times), whatever else
shares the pool.

``serve(requests)`` plays a schedule of timed arrivals in real time and
returns the per-request results and latencies (arrival to result on the
host).
"""
from __future__ import annotations

import ctypes as C
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .core import c_params, retag, upload_mesh_fields
from .parameters import Parameters


@dataclass
class Request:
    """One dispersion run: positions [n, 2] released at step 0, ``horizon``
    steps of the LSM given by ``parameters`` (the reference's parameter
    dict), particle-set keywords ``pset`` (particle_density,
    particle_diameter, drag_coefficient_model, ...), PCG32 ``seed``."""
    rid: int
    position: np.ndarray
    horizon: int
    parameters: dict
    seed: int = 0
    pset: dict = field(default_factory=dict)
    arrival: float = 0.0          # seconds after the start of serve()
    deadline: float | None = None  # seconds from admission to result, or none


@dataclass
class Result:
    rid: int
    position: np.ndarray
    velocity: np.ndarray
    fluid_velocity_seen: np.ndarray
    tri: np.ndarray
    tag: np.ndarray
    inactive: np.ndarray
    arrival: float = 0.0
    admitted: float = 0.0
    finished: float = 0.0
    error: str | None = None      # set when the run was cancelled (no state)

    @property
    def latency(self):
        return self.finished - self.arrival


class DispersionServer:
    """Pool of ``capacity`` particles on ``field_set`` (2D, frozen fields).

    precision: "fp64" (plain) or "mixed"; schmidt_number: the one of the
    nodal k-epsilon diffusivity (LSM1 k-epsilon runs must use it)."""

    def __init__(self, field_set, precision="mixed", capacity=64 << 20, max_runs=4096,
                 device=0, hbm_budget=0, schmidt_number=1.0):
        if field_set.dim != 2:
            raise NotImplementedError("the serving pool steps 2D runs")
        self.prec = {"fp64": _lib.CG_PRECISION_FP64, "plain": _lib.CG_PRECISION_FP64,
                     "mixed": _lib.CG_PRECISION_MIXED}[precision]
        self.field_set = field_set
        self.L = _lib.load()
        self._ctx = C.c_void_p()
        _lib.check(None, self.L.cg_ctx_create(device, int(hbm_budget), C.byref(self._ctx)))
        self._keep = upload_mesh_fields(self.L, self._ctx, field_set)
        self._srv = C.c_void_p()
        _lib.check(self._ctx, self.L.cg_server_create(self._ctx, self.prec, int(capacity),
                                                      int(max_runs), float(schmidt_number),
                                                      C.byref(self._srv)))
        self.runs = {}      # run id -> (request, admitted wall time)

    # ---- one run ------------------------------------------------------------
    def admit(self, req: Request, now: float = 0.0):
        """Admits a request; False when the pool has no room for it yet."""
        P = Parameters(dict(req.parameters, frozen_eulerian_fields=True))
        P.check_values()
        ps = dict(req.pset)
        prm = c_params(P, 2, ps.get("particle_density", 1000.),
                       ps.get("drag_coefficient_model", 1), ps.get("drag_coefficient", 0.44),
                       ps.get("added_mass_force", False), ps.get("added_mass_coef", 0.5),
                       ps.get("buoyancy_velocity_model", 0), ps.get("buoyancy_velocity", 0.0),
                       self.prec, req.seed, 0)
        pos = np.ascontiguousarray(req.position, dtype=np.float64)
        diam = ps.get("diameter")
        diam = None if diam is None else np.ascontiguousarray(diam, dtype=np.float64)
        rid = C.c_int32(-1)
        rc = self.L.cg_server_admit(self._srv, C.byref(prm), len(pos), pos.ctypes.data,
                                    float(ps.get("particle_diameter", 0.01)),
                                    None if diam is None else diam.ctypes.data,
                                    int(req.horizon), C.byref(rid))
        if rc == _lib.CG_ENOMEM_BUDGET:
            return False
        _lib.check(self._ctx, rc)
        self.runs[rid.value] = (req, now)
        return True

    def step(self, nsteps=1):
        _lib.check(self._ctx, self.L.cg_server_step(self._srv, int(nsteps)))

    def steps_left(self, run_id):
        left = C.c_int32()
        _lib.check(self._ctx, self.L.cg_server_run_status(self._srv, run_id, C.byref(left)))
        return left.value

    def finished(self):
        """Runs whose last step has been queued."""
        return [r for r in self.runs if self.steps_left(r) == 0]

    def collect(self, run_ids=None, now_fn=None):
        """Reads and releases the given finished runs (default: all)."""
        out = []
        for run_id in (self.finished() if run_ids is None else run_ids):
            req, t_adm = self.runs.pop(run_id)
            n = len(req.position)
            pos = np.empty((n, 2))
            vel = np.empty((n, 2))
            fvs = np.empty((n, 2))
            tri = np.empty(n, np.int32)
            tag = np.empty(n, np.int32)
            flags = C.c_uint32()
            rc = self.L.cg_server_read(self._srv, run_id, pos.ctypes.data, vel.ctypes.data,
                                       fvs.ctypes.data, tri.ctypes.data, tag.ctypes.data, None,
                                       C.byref(flags))
            _lib.check(self._ctx, self.L.cg_server_release(self._srv, run_id))
            _lib.check(self._ctx, rc)
            tag, _ = retag(tag, n - 1)
            t = now_fn() if now_fn else 0.0
            out.append(Result(req.rid, pos, vel, fvs, tri, tag, (tri == -1).astype(np.int32),
                              req.arrival, t_adm, t))
        return out

    def cancel(self, run_id):
        """Drops a run before its horizon (its range is reused after the
        steps already queued)."""
        _lib.check(self._ctx, self.L.cg_server_release(self._srv, run_id))
        self.runs.pop(run_id)

    def expire(self, now):
        """The watchdog: cancels every run whose request has a deadline that
        passed (``now`` - admission > deadline) before its last step was
        queued, and returns an error result for each (no particle state)."""
        out = []
        for run_id, (req, t_adm) in list(self.runs.items()):
            if req.deadline is None or now - t_adm <= req.deadline:
                continue
            if self.steps_left(run_id) == 0:
                continue   # finished: its result is collected as usual
            self.cancel(run_id)
            e = np.zeros((0, 2))
            ei = np.zeros(0, np.int32)
            out.append(Result(req.rid, e, e, e, ei, ei, ei, req.arrival, t_adm, now,
                              error=f"deadline of {req.deadline:g} s exceeded after "
                                    f"{now - t_adm:.3f} s"))
        return out

    def stats(self):
        ar, ap, lf, si, ms = C.c_int32(), C.c_int64(), C.c_int64(), C.c_int64(), C.c_double()
        _lib.check(self._ctx, self.L.cg_server_stats(self._srv, C.byref(ar), C.byref(ap),
                                                     C.byref(lf), C.byref(si), C.byref(ms)))
        return dict(active_runs=ar.value, active_particles=ap.value,
                    largest_free_range=lf.value, steps_issued=si.value, last_step_ms=ms.value)

    # ---- a schedule of arrivals ---------------------------------------------------
    def serve(self, requests, realtime=True, chunk=32, log=None, clock=None):
        """Plays the requests (sorted by arrival) and returns their results in
        completion order.  Each loop admits what has arrived and fits (in
        arrival order), queues up to ``chunk`` steps (fewer when a run
        completes earlier), then reads back the runs finished by the previous
        queue, which overlaps the copies with the steps on the GPU, and
        cancels the runs whose deadline passed (``expire``).  ``clock``:
        seconds since the start (default: the wall clock)."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        t0 = time.perf_counter()
        if clock is None:
            clock = (lambda: time.perf_counter() - t0)
        now = clock if realtime else (lambda: float("inf"))
        pending = deque()
        results = []
        i = 0
        while i < len(reqs) or pending or self.runs:
            t = now()
            while i < len(reqs) and reqs[i].arrival <= t:
                pending.append(reqs[i])
                i += 1
            while pending and self.admit(pending[0], clock()):
                pending.popleft()
            if self.runs:
                done = self.finished()
                todo = [x for x in (self.steps_left(r) for r in self.runs) if x > 0]
                if todo:
                    self.step(min(chunk, min(todo)))
                # runs finished by earlier queues: their copies overlap these steps
                results.extend(self.collect(done, clock))
                results.extend(self.expire(clock()))
            elif pending:
                # nothing runs, so nothing will free room for it
                raise RuntimeError(f"request {pending[0].rid} does not fit in an empty pool")
            elif i < len(reqs):
                time.sleep(max(0.0, min(reqs[i].arrival - now(), 0.05)))
            if log and results and len(results) % 50 == 0:
                log(f"{len(results)} done, {len(self.runs)} active, {len(pending)} waiting")
        return results

    def close(self):
        if self._srv:
            self.L.cg_server_destroy(self._srv)
            self._srv = C.c_void_p()
        if self._ctx:
            self.L.cg_ctx_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# the serving mix: Poisson arrivals on the Couette channel
# ---------------------------------------------------------------------------
LSM1_PARAMS = {"model": 1, "diffusion_model": 1, "horizontal_diffusivity": 0.01,
               "time_scheme": 1, "time_step": 1.0, "frozen_eulerian_fields": True}
LSM2_PARAMS = {"model": 2, "diffusion_model": 1, "horizontal_diffusivity": 0.01,
               "time_scheme": 5, "time_step": 1.0, "frozen_eulerian_fields": True}


def disc(rng, n, cx, cy, r):
    rr = r * np.sqrt(rng.uniform(0.0, 1.0, n))
    th = rng.uniform(0.0, 2 * np.pi, n)
    return np.stack([cx + rr * np.cos(th), cy + rr * np.sin(th)], axis=1)


def poisson_mix(rate=10.0, duration=60.0, seed=5, lx=1000.0, ly=100.0, nmin=1e3, nmax=1e6,
                hmin=100, hmax=5000, scale_particles=1.0):
    """Poisson arrivals (``rate`` per s for ``duration`` s); each request a
    disc release (centre uniform in the lx x ly channel, radius U[0, 50] m),
    log-uniform particle count in [nmin, nmax] (times ``scale_particles``),
    horizon U[hmin, hmax] steps at dt = 1 s, LSM1 or LSM2 with probability
    1/2 (reference particle defaults), its own PCG32 seed."""
    rng = np.random.default_rng(seed)
    t, reqs = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        k = len(reqs)
        n = max(1, int(round(10 ** rng.uniform(np.log10(nmin), np.log10(nmax)) * scale_particles)))
        cx, cy, r = rng.uniform(0, lx), rng.uniform(0, ly), rng.uniform(0, 50.0)
        horizon = int(rng.integers(hmin, hmax + 1))
        params = dict(LSM1_PARAMS if rng.uniform() < 0.5 else LSM2_PARAMS)
        params["final_time"] = horizon * params["time_step"]
        pos = disc(np.random.default_rng([seed, k]), n, cx, cy, r)
        reqs.append(Request(k, pos, horizon, params, seed=int(rng.integers(0, 2**62)),
                            arrival=t))
    return reqs
