"""The serving pool's host-side schedule (DispersionServer.serve), on CPU:
the device pool is replaced by a model of it (capacity in particles, steps
left per run), so the admission order, the step chunks and the collection
of finished runs are checked without a GPU."""
import numpy as np
import pytest

from cylag_gb300.serve import DispersionServer, Request, Result


class PoolModel(DispersionServer):
    """A pool of `capacity` particles; a run holds its particles from
    admission to collection and finishes after `horizon` queued steps."""

    def __init__(self, capacity):
        self.capacity = capacity
        self.used = 0
        self.runs = {}
        self.left = {}
        self.next_id = 0
        self.admitted = []   # request ids in admission order
        self.chunks = []     # (steps queued, smallest steps left among active runs)

    def admit(self, req, now=0.0):
        n = len(req.position)
        if self.used + n > self.capacity:
            return False
        rid = self.next_id
        self.next_id += 1
        self.used += n
        self.runs[rid] = (req, now)
        self.left[rid] = req.horizon
        self.admitted.append(req.rid)
        return True

    def step(self, nsteps=1):
        active = [v for v in self.left.values() if v > 0]
        self.chunks.append((nsteps, min(active)))
        for r in self.left:
            self.left[r] = max(0, self.left[r] - nsteps)

    def steps_left(self, run_id):
        return self.left[run_id]

    def collect(self, run_ids=None, now_fn=None):
        out = []
        for rid in (self.finished() if run_ids is None else run_ids):
            req, t_adm = self.runs.pop(rid)
            del self.left[rid]
            n = len(req.position)
            self.used -= n
            z = np.zeros((n, 2))
            zi = np.zeros(n, np.int32)
            out.append(Result(req.rid, z, z, z, zi, zi, zi, req.arrival, t_adm, 0.0))
        return out

    def close(self):
        pass


def _requests(sizes, horizons):
    return [Request(k, np.zeros((n, 2)), h, {"model": 1}, seed=k, arrival=0.01 * k)
            for k, (n, h) in enumerate(zip(sizes, horizons))]


def test_schedule_admits_in_arrival_order_and_finishes_every_run():
    rng = np.random.default_rng(0)
    sizes = rng.integers(1, 400, 60)
    horizons = rng.integers(1, 120, 60)
    reqs = _requests(sizes, horizons)
    pool = PoolModel(capacity=1000)
    res = pool.serve(reqs, realtime=False, chunk=16)
    assert sorted(r.rid for r in res) == list(range(60))
    # first come, first admitted: a request that does not fit holds the later ones
    assert pool.admitted == list(range(60))
    assert pool.used == 0 and not pool.runs
    # a queue of steps never runs past the first active run to finish
    for k, smallest in pool.chunks:
        assert 1 <= k <= min(16, smallest)


def test_schedule_never_overfills_the_pool():
    reqs = _requests([600, 500, 400, 300], [5, 3, 8, 2])
    pool = PoolModel(capacity=1000)
    seen = []
    step = pool.step

    def step_and_check(nsteps=1):
        seen.append(pool.used)
        step(nsteps)

    pool.step = step_and_check
    res = pool.serve(reqs, realtime=False, chunk=32)
    assert len(res) == 4 and max(seen) <= 1000
    assert pool.admitted == [0, 1, 2, 3]


def test_schedule_refuses_a_request_larger_than_the_pool():
    reqs = _requests([10, 5000], [3, 3])
    with pytest.raises(RuntimeError, match="does not fit in an empty pool"):
        PoolModel(capacity=1000).serve(reqs, realtime=False)


class ClockedPool(PoolModel):
    """The pool model with a fake clock that each queued step advances by
    `dt` seconds, and cancellation that frees the run's particles."""

    def __init__(self, capacity, dt):
        super().__init__(capacity)
        self.t = 0.0
        self.dt = dt
        self.cancelled = []

    def step(self, nsteps=1):
        super().step(nsteps)
        self.t += self.dt * nsteps

    def cancel(self, run_id):
        req, _ = self.runs.pop(run_id)
        del self.left[run_id]
        self.used -= len(req.position)
        self.cancelled.append(req.rid)


def test_watchdog_cancels_runs_past_their_deadline():
    """A run whose deadline passes before its last step is queued is
    cancelled (its pool range freed) and returned as an error result; runs
    that finish in time, or have no deadline, complete as usual; a request
    waiting for room is admitted once the cancelled run frees it."""
    reqs = _requests([300, 300, 600], [400, 20, 30])
    reqs[0].deadline = 5.0      # 400 steps at 0.1 s: cannot finish in 5 s
    reqs[1].deadline = 5.0      # 20 steps: finishes in 2 s
    pool = ClockedPool(capacity=700, dt=0.1)
    res = pool.serve(reqs, realtime=False, chunk=8, clock=lambda: pool.t)
    by = {r.rid: r for r in res}
    assert sorted(by) == [0, 1, 2]
    assert pool.cancelled == [0]
    assert by[0].error and "deadline" in by[0].error and len(by[0].position) == 0
    assert 5.0 < by[0].finished - by[0].admitted <= 5.0 + 8 * 0.1 + 1e-9
    assert by[1].error is None and by[2].error is None
    assert pool.admitted == [0, 1, 2] and pool.used == 0
