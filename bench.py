"""Throughput benchmark of the GPU particle step (particle-steps/s).

Workload (default, --workload lsm1_2d): LSM1 2D with k-epsilon
diffusivity-gradient drift at scale -- 4 km x 1 km jittered mesh (1001x251
vertices, 500,000 triangles), node fields interpolated in time between
records 600 s apart, 1e7 particles uniform in the domain, dt = 0.5 s.
Other workloads: lsm2_3d (LSM2 Langevin, direct integrator, k-epsilon
velocity diffusion in the 3D log-law channel: 2e5 triangles x 21 sigma
planes, 4e6 particles, dt = 0.1 s) and lsm3_3d (LSM3 polydisperse settling
in a Taylor-Green vortex on the same mesh, 1e7 particles, dt = 0.2 s).
One step = one Solver.forward over all particles (time interpolation of
the fields + the fused particle kernel).  Inputs are synthetic
(cylag_gb300.synth, seeded); the particle state is larger than L2, so no
flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp64|mixed]
                  [--workload lsm1_2d|lsm2_3d|lsm3_3d]
  python bench.py --impl reference ...   # the CPU implementation, host cores

Prints one JSON line (rank 0).  Under torchrun the particle set holds
N x 1e7 particles and each rank advances its share, split as the reference's
parallel solver splits particles (weak scaling, no data-path collective; the
timed region is the max over ranks).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "particle-steps/s on 1 GB300 (mixed vs plain FP64); p50/p99 request latency"
UNIT = "particle-steps/s"
WORKLOADS = {
    "serve": "serving_mix_couette_channel_poisson_10_per_s_60_s_lsm1_lsm2",
    "lsm1_2d": "lsm1_2d_keps_drift_500k_tri_1e7_particles",
    "lsm2_3d": "lsm2_3d_loglaw_di_keps_200k_tri_21_planes_4e6_particles",
    "lsm3_3d": "lsm3_3d_taylor_green_settling_200k_tri_21_planes_1e7_particles",
}


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: 1000 for lsm1_2d, one call over half of its "
                         "2,000-step horizon, so that warm-up, timed and end-to-end steps stay "
                         "within its field records; 100 for the others)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--precision", choices=["both", "fp64", "mixed"], default="both")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="lsm1_2d")
    ap.add_argument("--npart", type=int, default=None,
                    help="particles per GPU (default: the workload's own count)")
    ap.add_argument("--nx", type=int, default=None)
    ap.add_argument("--ny", type=int, default=None)
    ap.add_argument("--sort-period", type=int, default=25,
                    help="steps between re-sorts of the particles by element (0: never)")
    ap.add_argument("--serve-rate", type=float, default=10.0, help="requests per s (serve)")
    ap.add_argument("--serve-duration", type=float, default=60.0, help="arrival window, s (serve)")
    ap.add_argument("--serve-chunk", type=int, default=32, help="steps queued per loop (serve)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-oracle-error", action="store_true",
                    help="skip the mixed form's error against the FP64 oracle subsample")
    ap.add_argument("--legs", type=int, default=1,
                    help="also measure the LSM2 3D, LSM3 3D and serving legs (default line only)")
    ap.add_argument("--leg-steps", type=int, default=20, help="timed steps of each 3D leg")
    ap.add_argument("--leg-serve-duration", type=float, default=10.0,
                    help="arrival window of the serving leg, s")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--e2e-chunk", type=int, default=0,
                    help="particles per copy/step chunk of the end-to-end steps (0: the library's "
                         "default, four chunks)")
    args = ap.parse_args(argv)
    if args.steps is None:
        args.steps = 1000 if args.workload == "lsm1_2d" else 100
    return args


_T0 = time.perf_counter()


def log(msg):
    """Phase log on stderr (the JSON line alone goes to stdout)."""
    if os.environ.get("CYLAG_BENCH_QUIET") != "1":
        print(f"[bench {time.perf_counter() - _T0:8.2f}s] {msg}", file=sys.stderr, flush=True)


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------
def make_workload(args, world=1, workload=None):
    """The workload's case dict (mesh, fields, particles, parameters).  With
    several ranks the particle set holds world x the per-GPU count; each
    rank's Solver steps its share (Solver(shard=(rank, world)), the
    reference's parallel split)."""
    from cylag_gb300 import synth
    workload = workload or args.workload
    kw = {k: v for k, v in (("npart", args.npart), ("nx", args.nx), ("ny", args.ny)) if v} \
        if workload == args.workload else {}
    if world > 1:
        per = kw.get("npart") or {"lsm1_2d": 10_000_000, "lsm2_3d": 4_000_000,
                                  "lsm3_3d": 10_000_000}[workload]
        kw["npart"] = per * world
    if workload == "lsm1_2d":
        # field records A, B, A, ... every 600 s covering warm-up, timed and
        # end-to-end steps at dt = 0.5 s (0 / 600 / 1200 s up to 1197 timed
        # steps, the default case)
        horizon = max(1200.0, 0.5 * (args.warmup + 2 * args.steps))
        c = synth.keps_drift_channel(seed=0, horizon=horizon, **kw)
        c.update(dim=2, nlayers=1, pset={})
    elif workload == "lsm2_3d":
        c = synth.lsm2_loglaw_workload(seed=0, **kw)
    else:
        c = synth.lsm3_taylor_green_workload(seed=0, **kw)
    if c["parameters"].get("frozen_eulerian_fields"):
        # frozen fields: a horizon covering warm-up, timed and end-to-end steps
        dt = c["parameters"]["time_step"]
        c["parameters"]["final_time"] = dt * (args.warmup + 2 * max(args.steps, args.leg_steps)
                                              + 10)
    return c


def bytes_per_particle_step(workload, precision):
    """Algorithmic (compulsory) DRAM bytes per particle-step of the fused
    step, per particle: the state it must read and write.
    LSM1 2D: position r+w 32, tri r+w 8, PCG32 state r+w 16, tag r 4.
    LSM2 3D: position r+w 48, velocity r+w 48 (FP64) or 24 (the mixed form's
             FP32 working copies), tri r+w 8, layer r+w 8, PCG32 r+w 16,
             tag r 4, diameter r 8.
    LSM3 3D: the LSM2 set + fluid velocity seen r+w 48 (FP64) or 24."""
    if workload == "lsm1_2d":
        return 32 + 8 + 16 + 4
    v = 24 if precision == "mixed" else 48
    b = 48 + v + 8 + 8 + 16 + 4 + 8
    return b + v if workload == "lsm3_3d" else b


# DRAM bytes per particle-step of one step kernel launch, from ncu captures
# of the same kernel on smaller particle counts (element-sorted; the traffic
# grows with the particles processed)
NCU_TRAFFIC_B_PER_PARTICLE_STEP = {("lsm1_2d", "mixed"): 55.8, ("lsm1_2d", "fp64"): 147.0,
                                   ("lsm2_3d", "mixed"): 153.4, ("lsm3_3d", "mixed"): 185.3}
NCU_TRAFFIC_SOURCE = {
    ("lsm1_2d", "mixed"): "ncu dram bytes (read+write) of the element-sorted step kernel's "
                          "form for the run's configuration at 4e6 particles, scaled to the "
                          "launch",
    ("lsm1_2d", "fp64"): "ncu dram bytes (read+write) of the element-sorted step and walk "
                         "kernels at 4e6 particles, scaled to the launch",
    ("lsm2_3d", "mixed"): "ncu dram bytes (read+write) of the element-sorted step kernel's "
                          "form for the run's configuration at 2e6 particles, scaled to the "
                          "launch",
    ("lsm3_3d", "mixed"): "ncu dram bytes (read+write) of the element-sorted step kernel's "
                          "form for the run's configuration at 2e6 particles, scaled to the "
                          "launch"}


def field_set_of(c):
    import cylag_gb300 as cg
    from cylag_gb300.mesh import TriangularMesh
    mesh = TriangularMesh(c["x"], c["y"], c["triangles"])
    fs = cg.EulerianFieldSet(mesh, dim=c["dim"], nlayers=c["nlayers"], times=c["times"],
                             elevation=c["elevation"], velocity_x=c["velocity_x"],
                             velocity_y=c["velocity_y"], velocity_z=c.get("velocity_z"),
                             opt_fields=c.get("opt_fields"),
                             opt_fields_names=c.get("opt_fields_names"))
    return mesh, fs


def fields_dict(c):
    return dict(dim=c["dim"], nlayers=c["nlayers"], times=c["times"], elevation=c["elevation"],
                velocity_x=c["velocity_x"], velocity_y=c["velocity_y"],
                velocity_z=c.get("velocity_z"), opt_fields=c.get("opt_fields"),
                opt_fields_names=c.get("opt_fields_names"))


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# CPU implementation (oracle port, all host threads) on a bounded sample
# ---------------------------------------------------------------------------
def cpu_rate(c, params, nsample, nsteps, threads):
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    from cylag_gb300.mesh import TriangularMesh
    mesh = TriangularMesh(c["x"], c["y"], c["triangles"])
    diam = c["diameter"][:nsample] if "diameter" in c else None
    o = oracle.OracleSolver(mesh, fields_dict(c), params, c["position"][:nsample],
                            pset=c.get("pset"), nthreads=threads, diameter=diam)
    o.forward()  # warm
    t0 = time.perf_counter()
    for _ in range(nsteps):
        o.forward()
    dt = time.perf_counter() - t0
    return nsample * nsteps / dt, dt


def _reference_worker(job):
    """One host process of the reference's parallel decomposition
    (solver_parallel.pyx:113-179 without MPI): the unmodified compiled
    reference's Solver over a contiguous slice of the sample, set up
    untimed, W warm-up steps, then K timed forward() calls.  Returns the
    seconds of the timed steps."""
    import tempfile
    workload, argv, lo, hi, warmup, steps = job
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "oracle"))
    import refpath
    cy = refpath.use_reference()
    ns = parse_args(argv)
    c = make_workload(ns, workload=workload)
    params = dict(c["parameters"], listing=False,
                  output_rep=tempfile.mkdtemp(prefix="cylag_ref_"))
    mesh = cy.TriangularMesh(c["x"], c["y"], c["triangles"])
    f = fields_dict(c)
    fset = cy.EulerianFieldSet(mesh, dim=f["dim"], nlayers=f["nlayers"], times=f["times"],
                               elevation=f["elevation"], velocity_x=f["velocity_x"],
                               velocity_y=f["velocity_y"], velocity_z=f["velocity_z"],
                               opt_fields=f["opt_fields"],
                               opt_fields_names=f["opt_fields_names"])
    ps = cy.LagrangianParticleSet(np.ascontiguousarray(c["position"][lo:hi]), dim=c["dim"],
                                  **c.get("pset", {}))
    if "diameter" in c:
        np.asarray(ps.diameter)[:] = c["diameter"][lo:hi]
        np.asarray(ps.volume)[:] = np.pi * c["diameter"][lo:hi] ** 3 / 6.
    cy.random_utils.pcg32_seed(0, lo)
    s = cy.Solver(fset, ps, params)
    for _ in range(warmup):
        s.forward(s.simutime.time_step)
    t0 = time.perf_counter()
    for _ in range(steps):
        s.forward(s.simutime.time_step)
    return time.perf_counter() - t0


def reference_rate(args, nsample, steps, warmup, procs):
    """particle-steps/s of the compiled reference on `procs` host processes
    over the first `nsample` particles of the workload (the slowest process
    sets the time), or None when the reference is not built here."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import refpath
    if not refpath.available():
        return None
    import multiprocessing as mp
    from cylag_gb300.shard import split
    argv = [a for a in sys.argv[1:] if a not in ("--impl", "reference", "gb300")]
    jobs = [(args.workload, argv, a, a + n, warmup, steps) for a, n in split(nsample, procs)]
    with mp.get_context("spawn").Pool(procs) as pool:
        secs = pool.map(_reference_worker, jobs)
    return nsample * steps / max(secs), max(secs)


def run_reference_arm(args):
    rank, world, local = dist_info()
    if rank != 0:
        print(json.dumps({"impl": "reference", "rank": rank, "skipped": True}), file=sys.stderr)
        return
    threads = os.cpu_count() or 1
    if args.workload == "serve":
        from cylag_gb300 import synth
        c = synth.couette_channel(npart=10)
        value = serve_cpu_rate(c, threads)
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
            "n_gpus": args.gpus, "steps": 4, "warmup": 1, "ms_per_step": None,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": WORKLOADS["serve"]},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "100,000 LSM1 + 100,000 LSM2 particles x 4 steps"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return
    # the compiled reference (its own Solver, one process per host core),
    # else the C restatement on all host threads
    nall = len(make_workload(args)["position"])
    nref = min(nall, int(os.environ.get("CYLAG_REF_SAMPLE", str(25000 * threads))))
    procs = max(1, min(threads, nref))
    got = reference_rate(args, nref, args.steps, args.warmup, procs)
    if got is not None:
        value, secs = got
        kind, nsample, ms = "reference", nref, 1e3 * secs / args.steps
        sample = (f"{nref} particles of the workload in {procs} processes, each the compiled "
                  f"reference's Solver over a contiguous slice, one forward() per timed step")
    else:
        c = make_workload(args)
        params = dict(c["parameters"])
        nsample = int(os.environ.get("CYLAG_REF_SAMPLE", "200000"))
        # one solver over the sample (mesh and solver set up once, untimed); W
        # warm-up steps, then each timed step advances the sample by one step
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle
        from cylag_gb300.mesh import TriangularMesh
        mesh = TriangularMesh(c["x"], c["y"], c["triangles"])
        diam = c["diameter"][:nsample] if "diameter" in c else None
        o = oracle.OracleSolver(mesh, fields_dict(c), params, c["position"][:nsample],
                                pset=c.get("pset"), nthreads=threads, diameter=diam)
        for _ in range(args.warmup):
            o.forward()
        t_all = 0.
        for _ in range(args.steps):
            t0 = time.perf_counter()
            o.forward()
            t_all += time.perf_counter() - t0
        value = float(nsample * args.steps / t_all)
        kind, ms = "port", 1e3 * t_all / args.steps
        sample = f"{nsample} particles of the workload advanced one step per timed step"
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOADS[args.workload], "sample_particles": nsample,
                   "note": "each step advances a bounded sample of the particles on all host cores"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind,
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def measure(args, c, params, precision, rank, world, local, dist, do_e2e, steps=None,
            sort_period=None):
    """Warm-up, then K timed steps (CUDA events on the library's stream),
    then optionally K end-to-end steps through the C ABI with host buffers."""
    import torch
    import cylag_gb300 as cg
    from cylag_gb300 import _lib
    steps = args.steps if steps is None else steps
    sort_period = args.sort_period if sort_period is None else sort_period
    mesh, fs = field_set_of(c)
    ps = cg.LagrangianParticleSet(c["position"], dim=c["dim"], **c.get("pset", {}))
    if "diameter" in c:
        ps.diameter = c["diameter"]
    log(f"creating solver ({precision})")
    solver = cg.Solver(fs, ps, params, precision=precision, seed=0, device=local,
                       sort_period=sort_period, shard=(rank, world) if world > 1 else None)
    L = solver.L
    # all library work on a torch-owned stream (torch manages its lifetime)
    stream = torch.cuda.Stream(device=local)
    _lib.check(solver._ctx, L.cg_ctx_set_stream(solver._ctx, stream.cuda_stream))
    n = ps.npart
    log("warm-up")
    solver.forward(nsteps=args.warmup)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    if dist:
        dist.barrier()
    clocks.start()
    time.sleep(0.3)
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    log("timed region")
    ev0.record(stream)
    solver.forward(nsteps=steps)
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    kern_ms, launches = solver.last_kernel_ms()
    step_ms, walk_ms = solver.last_kernel_split_ms()
    if dist:
        from cylag_gb300.shard import allreduce_max
        ms = allreduce_max(ms, dist)
    log(f"{precision}: timed {ms:.3f} ms, kernel {kern_ms:.4f} ms/launch")
    res = {"precision": precision, "ms": ms, "kernel_ms": kern_ms, "launches": launches,
           "step_ms": step_ms, "walk_ms": walk_ms,
           "value": world * n * steps / (ms / 1e3), "clocks": clk, "n": n,
           "position": ps.position, "velocity": ps.velocity, "inactive": ps.inactive,
           "nt": int(mesh.nt), "steps": steps}
    if do_e2e:
        # end to end: the particle state lives in pinned host memory; every
        # step, one C-ABI call copies it in, steps and copies it back
        # (cg_run_step_host: chunked, copies overlapping the step)
        log("end-to-end region")
        ps._sync()
        d = ps._dev
        keys = ["position", "tri", "tag", "rng_state"]
        if c["dim"] == 3:
            keys.append("lowerlayer")
        if params["model"] >= 2:
            keys.append("velocity")
        if params["model"] == 3:
            keys.append("fluid_velocity_seen")
        host = {k: torch.empty_like(d[k], device="cpu").pin_memory() for k in keys}
        for k in keys:
            host[k].copy_(d[k])
        h2d = d2h = sum(host[k].numel() * host[k].element_size() for k in keys)
        ptr = lambda k: host[k].data_ptr() if k in host else None
        arr = _lib.HostArrays(ptr("position"), ptr("velocity"), ptr("fluid_velocity_seen"),
                              ptr("tri"), ptr("lowerlayer"), ptr("tag"), ptr("rng_state"))
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        e0.record(stream)
        # one call of K steps: every step copies its whole state in from the
        # pinned host arrays and its results back out, chunk by chunk, and the
        # copy pipeline runs on from one step to the next
        rc = L.cg_run_step_host(solver._run, steps, C.byref(arr), C.byref(arr), args.e2e_chunk,
                                None)
        _lib.check(solver._ctx, rc)
        e1.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        del host
        ems = e0.elapsed_time(e1)
        if dist:
            from cylag_gb300.shard import allreduce_max
            ems = allreduce_max(ems, dist)
        res["e2e"] = {"value": world * n * steps / (ems / 1e3), "unit": UNIT,
                      "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                      "wall_s": wall}
    torch.cuda.synchronize()
    solver.close()
    del ps, solver
    torch.cuda.empty_cache()
    return res


def oracle_subsample_error(c, params, res, nsteps, every, threads):
    """The mixed form's error against the FP64 oracle: the oracle advances
    every `every`-th particle (tags = their indices, so their PCG32 streams
    are the GPU's) by the same steps; ensemble mean and variance of the
    displacement (and of the velocity for LSM2/LSM3) compared on that
    subsample."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    from cylag_gb300.mesh import TriangularMesh
    from cylag_gb300.stats import displacement_report
    n = len(c["position"])
    idx = np.arange(0, n, every)
    mesh = TriangularMesh(c["x"], c["y"], c["triangles"])
    diam = c["diameter"][idx] if "diameter" in c else None
    o = oracle.OracleSolver(mesh, fields_dict(c), params, c["position"][idx], pset=c.get("pset"),
                            seed=0, tags=idx, nthreads=threads, diameter=diam)
    o.solve(nsteps)
    act = (res["inactive"][idx] == 0) & (o.inactive == 0)
    rep = displacement_report(c["position"][idx], res["position"][idx], o.pos, act)
    out = {"steps": nsteps, "particles": int(act.sum()),
           "rms_displacement_diff_m": rep["rms_displacement_diff"],
           "var_rel_err": max(rep["var_rel_err"]), "mean_rel_err": max(rep["mean_rel_err"])}
    if params["model"] >= 2:
        va, vb = res["velocity"][idx][act], o.vel[act]
        out["velocity_var_rel_err"] = float(
            np.max(np.abs(va.var(0) - vb.var(0)) / np.maximum(vb.var(0), 1e-300)))
    return out


MODEL_DESC = {"lsm1_2d": "LSM1 Euler, k-eps drift",
              "lsm2_3d": "LSM2 direct integrator, k-eps velocity diffusion",
              "lsm3_3d": "LSM3 direct integrator, constant K, polydisperse settling"}


def workload_line(args, workload, c, params, res, main_form, peak, peak_kind, world):
    """The bench line's fields of one workload: throughput, roofline of its
    step kernels, the plain form beside the mixed one."""
    r = res[main_form]
    n = r["n"]
    bpp = bytes_per_particle_step(workload, main_form)
    # the dominant kernel: the step kernel (it moves the particle state); the
    # walk kernel that finishes the queued particles is timed beside it
    kms = r["step_ms"] if r.get("step_ms") else r["kernel_ms"]
    achieved = bpp * n / (kms / 1e3) / 1e9
    traffic = NCU_TRAFFIC_B_PER_PARTICLE_STEP.get((workload, main_form))
    line = {
        "value": r["value"], "ms_per_step": r["ms"] / r["steps"], "steps": r["steps"],
        "config": {"workload": WORKLOADS[workload], "particles_per_gpu": n,
                   "triangles": r["nt"], "layers": c["nlayers"], "precision": main_form,
                   "dt": params["time_step"], "l2": "state larger than L2 (no flush)",
                   "model": MODEL_DESC[workload], "sort_period": args.sort_period},
        "gpu_launches": int(r["launches"]),   # every kernel of the timed cg_run_step call
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak,
                     "traffic": float(traffic * n) if traffic else None,
                     "traffic_source": NCU_TRAFFIC_SOURCE.get((workload, main_form)),
                     "peak_kind": peak_kind, "kernel": "step kernel", "kernel_ms": kms,
                     "walk_kernel_ms": r.get("walk_ms"),
                     "step_and_walk_ms": r["kernel_ms"],
                     "frac_step_and_walk": bpp * n / (r["kernel_ms"] / 1e3) / 1e9 / peak,
                     "bytes_per_particle_step": bpp},
        "clocks": r["clocks"],
    }
    if "fp64" in res and main_form != "fp64":
        q = res["fp64"]
        line["plain_fp64"] = {"value": q["value"], "kernel_ms": q["kernel_ms"],
                              "ms_per_step": q["ms"] / q["steps"], "clocks": q["clocks"]}
        line["mixed_over_plain"] = r["value"] / q["value"]
    return line


def run_gpu_arm(args):
    import torch
    rank, world, local = dist_info()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    torch.cuda.set_device(local)
    log("building workload")
    c = make_workload(args, world)
    params = dict(c["parameters"])
    total_steps = args.warmup + args.steps + (0 if args.no_e2e else args.steps)
    if not params.get("frozen_eulerian_fields") and \
            total_steps * params["time_step"] > float(c["times"][-1]):
        raise SystemExit("warmup + 2*steps must stay within the field records")
    forms = [args.precision] if args.precision != "both" else ["mixed", "fp64"]
    res = {}
    for prec in forms:
        res[prec] = measure(args, c, params, prec, rank, world, local, dist,
                            do_e2e=(not args.no_e2e and prec == forms[0]))
    threads = os.cpu_count() or 1
    peak, peak_kind = peaks()
    main_form = forms[0]
    line = None
    if rank == 0:
        wl = workload_line(args, args.workload, c, params, res, main_form, peak, peak_kind,
                           world)
        line = {"metric": METRIC, "value": wl["value"], "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": wl["ms_per_step"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64" if main_form == "fp64" else "f32+f64", "data": "synthetic"}
        line.update({k: v for k, v in wl.items() if k not in ("value", "ms_per_step", "steps")})
        if "e2e" in res[main_form]:
            line["e2e"] = res[main_form]["e2e"]
        if main_form == "mixed" and not args.no_oracle_error and world == 1:
            log("mixed form vs the FP64 oracle")
            line["mixed_error_vs_oracle"] = oracle_subsample_error(
                c, params, res["mixed"], args.warmup + args.steps,
                max(1, len(c["position"]) // 50_000), threads)
        if not args.no_cpu_baseline:
            log("cpu baseline")
            nsample = int(os.environ.get("CYLAG_CPU_SAMPLE", "200000"))
            rate, dt = cpu_rate(c, params, nsample, 4, threads)
            port = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                    "sample": f"{nsample} particles x 4 steps of the workload"}
            nref = min(len(c["position"]), 25000 * threads)
            got = reference_rate(args, nref, 8, 2, threads) if world == 1 else None
            if got is not None:
                line["cpu_baseline"] = {
                    "value": got[0], "unit": UNIT, "cores": threads, "kind": "reference",
                    "sample": f"{nref} particles x 8 steps of the workload in {threads} "
                              "processes, each the compiled reference's Solver over a slice"}
                line["cpu_port"] = port
            else:
                line["cpu_baseline"] = port
    del res
    # the other configurations of the metric, as legs of the same line: the
    # 3D LSM2 and LSM3 workloads at their full sizes, and the serving mix on
    # a shortened arrival window (p50/p99 latency); each in its own process,
    # so that host memory is released between workloads
    if args.legs and args.workload == "lsm1_2d" and world == 1 and rank == 0:
        legs = {}
        for wl_name, extra in (("lsm2_3d", ["--steps", str(args.leg_steps), "--no-e2e"]),
                               ("lsm3_3d", ["--steps", str(args.leg_steps), "--no-e2e"]),
                               ("serve", ["--serve-duration", str(args.leg_serve_duration),
                                          "--precision", "mixed"])):
            log(f"leg {wl_name}")
            cmd = [sys.executable, str(ROOT / "bench.py"), "--workload", wl_name,
                   "--warmup", str(args.warmup), "--legs", "0", "--no-cpu-baseline",
                   "--sort-period", str(args.sort_period)] + extra
            r = subprocess.run(cmd, stdout=subprocess.PIPE, text=True)
            out = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
            if r.returncode != 0 or not out:
                legs[wl_name] = {"error": f"exit {r.returncode}"}
                continue
            d = json.loads(out[-1])
            legs[wl_name] = {k: v for k, v in d.items()
                             if k not in ("metric", "unit", "n_gpus", "higher_is_better",
                                          "scaling", "vs_baseline", "data", "warmup")}
        line["legs"] = legs
    if rank == 0:
        print(json.dumps(line), flush=True)
    log("done")


# ---------------------------------------------------------------------------
# serving mix: requests arriving in real time, continuous batching
# ---------------------------------------------------------------------------
def serve_cpu_rate(fs_case, threads, nsample=100_000, nsteps=4):
    """The CPU implementation on half LSM1, half LSM2 particles of the mix's
    parameters on the same channel."""
    from cylag_gb300.serve import LSM1_PARAMS, LSM2_PARAMS
    rates = []
    for prm in (LSM1_PARAMS, LSM2_PARAMS):
        c = dict(fs_case, dim=2, nlayers=1, pset={})
        rng = np.random.default_rng(9)
        c["position"] = np.stack([rng.uniform(0, 1000.0, nsample), rng.uniform(0, 100.0, nsample)], 1)
        r, _ = cpu_rate(c, dict(prm, final_time=1e6), nsample, nsteps, threads)
        rates.append(r)
    return 2.0 / (1.0 / rates[0] + 1.0 / rates[1])


def serve_once(fs, reqs, prec, local, chunk):
    """Plays the requests in real time through one serving pool; per-request
    latency (arrival -> result on the host), throughput over the wall time."""
    import torch
    from cylag_gb300.serve import DispersionServer, poisson_mix
    work = sum(len(r.position) * r.horizon for r in reqs)
    npart = sum(len(r.position) for r in reqs)
    # pool: every particle of the mix fits (120 GB admission budget)
    srv = DispersionServer(fs, precision=prec, capacity=max(npart, 1 << 20) + 32 * len(reqs),
                           max_runs=len(reqs) + 8, device=local, hbm_budget=120 * 10**9)
    warm = poisson_mix(rate=100.0, duration=0.05, seed=99, nmax=1e4, hmax=200)
    srv.serve(warm, realtime=False)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    log(f"{prec}: serving")
    t0 = time.perf_counter()
    res = srv.serve(reqs, realtime=True, chunk=chunk)
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    st = srv.stats()
    srv.close()
    lat = np.array([r.latency for r in res])
    queue = np.array([r.admitted - r.arrival for r in res])
    out = {"value": work / wall, "wall_s": wall, "p50_s": float(np.percentile(lat, 50)),
           "p99_s": float(np.percentile(lat, 99)), "max_s": float(lat.max()),
           "admission_wait_p99_s": float(np.percentile(queue, 99)),
           "steps": int(st["steps_issued"]), "clocks": clk, "completed": len(res)}
    log(f"{prec}: {wall:.1f} s, p50 {out['p50_s']:.2f} s, p99 {out['p99_s']:.2f} s")
    return out


def run_serve(args):
    import torch
    from cylag_gb300 import synth
    from cylag_gb300.serve import poisson_mix
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    c = synth.couette_channel(npart=10)
    c.update(dim=2, nlayers=1)
    mesh, fs = field_set_of(c)
    reqs = poisson_mix(rate=args.serve_rate, duration=args.serve_duration, seed=5 + rank)
    work = sum(len(r.position) * r.horizon for r in reqs)
    npart = sum(len(r.position) for r in reqs)
    log(f"serving mix: {len(reqs)} requests, {npart:.3e} particles, {work:.3e} particle-steps")
    forms = [args.precision] if args.precision != "both" else ["mixed", "fp64"]
    out = {prec: serve_once(fs, reqs, prec, local, args.serve_chunk) for prec in forms}
    if rank != 0:
        return
    m = out[forms[0]]
    peak, peak_kind = peaks()
    # LSM1: position, tri, PCG32 r+w, tag r (60 B); LSM2 adds velocity r+w
    # and diameter r (100 B); half of the requests each
    bpp = 80.0
    achieved = bpp * work / m["wall_s"] / 1e9
    line = {
        "metric": METRIC, "value": m["value"], "unit": UNIT, "n_gpus": world,
        "steps": m["steps"], "warmup": 1, "ms_per_step": 1e3 * m["wall_s"] / max(m["steps"], 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if forms[0] == "fp64" else "f32+f64", "data": "synthetic",
        "config": {"workload": WORKLOADS["serve"], "requests": len(reqs), "particles": npart,
                   "particle_steps": work, "precision": forms[0], "arrival_rate_per_s": args.serve_rate,
                   "arrival_window_s": args.serve_duration, "chunk_steps": args.serve_chunk,
                   "hbm_budget_bytes": 120 * 10**9,
                   "l2": "per-step state of the mix larger than L2 at load (no flush)"},
        "latency_s": {"p50": m["p50_s"], "p99": m["p99_s"], "max": m["max_s"],
                      "admission_wait_p99": m["admission_wait_p99_s"]},
        "gpu_launches": m["steps"] + 3 * len(reqs),   # graph steps + prepare/seed/init per request
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None, "peak_kind": peak_kind,
                     "note": "serving-window average (wall clock incl. idle between arrivals)",
                     "bytes_per_particle_step": bpp},
        "clocks": m["clocks"],
        "e2e": {"value": m["value"], "unit": UNIT,
                "h2d_bytes_per_step": int(16 * npart / max(m["steps"], 1)),
                "d2h_bytes_per_step": int(48 * npart / max(m["steps"], 1)),
                "note": "requests enter as host arrays and results return to host arrays"},
    }
    if "fp64" in out and forms[0] != "fp64":
        q = out["fp64"]
        line["plain_fp64"] = {"value": q["value"], "latency_s": {"p50": q["p50_s"], "p99": q["p99_s"],
                                                                 "max": q["max_s"]},
                              "wall_s": q["wall_s"], "clocks": q["clocks"]}
        line["mixed_over_plain"] = m["value"] / q["value"]
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        line["cpu_baseline"] = {"value": serve_cpu_rate(c, threads), "unit": UNIT, "cores": threads,
                                "kind": "port",
                                "sample": "100,000 LSM1 + 100,000 LSM2 particles x 4 steps on the channel"}
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference_arm(args)
    elif args.workload == "serve":
        run_serve(args)
    else:
        run_gpu_arm(args)


if __name__ == "__main__":
    main()
