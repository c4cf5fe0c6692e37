"""ctypes driver for the C restatement of CyLag's particle step (the oracle).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of bench.py, never by the product package.

``OracleSolver`` replays ``Solver.__init__`` + ``Solver.forward``
(cylag/core/solver.pyx:74-236, 413-585) on the host: time interpolation of the
node fields at the step-start time (eulerian_field_set.pyx:866-938), then
the per-particle step of ``oracle/cylag_oracle.c`` over every particle, then
``time += dt`` (simutime.pyx:77-84).  Particle state is kept in the
reference's own layout (``double[npart, dim]`` rows).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libcylag_oracle.so"
_lock = threading.Lock()
_lib = None

EPSILON = 1.0e-16


def build(force: bool = False) -> Path:
    """Compile the oracle with gcc (no FMA contraction, OpenMP)."""
    src = [HERE / "cylag_oracle.c"]
    hdr = HERE / "cylag_oracle.h"
    BUILD.mkdir(exist_ok=True)
    newest = max(p.stat().st_mtime for p in src + [hdr])
    if not force and LIB.exists() and LIB.stat().st_mtime >= newest:
        return LIB
    tmp = LIB.with_suffix(f".so.{os.getpid()}")
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-fopenmp",
           "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wno-unused-function",
           *map(str, src), "-o", str(tmp), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


class Mesh(C.Structure):
    _fields_ = [("nv", C.c_int), ("nt", C.c_int), ("ne", C.c_int),
                ("x", C.c_void_p), ("y", C.c_void_p), ("tri", C.c_void_p),
                ("gradx", C.c_void_p), ("grady", C.c_void_p), ("det", C.c_void_p),
                ("edges", C.c_void_p), ("triedge", C.c_void_p),
                ("edgetri", C.c_void_p), ("edge_labels", C.c_void_p),
                ("gx0", C.c_double), ("gy0", C.c_double), ("ginv", C.c_double),
                ("gnx", C.c_int), ("gny", C.c_int), ("gstart", C.c_void_p), ("gtris", C.c_void_p)]


class Fields(C.Structure):
    _fields_ = [("dim", C.c_int), ("nlayers", C.c_int), ("npoints", C.c_int),
                ("frozen", C.c_int), ("prev_valid", C.c_int),
                ("zs", C.c_void_p), ("ux", C.c_void_p), ("uy", C.c_void_p),
                ("uz", C.c_void_p), ("kt", C.c_void_p), ("ep", C.c_void_p),
                ("zb", C.c_void_p), ("z0", C.c_void_p), ("u0", C.c_void_p),
                ("v0", C.c_void_p), ("w0", C.c_void_p)]


class Params(C.Structure):
    _fields_ = [("model", C.c_int), ("time_scheme", C.c_int), ("rng_method", C.c_int),
                ("diffusion_model", C.c_int), ("diffusion_lsm2_option", C.c_int),
                ("lsm3_edge_opt", C.c_int), ("boundary_conditions", C.c_int),
                ("bc_type", C.c_int), ("max_wall_rebounds", C.c_int),
                ("bnd_statistics", C.c_int), ("particle_velocity_init", C.c_int),
                ("dt", C.c_double), ("time", C.c_double),
                ("nux", C.c_double), ("nuz", C.c_double), ("sigc", C.c_double),
                ("tl_h", C.c_double), ("tl_v", C.c_double),
                ("damp_coef", C.c_double), ("roughness_deg", C.c_double),
                ("strand_prob", C.c_double),
                ("pdim", C.c_int), ("rho0", C.c_double), ("density", C.c_double),
                ("drag_model", C.c_int), ("drag_coef", C.c_double),
                ("added_mass", C.c_int), ("added_mass_coef", C.c_double),
                ("buoy_model", C.c_int), ("buoy_value", C.c_double),
                ("a0c", C.c_double), ("a1c", C.c_double), ("a2c", C.c_double),
                ("a3c", C.c_double), ("friction_model", C.c_int),
                ("friction_coef", C.c_double), ("compute_depth", C.c_int)]


class Particles(C.Structure):
    _fields_ = [("n", C.c_int),
                ("pos", C.c_void_p), ("vel", C.c_void_p), ("fvs", C.c_void_p),
                ("last_pos", C.c_void_p), ("last_vel", C.c_void_p),
                ("tri", C.c_void_p), ("last_tri", C.c_void_p),
                ("lowerlayer", C.c_void_p), ("inactive", C.c_void_p),
                ("tag", C.c_void_p), ("diameter", C.c_void_p), ("volume", C.c_void_p),
                ("rng_state", C.c_void_p), ("rng_inc", C.c_void_p),
                ("depth", C.c_void_p)]


def lib():
    global _lib
    with _lock:
        if _lib is None:
            L = C.CDLL(str(build()))
            P = C.c_void_p
            L.cgo_pcg32_seed.argtypes = [P, P, C.c_uint64, C.c_uint64]
            L.cgo_pcg32_advance.argtypes = [P, C.c_uint64, C.c_uint64]
            L.cgo_rng_draws.argtypes = [C.c_uint64, C.c_uint64, C.c_int, C.c_int, C.c_int64, P]
            L.cgo_ziggurat_tables.argtypes = [P, P, P]
            L.cgo_time_interp.argtypes = [C.c_int64, C.c_double, P, P, P]
            L.cgo_step.argtypes = [P, P, P, P, P, C.c_int]
            L.cgo_step.restype = C.c_int
            L.cgo_init_range.argtypes = [P, P, P, P, C.c_int, C.c_int]
            L.cgo_init_range.restype = C.c_int
            L.cgo_take_errors.argtypes = []
            L.cgo_take_errors.restype = C.c_int
            L.cgo_set_stranding.argtypes = [C.c_int]
            L.cgo_take_stranded.argtypes = [P, C.c_int]
            L.cgo_take_stranded.restype = C.c_int
            L.cgo_set_sections.argtypes = [C.c_int, P]
            L.cgo_set_sections.restype = C.c_int
            L.cgo_take_section_counts.argtypes = [P]
            L.cgo_retag.argtypes = [P, C.c_int]
            L.cgo_retag.restype = C.c_int
            L.cgo_xy_localize.argtypes = [P, C.c_int, C.c_double, C.c_double,
                                          C.c_double, C.c_double, P, P]
            L.cgo_locate_exhaustive.argtypes = [P, C.c_double, C.c_double]
            L.cgo_locate_exhaustive.restype = C.c_int
            L.cgo_locate.argtypes = [P, C.c_double, C.c_double]
            L.cgo_locate.restype = C.c_int
            L.cgo_lower_layer_index.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double]
            L.cgo_lower_layer_index.restype = C.c_int
            _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def pcg32_seed(seed: int, stream: int):
    st = np.zeros(1, np.uint64)
    inc = np.zeros(1, np.uint64)
    lib().cgo_pcg32_seed(_p(st), _p(inc), seed, stream)
    return int(st[0]), int(inc[0])


def seed_streams(seed: int, tags):
    """Per-particle PCG32 (state, inc) for pcg32_seed(seed, tag)."""
    tags = np.asarray(tags, dtype=np.uint64)
    inc = (tags << np.uint64(1)) | np.uint64(1)
    mult = np.uint64(6364136223846793005)
    with np.errstate(over="ignore"):
        st = np.zeros_like(tags) * mult + inc          # next() from state 0
        st = st + np.uint64(seed)
        st = st * mult + inc                            # next()
    return st, inc


def rng_draws(seed: int, stream: int, kind: int, n: int, method: int = 2):
    out = np.zeros(2 * n if kind == 3 else n)
    lib().cgo_rng_draws(seed, stream, kind, method, n, _p(out))
    return out


def ziggurat_tables():
    kn = np.zeros(128, np.uint32)
    wn = np.zeros(128)
    fn = np.zeros(128)
    lib().cgo_ziggurat_tables(_p(kn), _p(wn), _p(fn))
    return kn, wn, fn


class OracleSolver:
    """Host replay of Solver over the C oracle.

    ``mesh``: object with the TriangularMesh arrays; ``fields``: dict with
    dim, nlayers, times, elevation, velocity_x/y/z, opt_fields,
    opt_fields_names; ``pset``: dict of LagrangianParticleSet options.
    """

    def __init__(self, mesh, fields, params, position, pset=None, seed=0,
                 tags=None, nthreads=1, diameter=None, sources=None, initial_pool_size=None,
                 min_pool_size_update=1000, field_set=None, control_sections=None,
                 max_stranded=None, friction_model=1, friction_coefficient=40.):
        from cylag_gb300.parameters import Parameters
        L = lib()
        self.L = L
        self.nthreads = nthreads
        pset = dict(pset or {})
        self.params = Parameters(params)
        self.params.check_values()
        P = self.params
        self.mesh = mesh
        g = mesh.locator_grid()
        self._grid = g
        self._m = Mesh(mesh.nv, mesh.nt, mesh.ne, _p(mesh.x), _p(mesh.y),
                       _p(mesh.triangles), _p(mesh.gradx), _p(mesh.grady), _p(mesh.det),
                       _p(mesh.edges), _p(mesh.triedge_map), _p(mesh.edgetri_map),
                       _p(mesh.edges_labels), g[0], g[1], g[2], g[3], g[4], _p(g[5]), _p(g[6]))
        self._keep = []
        # ---- fields ---------------------------------------------------------
        fdim = fields.get("dim", 2)
        nl = fields.get("nlayers", 1)
        npts = mesh.nv
        self.times = np.asarray(fields["times"], dtype=np.float64)
        self.ntimes = len(self.times)
        names = list(fields.get("opt_fields_names") or [])
        opt = fields.get("opt_fields")
        src = {"zs": fields["elevation"], "ux": fields["velocity_x"],
               "uy": fields["velocity_y"]}
        if fdim == 3:
            src["uz"] = fields["velocity_z"]
        for nm, key in (("TURBULENT ENERG.", "kt"), ("DISSIPATION", "ep"), ("BOTTOM", "zb")):
            if nm in names:
                src[key] = opt[names.index(nm)]
        self.src = {k: np.ascontiguousarray(v, dtype=np.float64) for k, v in src.items()}
        size = npts * nl
        self.tmp = {k: v[0].copy() for k, v in self.src.items()}
        self.prev = {k: self.tmp[k].copy() for k in ("zs", "ux", "uy", "uz") if k in self.tmp}
        self.fdim, self.nl, self.npts, self.size = fdim, nl, npts, size
        self.frozen = bool(P.frozen_eulerian_fields) or self.ntimes == 1
        if self.ntimes == 1 and not P.frozen_eulerian_fields:
            raise ValueError("EulerianFieldSet has only one time step, use frozen_eulerian_fields=True")
        if not P.frozen_eulerian_fields and P.final_time > self.times[-1]:
            raise ValueError("final_time > EulerianFieldSet maximum time")
        self.record = 0
        self.interp_done = False
        self.prev_valid = False
        if not self.frozen:
            self.record = self._lower_index(P.initial_time, 0)
        # ---- particles ------------------------------------------------------
        # lagrangian_particle_set.pyx:158-261: a pool of initial_pool_size
        # entries (default: the positions given), the first ones active
        pos0 = np.ascontiguousarray(position, dtype=np.float64)
        na, pd = pos0.shape
        n = na if initial_pool_size is None else int(initial_pool_size)
        if n < na:
            raise ValueError("size of position > initial_pool_size")
        self.n, self.pd = n, pd
        self.seed = seed
        self.sources = list(sources or [])
        # what the sources see as the field set (record kept in step here)
        self.field_set = field_set
        self.min_pool_size_update = int(min_pool_size_update)
        self.pos = np.zeros((n, pd))
        self.pos[:na] = pos0
        self.vel = np.zeros((n, pd))
        self.fvs = np.zeros((n, pd))
        self.last_pos = self.pos.copy()
        self.last_vel = np.zeros((n, pd))
        self.tri = -np.ones(n, np.int32)
        self.last_tri = -np.ones(n, np.int32)
        self.lowerlayer = np.zeros(n, np.int32)
        self.inactive = np.ones(n, np.int32)
        self.inactive[:na] = 0
        self.tag = (np.arange(n, dtype=np.int32) if tags is None
                    else np.asarray(tags, dtype=np.int32).copy())
        self.maxtag = int(self.tag.max()) if n else -1
        dp = pset.get("particle_diameter", 0.01)
        self.dp = dp
        self.diameter = (np.full(n, dp) if diameter is None
                         else np.asarray(diameter, dtype=np.float64).copy())
        self.volume = np.pi * (self.diameter ** 3) / 6.
        # lagrangian_particle_set.pyx:212-219
        self.compute_depth = bool(pset.get("compute_depth", False))
        self.depth = np.zeros(n) if self.compute_depth else None
        self.rng_state, self.rng_inc = seed_streams(seed, self.tag)
        self._bind()
        # ---- params ----------------------------------------------------------
        rho0 = P.water_density
        rhop = pset.get("particle_density", 1000.)
        am = int(bool(pset.get("added_mass_force", False)))
        Ca = pset.get("added_mass_coef", 0.5)
        if am == 0:
            a0c, a1c, a2c, a3c = (rhop - rho0) / rhop, 0.5 * (rho0 / rhop), 0., 1. / rhop
        else:
            aux = 1. / (rhop + Ca * rho0)
            a0c, a1c, a2c, a3c = (rhop - rho0) * aux, 0.5 * rho0 * aux, rho0 * (1. + Ca) * aux, aux
        self._p = Params(
            P.model, P.time_scheme, P.rng_method, P.diffusion_model,
            P.diffusion_lsm2_option, P.lsm3_edge_opt, int(bool(P.boundary_conditions)),
            P.boundary_conditions_type, P.max_wall_rebounds, int(bool(P.bnd_statistics)),
            P.particle_velocity_init, P.time_step, P.initial_time,
            P.horizontal_diffusivity, P.vertical_diffusivity, P.schmidt_number,
            P.diffusion_lsm3_tl_horizontal, P.diffusion_lsm3_tl_vertical,
            P.rebound_damping_coef, P.wall_roughness_angle, P.stranding_probability,
            pd, rho0, rhop, pset.get("drag_coefficient_model", 1),
            pset.get("drag_coefficient", 0.44), am, Ca,
            pset.get("buoyancy_velocity_model", 0), pset.get("buoyancy_velocity", 0.0),
            a0c, a1c, a2c, a3c, int(friction_model), float(friction_coefficient),
            int(self.compute_depth))
        self.time = P.initial_time
        self.dt = P.time_step
        self.time_step = P.time_step
        self.nopen = int(getattr(mesh, "nopen", 0))
        self.bnd_stats = []
        if not self.frozen:
            self._time_interpolation(P.initial_time)
        # control sections: first segment of each (control_shapes.pyx:17-19)
        self.sections = []
        for cs in control_sections or []:
            poly = np.asarray(cs.poly if hasattr(cs, "poly") else cs, dtype=np.float64)
            self.sections.append([poly[0, 0], poly[0, 1], poly[1, 0], poly[1, 1]])
        self.section_stats = []
        # stranding output buffer (lagrangian_particle_set.pyx:225-228)
        self.stranding = bool(P.stranding_output)
        self.max_stranded = n if max_stranded is None else int(max_stranded)
        self.stranded = []
        self.L.cgo_take_errors()
        self.L.cgo_init_range(C.byref(self._m), C.byref(self._fields()), C.byref(self._p),
                              C.byref(self._s), 0, n)
        self._raise_errors("initialization")
        self.maxtag = self.L.cgo_retag(C.byref(self._s), self.maxtag)
        self.iteration = 0
        self.final_time = P.final_time

    def _bind(self, n=None):
        """The C view of the particle arrays (its first n entries)."""
        self._s = Particles(self.n if n is None else n, _p(self.pos), _p(self.vel),
                            _p(self.fvs), _p(self.last_pos), _p(self.last_vel), _p(self.tri),
                            _p(self.last_tri), _p(self.lowerlayer), _p(self.inactive),
                            _p(self.tag), _p(self.diameter), _p(self.volume),
                            _p(self.rng_state), _p(self.rng_inc),
                            _p(self.depth) if self.depth is not None else None)

    # ---- particles added during the run (lagrangian_particle_set.pyx) ------------
    def _increase_pool_size(self, size):
        """lagrangian_particle_set.pyx:522-582"""
        add = max(self.min_pool_size_update, int(size))
        z = lambda *sh, dt=np.float64: np.zeros(sh, dtype=dt)
        cat = lambda a, b: np.ascontiguousarray(np.concatenate([a, b], axis=0))
        self.inactive = cat(self.inactive, np.ones(add, np.int32))
        self.diameter = cat(self.diameter, z(add))
        self.volume = cat(self.volume, z(add))
        for k in ("pos", "vel", "fvs", "last_pos", "last_vel"):
            setattr(self, k, cat(getattr(self, k), z(add, self.pd)))
        self.tag = cat(self.tag, np.arange(self.maxtag + 1, self.maxtag + 1 + add, dtype=np.int32))
        self.maxtag += add
        self.tri = cat(self.tri, -np.ones(add, np.int32))
        self.lowerlayer = cat(self.lowerlayer, z(add, dt=np.int32))
        self.last_tri = cat(self.last_tri, z(add, dt=np.int32))
        self.rng_state = cat(self.rng_state, z(add, dt=self.rng_state.dtype))
        self.rng_inc = cat(self.rng_inc, z(add, dt=self.rng_inc.dtype))
        if self.depth is not None:
            self.depth = cat(self.depth, z(add))
        self.n += add
        self._bind()

    def add(self, position):
        """lagrangian_particle_set.pyx:620-710 (method 1), plus the stream of
        each added particle: pcg32_seed(seed, tag)."""
        pos = np.asarray(position, dtype=np.float64)
        nadd = pos.shape[0] if pos.ndim == 2 else 0
        if nadd == 0:
            return
        free = np.flatnonzero(self.inactive == 1)
        if nadd > len(free):
            self._increase_pool_size(nadd - len(free))
            free = np.flatnonzero(self.inactive == 1)
        idx = free[:nadd]
        self.inactive[idx] = 0
        self.diameter[idx] = self.dp
        self.volume[idx] = np.pi * (self.dp ** 3) / 6.
        self.pos[idx] = pos
        self.tri[idx] = -2
        st, inc = seed_streams(self.seed, self.tag[idx])
        self.rng_state[idx] = st
        self.rng_inc[idx] = inc

    def _raise_errors(self, where):
        e = self.L.cgo_take_errors()
        if e:
            raise ValueError(f"{e} particle(s) failed during {where} (point outside the "
                             "mesh or the water column, or non-finite LSM2/LSM3 coefficients)")

    # simutime/zlocalizer helpers ------------------------------------------------
    def _lower_index(self, value, last):
        t = self.times
        for i in range(last, len(t) - 1):
            if value >= t[i] and value < t[i + 1]:
                return i
        if len(t) > 1 and value >= t[-1]:
            return len(t) - 2
        return 0

    def _time_interpolation(self, time):
        """eulerian_field_set.pyx:866-938"""
        if self.frozen:
            return
        for k in self.prev:
            self.prev[k][:] = self.tmp[k]
        self.prev_valid = self.interp_done
        self.interp_done = True
        self.record = self._lower_index(time, self.record)
        rec = self.record
        dt = self.times[rec] - self.times[rec + 1]
        if abs(dt) < EPSILON:
            raise ValueError("Time interpolation failed: duplicate times")
        tf = (time - self.times[rec + 1]) / dt
        for k, v in self.src.items():
            self.L.cgo_time_interp(self.size, tf, _p(v[rec]), _p(v[rec + 1]), _p(self.tmp[k]))

    def _fields(self):
        t, pv = self.tmp, self.prev
        f = Fields(self.fdim, self.nl, self.npts, int(self.frozen), int(self.prev_valid),
                   _p(t.get("zs")), _p(t.get("ux")), _p(t.get("uy")), _p(t.get("uz")),
                   _p(t.get("kt")), _p(t.get("ep")), _p(t.get("zb")),
                   _p(pv.get("zs")), _p(pv.get("ux")), _p(pv.get("uy")), _p(pv.get("uz")))
        self._keep = [f]
        return f

    def forward(self):
        """solver.pyx:413-585 (no control sections).  The sources are asked
        at the step's start (``self`` serves as the SimuTime: time,
        time_step, iteration, final_time); the step covers the pool size it
        started with (solver.pyx:430), so entries of a pool grown by this
        step's releases wait for the next step.  ``field_set`` (given at
        construction) is handed to the sources with this run's record."""
        self._time_interpolation(self.time)
        npart = self.n
        fs = self.field_set
        if fs is not None:
            fs.record = self.record
        for src in self.sources:
            if src.release_condition(self, fs):
                self.add(src.init_positions(fs, self.pd))
        self._bind(npart)
        self._p.time = self.time
        stats = np.zeros(max(1, self.nopen), np.int32)
        seg = np.ascontiguousarray(np.array(self.sections, dtype=np.float64).reshape(-1, 4))
        self.L.cgo_set_sections(len(self.sections), _p(seg))
        self.L.cgo_set_stranding(int(self.stranding))
        self.L.cgo_step(C.byref(self._m), C.byref(self._fields()), C.byref(self._p),
                        C.byref(self._s), _p(stats), self.nthreads)
        if self.sections:
            cnt = np.zeros(len(self.sections), np.int32)
            self.L.cgo_take_section_counts(_p(cnt))
            self.section_stats.append(cnt)
        if self.stranding:
            buf = np.zeros((npart, 4))
            k = self.L.cgo_take_stranded(_p(buf), npart)
            rec = buf[:k][np.argsort(buf[:k, 0], kind="stable")]
            for r in rec:   # compute_bc.pyx:109-121: kept while the buffer has room
                if len(self.stranded) < self.max_stranded:
                    self.stranded.append(r[1:].copy())
        self.L.cgo_set_sections(0, None)
        self.L.cgo_set_stranding(0)
        self._raise_errors(f"the step at t={self.time}")
        self.maxtag = self.L.cgo_retag(C.byref(self._s), self.maxtag)
        self._bind()
        self.bnd_stats.append(stats[: self.nopen].copy())
        self.time += self.dt
        self.iteration += 1

    def solve(self, nsteps):
        for _ in range(nsteps):
            self.forward()

    @property
    def npart_active(self):
        return int((self.inactive == 0).sum())
