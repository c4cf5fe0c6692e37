"""Host mirror of cylag.core: EulerianFieldSet, LagrangianParticleSet, Solver.

Same constructor signatures and public attributes as the reference
(cylag/core/eulerian_field_set.pyx:125-256,
cylag/core/lagrangian_particle_set.pyx:158-261, cylag/core/solver.pyx:74-236),
so that scripts written for cylag run unchanged.  The particle loop of
``Solver.forward`` (solver.pyx:459-549) runs as one fused CUDA launch per
step through libcylag_gpu.so; particle state lives in HBM in torch tensors
(plumbing only) in the reference's layout (``double[npart, dim]`` rows), and
reading a public array (``pset.position`` ...) copies it to the host.

Per-particle random streams: particle with tag t draws from
pcg32_seed(seed, t) (cylag/lsm/random_utils.pyx:30-37), so that results do
not depend on particle order or batch composition.
"""
from __future__ import annotations

import ctypes as C
import time as _time

import numpy as np

from . import _lib
from .mesh import TriangularMesh
from .parameters import Parameters

EPSILON = 1.0e-16
NU0 = 1.3e-6        # constants.pyx: kinematic viscosity of water, m2/s
GRAV = 9.80665      # constants.pyx: gravity, m/s2


def _cpow_re(x, y):
    """x**y for x > 0 as the compiled reference evaluates a double power:
    the real part of the C library's complex power, exp(y log x) with the
    complex logarithm's real part log1p((x-1)(x+1))/2 for 0.5 <= x < 2."""
    import math
    L = math.log1p((x - 1.) * (x + 1.)) / 2. if 0.5 <= x < 2. else math.log(x)
    return math.exp(y * L)
DEFAULT_INITIAL_POOL_SIZE = 10000
_OPT_NAMES = {
    "turbulent_energy": ("TURBULENT ENERG.", "TURBULENT ENERGY", "ENERGIE TURBUL."),
    "dissipation": ("DISSIPATION",),
    "bottom": ("BOTTOM", "FOND"),
}


def lower_index(times, value, last=0):
    """zlocalizer.pyx:125-151: i with times[i] <= value < times[i+1],
    searched from ``last``; the last interval at or past the end; 0 before
    the start."""
    n = len(times)
    for i in range(int(last), n - 1):
        if times[i] <= value < times[i + 1]:
            return i
    if n > 1 and value >= times[-1]:
        return n - 2
    return 0


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("cylag_gb300 needs a CUDA device (no CPU fallback)")
    return torch


class SimuTime:
    """cylag/core/simutime.pyx:25-125 (time bookkeeping on the host)."""

    def __init__(self, print_progress, initial_time=0., final_time=0., time_step=0.):
        if final_time <= initial_time:
            raise ValueError("final_time must be greater than initial_time")
        if time_step <= 0.:
            raise ValueError("time_step must be greater than 0")
        if final_time - initial_time < time_step:
            raise ValueError("final_time - initial_time must be greater than time_step")
        self.time = initial_time
        self.initial_time = initial_time
        self.time_step = time_step
        self.final_time = final_time
        self.nt = int((final_time - initial_time) / time_step)
        self._times = None
        self.iteration = 0
        self.is_finished = False
        self.print_progress = print_progress

    @property
    def times(self):
        """The nt + 1 step times, np.linspace(initial_time, final_time,
        nt + 1), built on first access (a long horizon makes it large)."""
        if self._times is None:
            self._times = np.linspace(self.initial_time, self.final_time, self.nt + 1)
        return self._times

    def increment(self):
        self.time += self.time_step
        self.iteration += 1
        if self.time >= self.final_time:
            self.is_finished = True


class _SimuTimeView:
    """A copy of a SimuTime's clock that can be moved forward on its own."""

    def __init__(self, st):
        self.time, self.time_step = st.time, st.time_step
        self.iteration, self.final_time = st.iteration, st.final_time
        self.initial_time, self.nt = st.initial_time, st.nt

    def advance(self):
        self.time += self.time_step
        self.iteration += 1


class EulerianFieldSet:
    """Mirror of cylag.EulerianFieldSet (eulerian_field_set.pyx:125-256)."""

    def __init__(self, triangular_mesh, dim=2, nlayers=1, times=None, elevation=None,
                 velocity_x=None, velocity_y=None, velocity_z=None, opt_fields=None,
                 opt_fields_names=None, trifinder=None, friction_model=1,
                 friction_coefficient=40.):
        if not isinstance(triangular_mesh, TriangularMesh):
            triangular_mesh = TriangularMesh(
                np.asarray(triangular_mesh.x), np.asarray(triangular_mesh.y),
                np.asarray(triangular_mesh.triangles), nopen=getattr(triangular_mesh, "nopen", 0))
        self.triangular_mesh = triangular_mesh
        self.npoints = triangular_mesh.nv
        self.nlayers = int(nlayers)
        self.dim = int(dim)
        self.trifinder = trifinder
        self.times = np.ascontiguousarray(times, dtype=np.float64)
        self.ntimes = len(self.times)
        self.record = 0
        self.frozen_hydro = self.ntimes == 1
        for i in range(self.ntimes - 1):
            dt = self.times[i + 1] - self.times[i]
            if dt <= EPSILON:
                raise ValueError(
                    f"Invalid times array: times must be strictly increasing. Found "
                    f"times[{i}]={self.times[i]:.6e} and times[{i+1}]={self.times[i+1]:.6e}")
        ref = (self.ntimes, self.npoints) if self.dim == 2 else (self.ntimes, self.npoints * self.nlayers)
        for name, f in (("elevation", elevation), ("velocity_x", velocity_x),
                        ("velocity_y", velocity_y)) + ((("velocity_z", velocity_z),) if self.dim == 3 else ()):
            if np.shape(f) != ref:
                raise ValueError(f"Field have wrong dimension, expected {ref}, found {np.shape(f)}")
        self.elevation = np.ascontiguousarray(elevation, dtype=np.float64)
        self.velocity_x = np.ascontiguousarray(velocity_x, dtype=np.float64)
        self.velocity_y = np.ascontiguousarray(velocity_y, dtype=np.float64)
        self.velocity_z = None if velocity_z is None else np.ascontiguousarray(velocity_z, dtype=np.float64)
        if self.dim == 3:
            self.check_regular_layers()
        self.nopt = 0 if opt_fields is None else len(opt_fields_names)
        self.opt_fields = None if opt_fields is None else np.ascontiguousarray(opt_fields, dtype=np.float64)
        self.opt_fields_names = opt_fields_names
        self.field_names = ["ELEVATION", "VELOCITY U", "VELOCITY V", "VELOCITY W"]
        self.fid_zs, self.fid_ux, self.fid_uy, self.fid_uz = 0, 1, 2, 3
        self.fid_turbeng = self.fid_dissip = self.fid_zb = -1
        self._opt = {}
        if opt_fields_names is not None:
            names = list(opt_fields_names)
            for key, alts in _OPT_NAMES.items():
                for nm in alts:
                    if nm in names:
                        j = names.index(nm)
                        self._opt[key] = np.ascontiguousarray(self.opt_fields[j])
                        if key == "turbulent_energy":
                            self.fid_turbeng = 4 + j
                        elif key == "dissipation":
                            self.fid_dissip = 4 + j
                        else:
                            self.fid_zb = 4 + j
                        break
        self.friction_model = friction_model
        self.friction_coefficient = friction_coefficient

    @staticmethod
    def from_telemac2d(file_name, main_var_names=("FREE SURFACE", "VELOCITY U", "VELOCITY V"),
                       bnd_file=None, optional_fields=None, init_trifinder=True,
                       friction_model=1, friction_coefficient=40.):
        """eulerian_field_set.pyx:316-398 from a TELEMAC-2D result file
        (cylag_gb300.telemac reads the Selafin format); times start at 0 at
        the first record.  ``init_trifinder`` is accepted and unused: the
        grid locator replaces matplotlib's trifinder."""
        from .telemac import SelafinFile, read_cli
        res = SelafinFile(file_name)
        bnd_pts, nopen = read_cli(bnd_file) if bnd_file is not None else (None, 0)
        mesh = TriangularMesh(res.x, res.y, res.ikle2, boundary_points=bnd_pts, nopen=nopen)
        nt, n = res.ntimestep, res.npoin2
        get = lambda name: np.stack([res.get_data_value(name, k)[:n] for k in range(nt)])
        opt = None
        if optional_fields is not None:
            opt = np.stack([get(nm) for nm in optional_fields])
        return EulerianFieldSet(mesh, 2, 1, res.times - res.times[0], get(main_var_names[0]),
                                get(main_var_names[1]), get(main_var_names[2]), None, opt,
                                None if optional_fields is None else list(optional_fields),
                                None, friction_model=friction_model,
                                friction_coefficient=friction_coefficient)

    @staticmethod
    def from_telemac3d(file_name,
                       main_var_names=("ELEVATION Z", "VELOCITY U", "VELOCITY V", "VELOCITY W"),
                       bnd_file=None, optional_fields=None, init_trifinder=True,
                       friction_model=1, friction_coefficient=40.):
        """eulerian_field_set.pyx:400-484 from a TELEMAC-3D result file:
        nplan layers of npoin2 nodes (the file's node order)."""
        from .telemac import SelafinFile, read_cli
        res = SelafinFile(file_name)
        bnd_pts, nopen = read_cli(bnd_file) if bnd_file is not None else (None, 0)
        mesh = TriangularMesh(res.x, res.y, res.ikle2, boundary_points=bnd_pts, nopen=nopen)
        nt = res.ntimestep
        get = lambda name: np.stack([res.get_data_value(name, k) for k in range(nt)])
        opt = None
        if optional_fields is not None:
            opt = np.stack([get(nm) for nm in optional_fields])
        return EulerianFieldSet(mesh, 3, res.nplan, res.times - res.times[0],
                                get(main_var_names[0]), get(main_var_names[1]),
                                get(main_var_names[2]), get(main_var_names[3]), opt,
                                None if optional_fields is None else list(optional_fields),
                                None, friction_model=friction_model,
                                friction_coefficient=friction_coefficient)

    @staticmethod
    def from_hdf5(fset_file="cylag_fset_file.h5", mesh_file="cylag_mesh_file.h5",
                  optional_fields=None, init_trifinder=True, friction_model=1,
                  friction_coefficient=40.):
        """eulerian_field_set.pyx:486-566 from a CyLag field-set file and mesh
        file (written by the reference's ``save_hdf5`` or by this one; read by
        ``cylag_gb300.hdf5``).  The optional fields are named from the file
        unless ``optional_fields`` names them.  ``init_trifinder`` is accepted
        and unused: the grid locator replaces matplotlib's trifinder."""
        from . import hdf5
        mesh = TriangularMesh.from_hdf5(file_name=mesh_file)
        f = hdf5.read(fset_file)
        first = lambda k: int(np.asarray(f[k]).reshape(-1)[0])
        dim, nplan, nopt = first("dim"), first("nplan"), first("nopt")
        opt = None
        if nopt != 0:
            if optional_fields is None:
                if "opt_fields_names" in f:
                    optional_fields = [n.decode("utf-8") if isinstance(n, bytes) else str(n)
                                       for n in f["opt_fields_names"]]
                else:
                    optional_fields = [f"opt_field_{i}" for i in range(nopt)]
            opt = f["opt_fields"]
        else:
            optional_fields = None
        if dim == 2:
            return EulerianFieldSet(mesh, 2, 1, f["times"], f["elevation"], f["velocity_x"],
                                    f["velocity_y"], None, opt, optional_fields, None,
                                    friction_model=friction_model,
                                    friction_coefficient=friction_coefficient)
        if dim == 3:
            return EulerianFieldSet(mesh, 3, nplan, f["times"], f["elevation"], f["velocity_x"],
                                    f["velocity_y"], f["velocity_z"], opt, optional_fields, None,
                                    friction_model=friction_model,
                                    friction_coefficient=friction_coefficient)
        raise ValueError(f"{fset_file}: dim {dim} is neither 2 nor 3")

    def save_hdf5(self, fset_file="cylag_fset_file.h5", mesh_file="cylag_mesh_file.h5"):
        """eulerian_field_set.pyx:568-604: the mesh file, then the field-set
        file with the same datasets (the optional fields' names as
        variable-length UTF-8 strings)."""
        from . import hdf5
        self.triangular_mesh.save_mesh_hdf5(mesh_file)
        d = {"dim": np.array([self.dim], dtype=np.int64),
             "nplan": np.array([self.nlayers], dtype=np.int64),
             "times": np.asarray(self.times), "elevation": np.asarray(self.elevation),
             "velocity_x": np.asarray(self.velocity_x), "velocity_y": np.asarray(self.velocity_y),
             "nopt": np.array([self.nopt], dtype=np.int64)}
        if self.dim == 3:
            d["velocity_z"] = np.asarray(self.velocity_z)
        if self.nopt != 0:
            d["opt_fields"] = np.asarray(self.opt_fields)
            d["opt_fields_names"] = [str(n) for n in self.opt_fields_names]
        hdf5.write(fset_file, d)

    def _get_field_from_id(self, field_id):
        """eulerian_field_set.pyx:673-720: 0 elevation, 1-3 velocity, 4+ the
        optional fields in the given order ([ntimes, npoints*nlayers])."""
        if field_id == 0:
            return self.elevation
        if field_id == 1:
            return self.velocity_x
        if field_id == 2:
            return self.velocity_y
        if field_id == 3 and self.velocity_z is not None:
            return self.velocity_z
        if 4 <= field_id < 4 + self.nopt:
            return self.opt_fields[field_id - 4]
        raise ValueError(f"Invalid field id {field_id}")

    def _get_field_slice(self, field, k, l):
        """eulerian_field_set.pyx:623-648: record k, layer l (-1: all)."""
        if self.dim == 2:
            return field[k, 0:self.npoints]
        if l != -1:
            return field[k, l * self.npoints:(l + 1) * self.npoints]
        return field[k, :]

    def _set_record(self, time, follow=True):
        """eulerian_field_set.pyx:845-864: the record whose [t_r, t_r+1)
        holds ``time`` (searched from the current one when following); 0
        when the fields are frozen.  The device run keeps its own copy; this
        one is what the sources see."""
        if not self.frozen_hydro:
            self.record = lower_index(self.times, time, self.record if follow else 0)
        else:
            self.record = 0

    def check_dim(self, field):
        """eulerian_field_set.pyx:258-279: ValueError unless the field has
        the set's record shape."""
        ref = (self.ntimes, self.npoints) if self.dim == 2 else \
            (self.ntimes, self.npoints * self.nlayers)
        if np.shape(field) != ref:
            raise ValueError(f"Field have wrong dimension, expected {ref}, found {np.shape(field)}")

    # ---- pre- and post-processing (eulerian_field_set.pyx:606-1886) ---------
    def get_field_list(self):
        """Field names and ids: the main fields, then the optional ones."""
        names = self.field_names + list(self.opt_fields_names or [])
        return names, list(range(len(names)))

    def _field_at(self, field_id, time):
        """A field's node values at `time` (eulerian_field_set.pyx:940-993):
        linear in time between the records holding it, record 0 when the
        fields are frozen.  The record is searched from the first one and
        the set's own record is left as it is."""
        if self.dim == 2 and field_id == 3:
            raise ValueError("Wrong field id")
        f = self._get_field_from_id(field_id)
        if f is None:
            raise ValueError(f"no field with id {field_id}")
        if self.frozen_hydro:
            return np.asarray(f[0], dtype=np.float64)
        rec = lower_index(self.times, time, 0)
        dt = self.times[rec] - self.times[rec + 1]
        if abs(dt) < EPSILON:
            raise ValueError(f"Time interpolation failed: duplicate times at record {rec}")
        tf = (time - self.times[rec + 1]) / dt
        return tf * f[rec] + (1. - tf) * f[rec + 1]

    def get_field(self, field_id, time, layer=-1):
        """eulerian_field_set.pyx:1770-1795: a field at `time`, one layer
        (3D, layer >= 0) or all."""
        v = self._field_at(field_id, time)
        if self.dim == 2:
            return v[:self.npoints]
        if layer != -1:
            return v[layer * self.npoints:(layer + 1) * self.npoints]
        return v

    def _locate(self, point, k):
        if k is None:
            k = (self.trifinder(point[0], point[1]) if self.trifinder is not None
                 else self.triangular_mesh.find_triangle(float(point[0]), float(point[1])))
        return int(k)

    def _interp(self, values, k, point):
        """P1 interpolation on triangle k (eulerian_field_set.pyx:994-1055);
        in 3D between the P1 values on the layers below and above the point,
        linear in z between their elevations (1184-1287)."""
        m = self.triangular_mesh
        x, y = float(point[0]), float(point[1])
        i0, i1, i2 = (int(i) for i in m.triangles[k])
        f = [m.det[k, j] + x * m.gradx[k, j] + y * m.grady[k, j] for j in range(3)]

        def p1(v, off=0):
            return v[off + i0] * f[0] + v[off + i1] * f[1] + v[off + i2] * f[2]

        if self.dim == 2:
            return p1(values)
        return self._interp_z(values, p1, float(point[2]))

    def _interp_z(self, values, p1, z):
        nl, npt = self.nlayers, self.npoints
        elev = self._elev_now
        zb, zs = p1(elev, 0), p1(elev, (nl - 1) * npt)
        # zlocalizer.pyx:51-71
        ll = 0
        if nl > 1:
            hl = (zs - zb) / (nl - 1)
            if hl > 0.:
                fi = (z - zb) // hl
                ll = 0 if not fi >= 0. else (nl - 2 if not fi <= nl - 2 else int(fi))
        jl, ju = ll * npt, (ll + 1) * npt
        zl, zu = p1(elev, jl), p1(elev, ju)
        dz = zl - zu
        if abs(dz) < EPSILON:
            raise ValueError(f"3D interpolation failed: degenerate vertical layer {ll}")
        return ((z - zu) / dz) * p1(values, jl) + ((zl - z) / dz) * p1(values, ju)

    def interpolate_field(self, field_id, point, time, k=None):
        """eulerian_field_set.pyx:1842-1886: a field at a point and time;
        k, the triangle holding the point, is located when not given."""
        values = self._field_at(field_id, time)
        k = self._locate(point, k)
        if k == -1:
            raise ValueError("Failed interpolation (5), point not in triangulation")
        if self.dim == 3:
            self._elev_now = self._field_at(self.fid_zs, time)
        return self._interp(values, k, point)

    def interpolate_velocity(self, point, time, k=None):
        """eulerian_field_set.pyx:1797-1840: (u, v) in 2D, (u, v, w) in 3D."""
        k = self._locate(point, k)
        if k == -1:
            raise ValueError("Failed interpolation (4), point not in triangulation")
        ids = (self.fid_ux, self.fid_uy) + ((self.fid_uz,) if self.dim == 3 else ())
        if self.dim == 3:
            self._elev_now = self._field_at(self.fid_zs, time)
        return tuple(self._interp(self._field_at(i, time), k, point) for i in ids)

    def check_regular_layers(self, rtol=1e-3):
        """eulerian_field_set.pyx:258-294 (uniform sigma layers)."""
        nl = self.nlayers
        if self.dim != 3 or nl < 2:
            return
        frac = (np.arange(nl) / (nl - 1.))[:, None]
        z = np.asarray(self.elevation)[0].reshape(nl, self.npoints)
        zb = z[0]
        hl = (z[-1] - zb) / (nl - 1.)
        expected = zb[None, :] + frac * (z[-1] - zb)[None, :]
        tol = rtol * np.abs(hl) + 1e-6 * (1. + np.abs(zb))
        err = np.abs(z - expected) - tol[None, :]
        if np.any(err > 0.):
            raise ValueError("Vertical layers are not regularly spaced (CyLag requires uniform sigma layers)")


class LagrangianParticleSet:
    """Mirror of cylag.LagrangianParticleSet (lagrangian_particle_set.pyx:158-261).

    Before a Solver attaches, arrays live on the host; afterwards the device
    copy is authoritative and attribute reads return fresh host copies.
    """

    _STATE = ("position", "velocity", "fluid_velocity_seen", "last_position", "last_velocity",
              "tri", "last_tri", "lowerlayer", "tag", "diameter")

    def __init__(self, position=None, velocity=None, fluid_velocity_seen=None, dim=2,
                 initial_pool_size=None, min_pool_size_update=1000, particle_density=1000.,
                 particle_diameter=0.01, particle_diameter_distribution=None,
                 drag_coefficient_model=1, drag_coefficient=0.44, added_mass_force=False,
                 added_mass_coef=0.5, buoyancy_velocity_model=0, buoyancy_velocity=0.0,
                 compute_depth=False, max_stranded=None):
        if position is not None and initial_pool_size is None:
            npart = np.shape(position)[0]
        else:
            npart = initial_pool_size if initial_pool_size is not None else DEFAULT_INITIAL_POOL_SIZE
        self.npart = int(npart)
        self.dim = int(dim)
        self.min_pool_size_update = min_pool_size_update
        self.rho0 = 1000.
        self.density = particle_density
        self.particle_diameter = particle_diameter
        self.particle_volume = np.pi * (particle_diameter ** 3) / 6.
        if particle_diameter_distribution is not None:
            raise NotImplementedError(
                "particle_diameter_distribution: draw diameters on the host and set "
                "pset.diameter before creating the Solver")
        self.diameter_distribution = "monodisperse"
        self.drag_coef_model = drag_coefficient_model
        self.drag_coef = drag_coefficient
        self.added_mass_force = added_mass_force
        self.added_mass_coef = added_mass_coef
        self.buoyancy_velocity_model = buoyancy_velocity_model
        self.buoyancy_velocity_value = buoyancy_velocity
        self.additional_velocity = False
        self.additional_force = False
        self.compute_depth = bool(compute_depth)
        if compute_depth and dim != 3:
            raise ValueError("compute_depth can only be True for 3D pset")
        self.max_stranded = max_stranded if max_stranded is not None else self.npart
        self.stranded_count = 0
        self.stranded_positions = np.zeros((self.max_stranded, 3))
        n, d = self.npart, self.dim
        h = {}
        h["position"] = np.zeros((n, d))
        h["velocity"] = np.zeros((n, d))
        h["fluid_velocity_seen"] = np.zeros((n, d))
        inactive = np.ones(n, dtype=np.int32)
        if position is not None:
            pos = np.asarray(position, dtype=np.float64)
            if pos.shape[0] > n:
                raise ValueError("size of position > initial_pool_size")
            if pos.shape[1] != d:
                raise ValueError("dim of position != LagrangianParticleSet.dim")
            h["position"][: pos.shape[0]] = pos
            inactive[: pos.shape[0]] = 0
            if velocity is not None:
                vel = np.asarray(velocity, dtype=np.float64)
                if vel.shape != pos.shape:
                    raise ValueError("size of velocity != size of position")
                h["velocity"][: pos.shape[0]] = vel
            if fluid_velocity_seen is not None:
                if velocity is None:
                    raise ValueError("velocity must be != None")
                fvs = np.asarray(fluid_velocity_seen, dtype=np.float64)
                if fvs.shape != pos.shape:
                    raise ValueError("size of fluid_velocity_seen != size of velocity")
                h["fluid_velocity_seen"][: pos.shape[0]] = fvs
        elif velocity is not None or fluid_velocity_seen is not None:
            raise ValueError("position must be != None")
        h["last_position"] = h["position"].copy()
        h["last_velocity"] = h["velocity"].copy()
        # -2: active, awaiting Solver.initialize_particle_state; -1: inactive
        h["tri"] = np.where(inactive == 0, -2, -1).astype(np.int32)
        h["last_tri"] = -np.ones(n, dtype=np.int32)
        h["lowerlayer"] = np.zeros(n, dtype=np.int32)
        h["tag"] = np.arange(n, dtype=np.int32)
        h["diameter"] = np.full(n, float(particle_diameter))
        if self.compute_depth:
            # depth below the free surface (lagrangian_particle_set.pyx:212-219),
            # set by the solver at initialization and after every step
            h["depth"] = np.zeros(n)
        self.maxtag = n - 1
        # new tags are maxtag + tag_stride, + 2 tag_stride, ...: 1 as in the
        # reference; the rank count for a shard of a split set, so that the
        # ranks' new tags (and so their PCG32 streams) never coincide
        self.tag_stride = 1
        self._added = False     # entries set to tri = -2 since the run's last step
        self._host = h
        self._dev = None
        self._ctx = None

    # ---- one rank's share of a set split across ranks -------------------------
    def parallel_split(self, rank, world):
        """Keeps this rank's share of the set, as the reference's parallel
        solver splits it (solver_parallel.pyx:126-149 for the counts,
        lagrangian_particle_set.pyx:449-520 for the arrays): the active
        particles [offset, offset + count) with offset = rank * (na // world)
        and the remainder to the last rank, in a pool of max(1, n // world)
        entries (the remainder of the pool to the last rank), padded with
        inactive entries.  Kept particles keep their tags, so their PCG32
        streams are those of the unsplit run.  Unlike the reference, whose
        ranks share one generator, the streams here follow the tags, so new
        tags must not coincide across ranks: rank r draws them from
        maxtag + r + 1, maxtag + r + 1 + world, ... (tag_stride = world),
        starting with its padding entries.  Call before the Solver attaches."""
        if self._dev is not None:
            raise RuntimeError("parallel_split must come before the Solver attaches")
        rank, world = int(rank), int(world)
        if not 0 <= rank < world:
            raise ValueError(f"rank {rank} outside [0, {world})")
        n = self.npart
        active = np.flatnonzero(self._host["tri"] != -1)
        na = len(active)
        npart0 = [max(1, n // world)] * world
        npart0[-1] += n % world
        npartp = [na // world] * world
        npartp[-1] += na % world
        offset, count = rank * npartp[0], npartp[rank]
        new_n = max(npart0[rank], count)
        pad = new_n - count
        keep = active[offset:offset + count]
        h = self._host
        out = {}
        for k, v in h.items():
            fill = {"tri": -1, "last_tri": -1}.get(k, 0)
            a = np.full((new_n,) + v.shape[1:], fill, dtype=v.dtype)
            a[:count] = v[keep]
            out[k] = a
        out["tri"][:count] = -2             # awaiting initialization
        out["last_tri"][:] = -1
        out["lowerlayer"][:] = 0
        out["last_position"][:count] = out["position"][:count]
        out["last_velocity"][:count] = out["velocity"][:count]
        base = self.maxtag
        self.tag_stride = world
        self.maxtag = base + rank + 1 - world
        out["tag"][count:] = (self.maxtag + world * np.arange(1, pad + 1, dtype=np.int64)
                              ).astype(np.int32)
        self.maxtag += pad * world
        self._host = out
        self.npart = new_n
        self.max_stranded = max(self.max_stranded, new_n)
        self.stranded_positions = np.zeros((self.max_stranded, 3))
        return self

    # ---- device attachment -----------------------------------------------------
    def _attach(self, ctx, device):
        torch = _torch()
        dev = torch.device("cuda", device)
        self._dev = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in self._host.items()}
        self._dev["rng_state"] = torch.zeros(self.npart, dtype=torch.int64, device=dev)
        # the library works on its own (non-blocking) stream: make the copies land first
        torch.cuda.synchronize(dev)
        self._host = None
        self._ctx = ctx

    def _state_desc(self):
        d = self._dev
        p = lambda k: d[k].data_ptr()
        return _lib.StateDesc(self.npart, p("position"), p("velocity"), p("fluid_velocity_seen"),
                              p("last_position"), p("last_velocity"), p("tri"), p("last_tri"),
                              p("lowerlayer"), p("tag"), p("diameter"), p("rng_state"),
                              p("depth") if "depth" in d else None)

    def _sync(self):
        """Makes the device arrays the whole particle state and waits for
        the library's queued work: an element-sorted run keeps its newest
        state in working copies between steps (cg_run_writeback)."""
        if self._ctx is not None:
            L = _lib.load()
            solver = getattr(self, "_solver", None)
            run = getattr(solver, "_run", None) if solver is not None else None
            if run:
                _lib.check(self._ctx, L.cg_run_writeback(run))
            _lib.check(self._ctx, L.cg_ctx_sync(self._ctx))

    def _get(self, key):
        if self._dev is None:
            return self._host[key]
        self._sync()
        return self._dev[key].cpu().numpy()

    def _set(self, key, value):
        value = np.ascontiguousarray(value, dtype=np.float64 if key in
                                     ("position", "velocity", "fluid_velocity_seen",
                                      "last_position", "last_velocity", "diameter",
                                      "depth") else np.int32)
        if self._dev is None:
            self._host[key][...] = value
        else:
            self._sync()
            self._dev[key].copy_(_torch().from_numpy(value))
            _torch().cuda.synchronize()

    def _retag(self):
        """Gives the deleted particles their new tags (see retag)."""
        if self._dev is None:
            return
        self._sync()
        tag = self._dev["tag"]
        neg = (tag < 0).nonzero().flatten()
        if neg.numel() == 0:
            return
        new, self.maxtag = retag(tag.cpu().numpy(), self.maxtag, self.tag_stride)
        torch = _torch()
        tag.copy_(torch.from_numpy(new).to(tag.device))
        torch.cuda.synchronize()

    # ---- public arrays --------------------------------------------------------
    position = property(lambda s: s._get("position"), lambda s, v: s._set("position", v))
    velocity = property(lambda s: s._get("velocity"), lambda s, v: s._set("velocity", v))
    fluid_velocity_seen = property(lambda s: s._get("fluid_velocity_seen"),
                                   lambda s, v: s._set("fluid_velocity_seen", v))
    last_position = property(lambda s: s._get("last_position"))
    last_velocity = property(lambda s: s._get("last_velocity"))
    tri = property(lambda s: s._get("tri"))
    last_tri = property(lambda s: s._get("last_tri"))
    lowerlayer = property(lambda s: s._get("lowerlayer"))
    diameter = property(lambda s: s._get("diameter"), lambda s, v: s._set("diameter", v))

    @property
    def depth(self):
        """Depth below the free surface of each particle (compute_depth sets
        only; None otherwise, as the reference)."""
        return self._get("depth") if self.compute_depth else None

    @property
    def volume(self):
        d = self.diameter
        return np.pi * (d ** 3) / 6.

    @property
    def tag(self):
        self._retag()
        return self._get("tag")

    @property
    def inactive(self):
        return (self._get("tri") == -1).astype(np.int32)

    @property
    def npart_active(self):
        return int((self._get("tri") != -1).sum())

    def get_state(self):
        """lagrangian_particle_set.pyx:398-423: sorts active particles first,
        returns their position, velocity, fluid velocity seen."""
        self._sort_active_particles()
        na = self.npart_active
        return self.position[:na], self.velocity[:na], self.fluid_velocity_seen[:na]

    def get_particle_properties(self):
        self._sort_active_particles()
        na = self.npart_active
        d = self.diameter[:na]
        return d, np.pi * (d ** 3) / 6.

    def _sort_active_particles(self):
        """lagrangian_particle_set.pyx:584-618 (same np.argsort permutation)."""
        self._retag()
        idx = np.argsort(self.inactive)
        if np.array_equal(idx, np.arange(self.npart)):
            return
        if self._dev is None:
            for k in self._host:
                self._host[k] = self._host[k][idx]
            return
        torch = _torch()
        self._sync()
        ti = torch.from_numpy(idx).to(self._dev["tri"].device)
        for k in self._dev:  # in place: the run keeps pointing at these buffers
            self._dev[k].copy_(self._dev[k].index_select(0, ti))
        torch.cuda.synchronize()

    def _append_stranded(self, xyz):
        """compute_bc.pyx:109-121: appends stranded positions while the
        buffer (max_stranded) has room."""
        for row in np.asarray(xyz).reshape(-1, 3):
            if self.stranded_count < self.max_stranded:
                self.stranded_positions[self.stranded_count] = row
                self.stranded_count += 1
            else:
                print("Warning: stranded particle buffer is full"
                      "                       Increase max_stranded in LagrangianParticleSet")

    # ---- particles added during the run ---------------------------------------
    _PAD = {"position": 0., "velocity": 0., "fluid_velocity_seen": 0., "last_position": 0.,
            "last_velocity": 0., "tri": -1, "last_tri": 0, "lowerlayer": 0, "diameter": 0.,
            "depth": 0.}

    def _increase_pool_size(self, size):
        """lagrangian_particle_set.pyx:522-582: grows every array by
        max(min_pool_size_update, size) inactive entries (tri -1, last_tri 0,
        zero state) tagged maxtag+1, maxtag+2, ...; an attached run is
        pointed at the new arrays."""
        add = max(int(self.min_pool_size_update), int(size))
        newtags = (self.maxtag + self.tag_stride *
                   np.arange(1, add + 1, dtype=np.int64)).astype(np.int32)
        if self._dev is None:
            for k, v in self._host.items():
                if k == "tag":
                    pad = newtags
                else:
                    pad = np.full((add,) + v.shape[1:], self._PAD[k], dtype=v.dtype)
                self._host[k] = np.concatenate([v, pad], axis=0)
        else:
            torch = _torch()
            self._sync()   # nothing of the run may still touch the old arrays
            for k, v in list(self._dev.items()):
                if k == "tag":
                    pad = torch.from_numpy(newtags).to(v.device)
                elif k == "rng_state":
                    pad = torch.zeros(add, dtype=v.dtype, device=v.device)
                else:
                    pad = torch.full((add,) + tuple(v.shape[1:]), self._PAD[k], dtype=v.dtype,
                                     device=v.device)
                self._dev[k] = torch.cat([v, pad], dim=0)
            torch.cuda.synchronize(v.device)
        self.maxtag += add * self.tag_stride
        self.npart += add
        solver = getattr(self, "_solver", None)
        if solver is not None and self._dev is not None:
            solver._pool_resized()

    def add(self, position):
        """lagrangian_particle_set.pyx:620-710 (its method 1): the nadd new
        particles take the inactive entries in index order, after the pool
        grew by the shortfall; each gets the set's diameter, its position and
        tri = -2 (initialized by the next step of an attached run, with the
        PCG32 stream pcg32_seed(seed, tag)).  Velocities are left as they
        are (zero for a deleted or new entry)."""
        pos = np.ascontiguousarray(position, dtype=np.float64)
        nadd = pos.shape[0] if pos.ndim == 2 else 0
        if nadd == 0:
            return
        if pos.shape[1] != self.dim:
            raise ValueError("dim of position != LagrangianParticleSet.dim")
        self._retag()   # deleted entries carry their final tags before reuse
        free = np.flatnonzero(self._get("tri") == -1)
        if nadd > len(free):
            self._increase_pool_size(nadd - len(free))
            free = np.flatnonzero(self._get("tri") == -1)
        idx = free[:nadd]
        if self._dev is None:
            self._host["position"][idx] = pos
            self._host["diameter"][idx] = self.particle_diameter
            self._host["tri"][idx] = -2
        else:
            torch = _torch()
            dev = self._dev["tri"].device
            ti = torch.from_numpy(idx).to(dev)
            self._dev["position"].index_copy_(0, ti, torch.from_numpy(pos).to(dev))
            self._dev["diameter"].index_fill_(0, ti, float(self.particle_diameter))
            self._dev["tri"].index_fill_(0, ti, -2)
            torch.cuda.synchronize(dev)
            self._added = True

    def show_status(self, i):
        """lagrangian_particle_set.pyx:377-396: prints particle i's state."""
        print("~~~~~~~~~~~~~~~~~~~~~")
        print("Particle n°", i)
        for k in ("position", "velocity", "fluid_velocity_seen"):
            print(f"{k:<20}=", np.asarray(self._get(k)[i]))
        print("tag                 =", self.tag[i])
        print("inactive            =", self.inactive[i])
        for k in ("tri", "lowerlayer", "last_tri"):
            print(f"{k:<20}=", self._get(k)[i])
        print("last_position       =", np.asarray(self._get("last_position")[i]))

    def drag_coefficient(self, U, dp):
        """lagrangian_particle_set.pyx:790-832 on the host: the constant,
        Schiller-Naumann (1935) or Almedeij (2008) drag coefficient at
        relative speed U and diameter dp, with the powers evaluated as the
        compiled reference and the device do (_cpow_re)."""
        Re = max(EPSILON, U * dp / NU0)
        if self.drag_coef_model == 0:
            return float(self.drag_coef)
        if self.drag_coef_model == 1:
            return (24. / Re) * (1. + 0.15 * _cpow_re(Re, 0.687)) if Re <= 1000. else 0.44
        if self.drag_coef_model == 2:
            phi1 = (24. / Re) ** 10. + _cpow_re(21. * _cpow_re(Re, -0.67), 10.) + \
                _cpow_re(4. * _cpow_re(Re, -0.33), 10.) + 0.4 ** 10.
            phi2 = 1. / (_cpow_re(0.148 * _cpow_re(Re, 0.11), -10.) + 0.5 ** -10.)
            phi3 = _cpow_re(1.57 * _cpow_re(Re, -1.625) * 1.e8, 10.)
            phi4 = 1. / (_cpow_re(6e-17 * _cpow_re(Re, 2.63), -10.) + 0.2 ** -10.)
            return (1. / ((phi1 + phi2) ** -1. + phi3 ** -1.) + phi4) ** (1. / 10.)
        return 0.44

    def buoyancy_velocity(self, dp, model_hr, rho0):
        """lagrangian_particle_set.pyx:834-890 on the host: the user's
        constant, or the settling velocity of Stokes (dp < 1e-4 m), Ruby and
        Zanke (1977, in between), constant-drag turbulent (model_hr 0) or
        Van Rijn (1985) (dp > 1e-3 m); negative for particles denser than
        the fluid."""
        if self.buoyancy_velocity_model == 0:
            return float(self.buoyancy_velocity_value)
        s = self.density / rho0
        if dp < 1.e-4:
            wb = abs(s - 1.) * (GRAV * (dp * dp)) / (18. * NU0)
        elif dp > 1.e-3:
            if model_hr == 0:
                wb = np.sqrt(abs(s - 1.) * (4. * dp * GRAV) / (3. * self.drag_coef))
            else:
                wb = 1.1 * np.sqrt((s - 1.) * GRAV * dp)
        else:
            wb = (10. * NU0 / dp) * (np.sqrt(1. + abs(s - 1.) * GRAV * dp ** 3.0 /
                                             (100. * (NU0 * NU0))) - 1.)
        return float(-wb if s > 1. else wb)

    def delete_single(self, i):
        """lagrangian_particle_set.pyx:754-788"""
        self.delete(np.array([i]))

    def delete(self, particles_id):
        """lagrangian_particle_set.pyx:712-750: deactivates the listed
        particles that are active (an index listed twice is deleted once),
        zeroing their state, and gives them the tags maxtag+1, maxtag+2, ...
        in the order listed.  Particles deleted by earlier steps get their
        tags first (they were deleted before)."""
        ids = np.asarray(particles_id, dtype=np.int64).ravel()
        if len(ids) == 0:
            return
        self._retag()
        gone = self._get("tri") == -1
        order = []
        for i in ids:
            if not gone[i]:
                gone[i] = True
                order.append(i)
        if not order:
            return
        idx = np.array(order, dtype=np.int64)
        for k in ("position", "velocity", "fluid_velocity_seen", "last_position", "last_velocity"):
            a = self._get(k)
            a[idx] = 0.
            self._set(k, a)
        for k, v in (("tri", -1), ("last_tri", -1), ("lowerlayer", 0)):
            a = self._get(k)
            a[idx] = v
            self._set(k, a)
        d = self._get("diameter")
        d[idx] = 0.
        self._set("diameter", d)
        if self.compute_depth:
            d = self._get("depth")
            d[idx] = 0.
            self._set("depth", d)
        t = self._get("tag")
        t[idx] = (self.maxtag + self.tag_stride *
                  np.arange(1, len(idx) + 1, dtype=np.int64)).astype(np.int32)
        self.maxtag += len(idx) * self.tag_stride
        self._set("tag", t)


def c_params(P, dim, density=1000., drag_model=1, drag_coef=0.44, added_mass=False,
             added_mass_coef=0.5, buoyancy_model=0, buoyancy_value=0.0,
             precision=_lib.CG_PRECISION_FP64, seed=0, sort_period=0):
    """The C-ABI parameter block (cg_params) of checked Parameters P and the
    particle-set scalars (lagrangian_particle_set.pyx:158-261)."""
    return _lib.Params(
        P.model, P.time_scheme, P.rng_method, P.diffusion_model, P.diffusion_lsm2_option,
        P.lsm3_edge_opt, int(bool(P.boundary_conditions)), P.boundary_conditions_type,
        P.max_wall_rebounds, int(bool(P.bnd_statistics)), P.particle_velocity_init,
        int(bool(P.frozen_eulerian_fields)), P.initial_time, P.final_time, P.time_step,
        P.horizontal_diffusivity, P.vertical_diffusivity, P.schmidt_number,
        P.diffusion_lsm3_tl_horizontal, P.diffusion_lsm3_tl_vertical,
        P.rebound_damping_coef, P.wall_roughness_angle, P.stranding_probability,
        P.water_density, dim, density, drag_model, drag_coef, int(bool(added_mass)),
        added_mass_coef, buoyancy_model, buoyancy_value, precision, int(seed), int(sort_period))


def retag(tag, maxtag, stride=1):
    """Deleted particles carry a negative marker (-1: deleted while being
    initialized, -2-it: deleted during iteration it); give them maxtag+1,
    maxtag+2, ... in deletion order then index order, as delete_single does
    (lagrangian_particle_set.pyx:786-788); with stride s (a shard of a split
    set), maxtag+s, maxtag+2s, ...  Returns (tags, new maxtag)."""
    tag = np.array(tag, dtype=np.int32, copy=True)
    idx = np.nonzero(tag < 0)[0]
    if len(idx) == 0:
        return tag, maxtag
    order = np.lexsort((idx, -tag[idx]))
    new = np.empty(len(idx), dtype=np.int32)
    new[order] = (maxtag + stride * np.arange(1, len(idx) + 1, dtype=np.int64)).astype(np.int32)
    tag[idx] = new
    return tag, maxtag + stride * len(idx)


def upload_mesh_fields(L, ctx, field_set):
    """cg_mesh_upload + cg_fields_upload of an EulerianFieldSet; returns the
    host arrays that must stay alive until the uploads return."""
    m = field_set.triangular_mesh
    g = m.locator_grid()
    keep = [m.x, m.y, m.triangles, m.gradx, m.grady, m.det, m.edges, m.triedge_map,
            m.edgetri_map, m.edges_labels, g[5], g[6]]
    md = _lib.MeshDesc(m.nv, m.nt, m.ne, m.nopen, m.x.ctypes.data, m.y.ctypes.data,
                       m.triangles.ctypes.data, m.gradx.ctypes.data, m.grady.ctypes.data,
                       m.det.ctypes.data, m.edges.ctypes.data, m.triedge_map.ctypes.data,
                       m.edgetri_map.ctypes.data, m.edges_labels.ctypes.data,
                       g[0], g[1], g[2], g[3], g[4], g[5].ctypes.data, g[6].ctypes.data)
    _lib.check(ctx, L.cg_mesh_upload(ctx, C.byref(md)))
    fs = field_set
    ptr = lambda a: None if a is None else a.ctypes.data
    fd = _lib.FieldsDesc(fs.dim, fs.nlayers, fs.npoints, fs.ntimes, ptr(fs.times),
                         ptr(fs.elevation), ptr(fs.velocity_x), ptr(fs.velocity_y),
                         ptr(fs.velocity_z), ptr(fs._opt.get("turbulent_energy")),
                         ptr(fs._opt.get("dissipation")), ptr(fs._opt.get("bottom")),
                         int(fs.friction_model), float(fs.friction_coefficient))
    _lib.check(ctx, L.cg_fields_upload(ctx, C.byref(fd)))
    return keep


class Solver:
    """Mirror of cylag.Solver (solver.pyx:42-236) running the GPU step.

    Extra keyword arguments (not in the reference): ``precision``
    ('fp64' plain form or 'mixed'), ``seed`` (PCG32 seed of every particle
    stream), ``device`` (CUDA ordinal), ``hbm_budget`` (bytes, 0 = none),
    ``sort_period`` (steps between re-sorts of the particles by element, 0 =
    never; results do not depend on it), ``shard`` ((rank, world): this
    process steps rank's share of the particle set, split as the
    reference's parallel solver splits it (LagrangianParticleSet.
    parallel_split); its exit counts are this rank's, to be summed over
    ranks, e.g. with cylag_gb300.shard.allreduce_sum).
    """

    def __init__(self, field_set, particle_set, parameters={}, sources=None,
                 control_sections=None, precision="fp64", seed=0, device=0, hbm_budget=0,
                 sort_period=25, shard=None):
        self.parameters = Parameters(parameters)
        self.parameters.check_values()
        P = self.parameters
        self.simutime = SimuTime(P.listing, P.initial_time, P.final_time, P.time_step)
        self.sources = sources
        self.control_sections = control_sections
        # solver.pyx:97-103
        P.control_sections = control_sections is not None
        P.ncsec = len(control_sections) if control_sections is not None else 0
        self.particle_set = particle_set
        self.field_set = field_set
        fs, ps = field_set, particle_set
        # one rank of a particle set split across ranks (solver_parallel.pyx:113-179)
        self.shard = None if shard is None else (int(shard[0]), int(shard[1]))
        if self.shard is not None and self.shard[1] > 1:
            ps.parallel_split(*self.shard)
        # solver.pyx:122-132: 3D particles on 2D fields (pseudo-3D) need the
        # free surface and the BOTTOM field
        if fs.dim != ps.dim:
            if fs.dim == 2 and ps.dim == 3:
                if fs.fid_zs == -1 or fs.fid_zb == -1:
                    raise ValueError(
                        "2D EulerianFieldSet with 3D LagrangianParticleSet : EulerianFieldSet "
                        "should contain free surface and bottom fields")
                if P.model != 1:
                    raise NotImplementedError(
                        "pseudo-3D (2D fields, 3D particles) is built for LSM1 (model 1)")
            else:
                raise ValueError(f"EulerianFieldSet dimension ({fs.dim}) does not match "
                                 f"LagrangianParticleSet set dimension ({ps.dim})")
        if P.frozen_eulerian_fields != 1 and P.final_time > fs.times[-1]:
            raise ValueError("final_time > EulerianFieldSet maximum time")
        fs.frozen_hydro = bool(P.frozen_eulerian_fields)
        if fs.ntimes == 1 and not fs.frozen_hydro:
            raise ValueError("EulerianFieldSet has only one time step, use frozen_eulerian_fields=True")
        if P.diffusion_model in (2, 3) and (fs.fid_turbeng == -1 or fs.fid_dissip == -1):
            raise ValueError(f"LSM: diffusion_model={P.diffusion_model} requires 'TURBULENT ENERG.' "
                             "and 'DISSIPATION' fields in EulerianFieldSet")
        prec = {"fp64": _lib.CG_PRECISION_FP64, "plain": _lib.CG_PRECISION_FP64,
                "mixed": _lib.CG_PRECISION_MIXED}.get(precision)
        if prec is None:
            raise ValueError(f"precision must be 'fp64' or 'mixed', got {precision!r}")
        ps.rho0 = P.water_density
        self.L = _lib.load()
        self.device = device
        self.seed = int(seed)
        self._ctx = C.c_void_p()
        _lib.check(None, self.L.cg_ctx_create(device, int(hbm_budget), C.byref(self._ctx)))
        self._upload_mesh_fields()
        ps._attach(self._ctx, device)
        ps._solver = self
        self._prm = c_params(P, ps.dim, ps.density, ps.drag_coef_model, ps.drag_coef,
                             ps.added_mass_force, ps.added_mass_coef, ps.buoyancy_velocity_model,
                             ps.buoyancy_velocity_value, prec, self.seed, sort_period)
        self._run = C.c_void_p()
        self._create_run()
        _lib.check(self._ctx, self.L.cg_run_seed(self._run))
        self.initialize_particle_state()
        nopen = fs.triangular_mesh.nopen
        self.nopen = nopen
        self._bnd_stats_times = []     # every step's exit counts (bnd_statistics())
        self._bnd_stats_data = []
        self._bnd_buf = 0              # how many of them flush_statistics has not written
        self._csec_stats_times = []
        self._csec_stats_data = []
        self._csec_buf = 0
        if P.ncsec:
            from .extra import section_segments
            seg = np.ascontiguousarray(section_segments(control_sections))
            _lib.check(self._ctx, self.L.cg_run_set_sections(self._run, P.ncsec,
                                                             seg.ctypes.data))
        if P.stranding_output:
            _lib.check(self._ctx, self.L.cg_run_set_stranding_output(self._run, 1))
        # solver.pyx:209-220
        if P.bnd_statistics or P.control_sections:
            from .statistics import prepare_secstats_output
            prepare_secstats_output(bool(P.bnd_statistics), nopen, P.output_rep,
                                    P.bnd_statistics_file_name, bool(P.control_sections),
                                    P.ncsec, P.control_sections_file_name)
        # solver.pyx:199-224: particle output header and the initial snapshot
        self._snapshots = None
        if P.output_file:
            from .output import SnapshotWriter, prepare_output
            prepare_output(ps, P.output_rep, P.output_file_format, P.output_file_name, P.model)
            self._snapshots = SnapshotWriter(P, P.model)
            self._snapshots.take(ps, self.simutime.time, 0)

    def _upload_mesh_fields(self):
        self._keep = upload_mesh_fields(self.L, self._ctx, self.field_set)

    def _create_run(self):
        sd = self.particle_set._state_desc()
        _lib.check(self._ctx, self.L.cg_run_create(self._ctx, C.byref(self._prm), C.byref(sd),
                                                   C.byref(self._run)))

    def initialize_particle_state(self, i=None):
        """solver.pyx:238-379, for every particle awaiting initialization."""
        _lib.check(self._ctx, self.L.cg_run_init(self._run))

    def _pool_resized(self):
        """The particle set grew its arrays: the run follows them."""
        sd = self.particle_set._state_desc()
        _lib.check(self._ctx, self.L.cg_run_resize(self._run, C.byref(sd)))

    def _released(self, clock):
        """solver.pyx:445-455: asks every source, in order, at the start of
        the step ``clock`` describes; returns the positions of those that
        release."""
        out = []
        self.field_set._set_record(clock.time)   # solver.pyx:440 precedes the sources
        for k, src in enumerate(self.sources or (), start=1):
            if src.release_condition(clock, self.field_set):
                pos = np.asarray(src.init_positions(self.field_set, self.particle_set.dim),
                                 dtype=np.float64)
                out.append(pos)
                if self.parameters.listing:
                    print(f" ~~> Adding {pos.shape[0]} particles from source {k}")
        return out

    def _add(self, released):
        """Adds the released positions and tells the run which particles its
        next step initializes: those below the pool size the step started
        with (solver.pyx:430, 462-467); entries of a pool grown in this step
        wait for the following one."""
        ps = self.particle_set
        npart0 = ps.npart
        for pos in released:
            ps.add(pos)
        _lib.check(self._ctx, self.L.cg_run_added(self._run, npart0))
        ps._added = ps.npart > npart0

    def _run_steps(self, nsteps):
        P = self.parameters
        nopen = max(1, self.nopen)
        stats = np.zeros((nsteps, nopen), dtype=np.int32)
        rc = self.L.cg_run_step(self._run, nsteps, stats.ctypes.data)
        _lib.check(self._ctx, rc)
        csec = None
        if P.ncsec:
            csec = np.zeros((nsteps, P.ncsec), dtype=np.int32)
            k = C.c_int32()
            _lib.check(self._ctx, self.L.cg_run_section_stats(self._run, csec.ctypes.data,
                                                              C.byref(k)))
        if P.stranding_output:
            cnt = C.c_int32()
            _lib.check(self._ctx, self.L.cg_run_stranded(self._run, None, C.byref(cnt)))
            xyz = np.zeros((cnt.value, 3))
            _lib.check(self._ctx, self.L.cg_run_stranded(self._run, xyz.ctypes.data,
                                                         C.byref(cnt)))
            self.particle_set._append_stranded(xyz)
        for s in range(nsteps):
            if P.bnd_statistics:
                self._bnd_stats_times.append(self.simutime.time)
                self._bnd_stats_data.append(stats[s, : self.nopen].copy())
                self._bnd_buf += 1
            if csec is not None:
                self._csec_stats_times.append(self.simutime.time)
                self._csec_stats_data.append(csec[s].copy())
                self._csec_buf += 1
            self.simutime.increment()

    def forward(self, time_step=None, nsteps=1):
        """solver.pyx:413-585: advances the run by one step (nsteps > 1
        batches several forward calls into one library call; a step in which
        a source releases, or which initializes added particles, starts a
        new call)."""
        if time_step is not None and time_step != self.simutime.time_step:
            raise ValueError("forward(time_step) must equal parameters['time_step']")
        t0 = self.simutime.time
        ps = self.particle_set
        P = self.parameters
        period = P.output_printout_period if self._snapshots is not None else 0
        if not self.sources and not ps._added and not period:
            self._run_steps(nsteps)
        else:
            clock = _SimuTimeView(self.simutime)
            batch = 0
            for _ in range(nsteps):
                released = self._released(clock) if self.sources else []
                if released or ps._added:
                    if batch:
                        self._run_steps(batch)
                        batch = 0
                    self._add(released)
                batch += 1
                clock.advance()
                # solver.pyx:557-566: snapshot after iterations that are
                # multiples of output_printout_period
                if period and clock.iteration % period == 0:
                    self._run_steps(batch)
                    batch = 0
                    self._snapshots.take(ps, self.simutime.time, self.simutime.iteration)
            if batch:
                self._run_steps(batch)
        self._last_forward = (t0, nsteps)

    def solve(self):
        """solver.pyx:382-411"""
        start = _time.time()
        remaining = self.simutime.nt - self.simutime.iteration
        if remaining > 0 and not self.simutime.is_finished:
            self.forward(nsteps=remaining)
        if self._snapshots is not None:
            self._snapshots.wait()
        self.wall_time = _time.time() - start
        self.flush_statistics()

    def flush_statistics(self):
        """solver.pyx:587-630: appends the steps not yet written to the
        boundary and control-section statistics files, writes the stranded
        positions, and empties those buffers."""
        from .statistics import write_secstats_buffer, write_stranded_particles_txt_2d
        P = self.parameters
        if P.bnd_statistics and self._bnd_buf > 0:
            k = self._bnd_buf
            write_secstats_buffer(self._bnd_stats_times[-k:], np.stack(self._bnd_stats_data[-k:]),
                                  k, self.nopen, P.output_rep, P.bnd_statistics_file_name)
            self._bnd_buf = 0
        if P.stranding_output:
            ps = self.particle_set
            write_stranded_particles_txt_2d(P.output_rep, P.stranding_output_file_name,
                                            ps.stranded_positions, ps.stranded_count)
            ps.stranded_count = 0
        if P.control_sections and self._csec_buf > 0:
            k = self._csec_buf
            write_secstats_buffer(self._csec_stats_times[-k:],
                                  np.stack(self._csec_stats_data[-k:]), k, P.ncsec,
                                  P.output_rep, P.control_sections_file_name)
            self._csec_buf = 0

    def bnd_statistics(self):
        """Per-step open-boundary exit counts, [nsteps, nopen] (every step
        since the Solver was made)."""
        if not self._bnd_stats_data:
            return np.zeros((0, self.nopen), dtype=np.int32)
        return np.stack(self._bnd_stats_data)

    def section_statistics(self):
        """Per-step control-section crossing counts, [nsteps, ncsec] (every
        step since the Solver was made)."""
        if not self._csec_stats_data:
            return np.zeros((0, self.parameters.ncsec), dtype=np.int32)
        return np.stack(self._csec_stats_data)

    def last_kernel_ms(self):
        ms, n = C.c_double(), C.c_int32()
        self.L.cg_run_last_kernel_ms(self._run, C.byref(ms), C.byref(n))
        return ms.value, n.value

    # ---- checkpoint / resume -------------------------------------------------
    _CHECKPOINT_ARRAYS = ("position", "velocity", "fluid_velocity_seen", "last_position",
                          "last_velocity", "tri", "last_tri", "lowerlayer", "tag", "diameter",
                          "rng_state", "depth")

    def save_checkpoint(self, file_name):
        """Writes the particle state (every device array, the PCG32 states
        included) and the clock to an .npz file; ``load_checkpoint`` on a
        Solver over the same field set and parameters resumes it bit for
        bit (the reference has no checkpoint: its snapshots lack the random
        streams)."""
        ps = self.particle_set
        ps._sync()
        t, ft, it = C.c_double(), C.c_double(), C.c_int64()
        _lib.check(self._ctx, self.L.cg_run_clock(self._run, C.byref(t), C.byref(ft),
                                                 C.byref(it)))
        arrays = {k: ps._dev[k].cpu().numpy() for k in self._CHECKPOINT_ARRAYS if k in ps._dev}
        np.savez(file_name, npart=ps.npart, maxtag=ps.maxtag, tag_stride=ps.tag_stride,
                 run_time=t.value, fields_time=ft.value, iteration=it.value,
                 simutime=np.array([self.simutime.time, self.simutime.iteration], dtype=np.float64),
                 **arrays)

    def load_checkpoint(self, file_name):
        """Restores a ``save_checkpoint`` file into this Solver's particle set
        (the same pool size) and clock; the next forward() continues the
        checkpointed run."""
        ps = self.particle_set
        f = np.load(file_name)
        if int(f["npart"]) != ps.npart:
            raise ValueError(f"checkpoint of {int(f['npart'])} particles, particle set of "
                             f"{ps.npart}")
        ps._sync()
        torch = _torch()
        for k in self._CHECKPOINT_ARRAYS:
            if k in ps._dev and k in f.files:
                ps._dev[k].copy_(torch.from_numpy(np.ascontiguousarray(f[k])))
        torch.cuda.synchronize()
        ps.maxtag = int(f["maxtag"])
        ps.tag_stride = int(f["tag_stride"])
        self.simutime.time = float(f["simutime"][0])
        self.simutime.iteration = int(f["simutime"][1])
        _lib.check(self._ctx, self.L.cg_run_resume(self._run, float(f["run_time"]),
                                                   float(f["fields_time"]),
                                                   int(f["iteration"])))

    def last_kernel_split_ms(self):
        """Mean ms per step of the last call: (step kernel, walk kernel)."""
        a, b = C.c_double(), C.c_double()
        self.L.cg_run_last_kernel_split_ms(self._run, C.byref(a), C.byref(b))
        return a.value, b.value

    def close(self):
        if getattr(self, "_snapshots", None) is not None:
            self._snapshots.close()
            self._snapshots = None
        if getattr(self, "_run", None):
            # the particle set outlives the run: its arrays get the state
            # held in the run's working copies
            self.L.cg_run_writeback(self._run)
            self.L.cg_ctx_sync(self._ctx)
            self.L.cg_run_destroy(self._run)
            self._run = None
        if getattr(self, "_ctx", None):
            self.L.cg_ctx_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
