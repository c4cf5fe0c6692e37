"""Particle sources and their schedulers (the callers that add particles to
the pool between steps).

Mirrors cylag/extra/scheduler.pyx, cylag/extra/particle_source.pyx and
cylag/extra/initial_conditions.pyx: a ``ParticleSource`` asks its scheduler
at the start of every step (the step-start ``SimuTime``) whether to release,
and then generates its release positions on a regular grid clipped to a
polygon.  The positions go to ``LagrangianParticleSet.add``; the GPU run
initializes and advances them in the same step (``cg_run_added``).

Host-side, like the reference's: these run once per step on a few hundred
numbers, off the particle hot path.
"""
from __future__ import annotations

import math

import numpy as np


# ---------------------------------------------------------------------------
# schedulers (cylag/extra/scheduler.pyx)
# ---------------------------------------------------------------------------
class Scheduler:
    """scheduler.pyx:23-31: never triggers."""
    iteration = 0

    def now(self, simutime):
        return False


class TimeDeltaScheduler(Scheduler):
    """scheduler.pyx:33-46: triggers in the step whose [t, t + dt) holds
    next_time, then moves next_time on by time_delta (one trigger per step
    at most, whatever time_delta is)."""

    def __init__(self, time_delta, ini_time=None):
        if ini_time is None:   # a C double attribute in the reference: None is refused
            raise TypeError("TimeDeltaScheduler: ini_time must be a float")
        self.time_delta = float(time_delta)
        self.next_time = float(ini_time)
        self.iteration = -1

    def now(self, simutime):
        if simutime.time <= self.next_time < simutime.time + simutime.time_step:
            self.next_time += self.time_delta
            self.iteration += 1
            return True
        return False


class IterationDeltaScheduler(Scheduler):
    """scheduler.pyx:48-57: every iteration_delta iterations (0 included)."""

    def __init__(self, iteration_delta):
        self.iteration = -1
        self.iteration_delta = int(iteration_delta)

    def now(self, simutime):
        if simutime.iteration % self.iteration_delta == 0:
            self.iteration += 1
            return True
        return False


class IterationScheduler(Scheduler):
    """scheduler.pyx:59-69: at the listed iterations."""

    def __init__(self, iterations):
        self.iteration = -1
        self.iterations = list(iterations)

    def now(self, simutime):
        if simutime.iteration in self.iterations:
            self.iteration += 1
            return True
        return False


class TimeScheduler(Scheduler):
    """scheduler.pyx:71-84: at the listed times, in order; each one fires in
    the step whose [t, t + dt) holds it (a time already passed blocks the
    ones after it)."""

    def __init__(self, times):
        self.iteration = 0
        self.times = np.array(times, dtype=np.float64)
        self.ntimes = len(self.times)

    def now(self, simutime):
        if self.iteration < self.ntimes:
            t = self.times[self.iteration]
            if simutime.time <= t < simutime.time + simutime.time_step:
                self.iteration += 1
                return True
        return False


class CountScheduler(Scheduler):
    """scheduler.pyx:86-102: ``count`` triggers at linspace(0, final_time,
    count)."""

    def __init__(self, count):
        self.iteration = 0
        self.count = int(count)
        self.is_ready = True

    def now(self, simutime):
        if self.iteration < self.count:
            t = np.linspace(0, simutime.final_time, self.count)[self.iteration]
            if simutime.time <= t < simutime.time + simutime.time_step:
                self.iteration += 1
                return True
        return False


class AlwaysScheduler(Scheduler):
    """scheduler.pyx:104-110: every step."""

    def __init__(self):
        self.iteration = 0

    def now(self, simutime):
        self.iteration += 1
        return True


def schedules(ini_time=0., time_delta=None, iteration_delta=None, times=None,
              iterations=None, count=None, never=None, always=None):
    """scheduler.pyx:112-179: one scheduler from exactly one keyword.
    ``never`` is accepted by the argument count but builds no scheduler,
    which raises ValueError("No argument found") as the reference does."""
    args = [time_delta, iteration_delta, times, iterations, count, never, always]
    n = len(args) - args.count(None)
    if n == 0:
        raise ValueError("At least one of these argument required: time_delta, "
                         "iteration_delta, times, iterations, count, never, always")
    if n > 1:
        raise ValueError("Only one of these arguments possible: time_delta, iteration_delta, "
                         f"times, iterations, count, never, always , got {n}")
    if time_delta is not None:
        return TimeDeltaScheduler(time_delta, ini_time)
    if iteration_delta is not None:
        return IterationDeltaScheduler(iteration_delta)
    if times is not None:
        return TimeScheduler(times)
    if iterations is not None:
        return IterationScheduler(iterations)
    if count is not None:
        return CountScheduler(count)
    if always is not None:
        return AlwaysScheduler()
    raise ValueError("No argument found")


# ---------------------------------------------------------------------------
# release positions (cylag/extra/initial_conditions.pyx, cylag/geom/utils.pyx)
# ---------------------------------------------------------------------------
def polygon_area(x, y):
    """geom/utils.pyx:200-225: shoelace sum over the closed ring, in vertex
    order (the order fixes the rounding, which the particle count of
    ``xy_method=1`` can depend on)."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    n = len(x)
    if n < 3:
        return 0.0
    acc = 0.0
    for i in range(n - 1):
        acc += float(x[i]) * float(y[i + 1]) - float(x[i + 1]) * float(y[i])
    acc += float(x[n - 1]) * float(y[0]) - float(x[0]) * float(y[n - 1])
    return 0.5 * abs(acc)


def points_in_polygon(px, py, poly):
    """Even-odd crossing test of each point against the closed ring
    ``poly`` (the answer of matplotlib's Path.contains_point with radius 0,
    used by initial_conditions.pyx:105-111, for points off the edges)."""
    px = np.asarray(px, dtype=np.float64)
    py = np.asarray(py, dtype=np.float64)
    v = np.asarray(poly, dtype=np.float64)
    inside = np.zeros(px.shape, dtype=bool)
    n = len(v)
    for i in range(n):
        x0, y0 = v[i]
        x1, y1 = v[(i + 1) % n]
        cross = (y0 > py) != (y1 > py)
        if not cross.any():
            continue
        with np.errstate(divide="ignore", invalid="ignore"):
            xc = x0 + (py - y0) * (x1 - x0) / (y1 - y0)
        inside ^= cross & (px < xc)
    return inside


def _grid_counts(poly, poly_area, xy_method, grid_res, xy_npart, xy_density):
    xlim = (float(np.min(poly[:, 0])), float(np.max(poly[:, 0])))
    ylim = (float(np.min(poly[:, 1])), float(np.max(poly[:, 1])))
    if xy_method == 0:
        ni, nj = int(grid_res[0]) + 1, int(grid_res[1]) + 1
    elif xy_method in (1, 2):
        dxy = (1. / math.sqrt(xy_npart / poly_area) if xy_method == 1
               else 1. / math.sqrt(xy_density))
        ni = int((xlim[1] - xlim[0]) / dxy) + 1
        nj = int((ylim[1] - ylim[0]) / dxy) + 1
    else:
        raise ValueError("Invalid initialization method")
    return xlim, ylim, ni, nj


def init_positions_2d(poly, poly_area=None, xy_method=0, grid_res=(5, 5), xy_npart=25,
                      xy_density=25.):
    """initial_conditions.pyx:24-114: cell centres of an (ni-1) x (nj-1)
    grid over the polygon's bounding box, x fastest, those inside kept."""
    poly = np.asarray(poly, dtype=np.float64)
    if poly.shape[0] < 3:
        raise ValueError("Invalid polygon")
    if poly_area is None:
        poly_area = polygon_area(poly[:, 0], poly[:, 1])
    xlim, ylim, ni, nj = _grid_counts(poly, poly_area, xy_method, grid_res, xy_npart,
                                      xy_density)
    xl = np.linspace(xlim[0], xlim[1], ni)
    yl = np.linspace(ylim[0], ylim[1], nj)
    xc = 0.5 * (xl[:-1] + xl[1:])
    yc = 0.5 * (yl[:-1] + yl[1:])
    X, Y = np.meshgrid(xc, yc)             # [nj-1, ni-1]: k = i + j*(ni-1)
    pos = np.stack([X.ravel(), Y.ravel()], axis=1)
    return np.ascontiguousarray(pos[points_in_polygon(pos[:, 0], pos[:, 1], poly)])


def init_positions_3d(poly, poly_area=None, xy_method=0, grid_res=(5, 5, 1), xy_npart=25,
                      xy_density=25., z_method=0, z_npart=1, z_density=1., zmin=0., zmax=1.):
    """initial_conditions.pyx:116-218: the 2D grid repeated on nl-1 levels
    between zmin and zmax (x fastest, then y, then z), those inside kept."""
    poly = np.asarray(poly, dtype=np.float64)
    if poly.shape[0] < 3:
        raise ValueError("Invalid polygon")
    if poly_area is None:
        poly_area = polygon_area(poly[:, 0], poly[:, 1])
    xlim, ylim, ni, nj = _grid_counts(poly, poly_area, xy_method, grid_res, xy_npart,
                                      xy_density)
    if z_method == 0:
        nl = int(grid_res[2]) + 1
    elif z_method == 1:
        nl = int(z_npart) + 1
    elif z_method == 2:
        nl = int(z_density * (zmax - zmin)) + 1
    else:
        raise ValueError("Invalid initialization method")
    xl = np.linspace(xlim[0], xlim[1], ni)
    yl = np.linspace(ylim[0], ylim[1], nj)
    zl = np.linspace(zmin, zmax, nl)
    xc = 0.5 * (xl[:-1] + xl[1:])
    yc = 0.5 * (yl[:-1] + yl[1:])
    zc = 0.5 * (zl[:-1] + zl[1:])
    Z, Y, X = np.meshgrid(zc, yc, xc, indexing="ij")   # k = i + j*(ni-1) + l*(ni-1)*(nj-1)
    pos = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    return np.ascontiguousarray(pos[points_in_polygon(pos[:, 0], pos[:, 1], poly)])


def circle(x0, y0, r, n):
    """initial_conditions.pyx:220-231: n points on a circle."""
    th = np.arange(n) * (2. * np.pi / n)
    return np.stack([x0 + r * np.cos(th), y0 + r * np.sin(th)], axis=1)


# ---------------------------------------------------------------------------
# sources (cylag/extra/particle_source.pyx)
# ---------------------------------------------------------------------------
class ParticleSource:
    """particle_source.pyx:31-112: releases the grid of ``poly`` whenever
    ``scheduler.now(simutime)`` holds."""

    def __init__(self, scheduler, poly, grid_res=np.array([5, 5, 1], dtype=np.int32),
                 xy_method=0, xy_npart=25, xy_density=25., z_method=0, z_npart=1,
                 z_density=1., zmin=0., zmax=1.):
        self.scheduler = scheduler
        self.poly = np.asarray(poly, dtype=np.float64)
        self.poly_area = polygon_area(self.poly[:, 0], self.poly[:, 1])
        self.grid_res = grid_res
        self.xy_method = xy_method
        self.xy_npart = xy_npart
        self.xy_density = xy_density
        self.z_method = z_method
        self.z_npart = z_npart
        self.z_density = z_density
        self.zmin = zmin
        self.zmax = zmax

    def release_condition(self, simutime, field_set):
        return int(bool(self.scheduler.now(simutime)))

    def init_positions(self, field_set, dim=-1):
        if dim == -1:
            dim = field_set.dim
        if dim == 2:
            return init_positions_2d(self.poly, self.poly_area, self.xy_method, self.grid_res,
                                     self.xy_npart, self.xy_density)
        return init_positions_3d(self.poly, self.poly_area, self.xy_method, self.grid_res,
                                 self.xy_npart, self.xy_density, self.z_method, self.z_npart,
                                 self.z_density, self.zmin, self.zmax)


# ---------------------------------------------------------------------------
# release where a field meets a criterion (particle_source.pyx:114-339)
# ---------------------------------------------------------------------------
INTERN_REF = -1          # vertex label of an interior node (constants.pyx:29)
_M64 = (1 << 64) - 1


class HostPCG32:
    """PCG32 (XSH-RR output, 64-bit LCG with multiplier 6364136223846793005;
    M. O'Neill's published generator) on the host, for release positions:
    the same seeding and uniform draw as random_utils.pyx:22-67."""

    def __init__(self, seed=0, stream=0):
        self.state = 0
        self.inc = ((int(stream) << 1) | 1) & _M64
        self.next_u32()
        self.state = (self.state + int(seed)) & _M64
        self.next_u32()

    def next_u32(self):
        old = self.state
        self.state = (old * 6364136223846793005 + self.inc) & _M64
        xs = (((old >> 18) ^ old) >> 27) & 0xFFFFFFFF
        rot = old >> 59
        return ((xs >> rot) | (xs << ((32 - rot) & 31))) & 0xFFFFFFFF

    def uniform(self):
        return self.next_u32() * (1.0 / 4294967296.0)


_CMP = {"eq": np.equal, "neq": np.not_equal, "geq": np.greater_equal,
        "leq": np.less_equal, "gt": np.greater, "lt": np.less}


class ParticleSourceFromField:
    """particle_source.pyx:114-339: releases around the interior nodes where
    a field's value (``val_*``) or its variation to the next record
    (``var_*``) meets ``criteria`` against ``threshold``; each such node gets
    max(1, int(density * dual_area)) particles uniform in the disc of its
    dual-cell area (density = the density field / virtual_mass).

    The reference draws the disc positions from its one global PCG32; here
    the source owns a stream, pcg32_seed(``seed``, ``stream``), or shares the
    HostPCG32 ``rng`` given, so releases do not depend on the particle draws
    (and equal the reference's when the global stream is seeded the same way
    and nothing else draws from it)."""

    def __init__(self, scheduler, field_id_criteria, field_id_density, criteria, threshold,
                 virtual_mass=1., single_release=False, seed=0, stream=0, rng=None):
        self.scheduler = scheduler
        self.field_id_criteria = field_id_criteria
        self.field_id_density = field_id_density
        self.criteria = criteria
        self.threshold = threshold
        self.virtual_mass = virtual_mass
        self.loc = np.empty(0, dtype=np.int64)
        self.single_release = single_release
        self.release_rec = -1
        self.rng = rng if rng is not None else HostPCG32(seed, stream)

    def release_condition(self, simutime, fset):
        rec = fset.record
        if not self.scheduler.now(simutime):
            return 0
        kind, _, op = self.criteria.partition("_")
        if kind not in ("var", "val") or op not in _CMP:
            if kind in ("var", "val"):
                raise ValueError("Unkwown criteria")
            return 0
        field = fset._get_field_from_id(self.field_id_criteria)
        f0 = np.asarray(fset._get_field_slice(field, rec, -1))
        if kind == "var":
            f1 = np.asarray(fset._get_field_slice(field, rec + 1, -1))
            values = f1 - f0
        else:
            values = f0
        self.loc = np.nonzero(_CMP[op](values, self.threshold))[0]
        if len(self.loc) > 0:
            if not self.single_release or rec != self.release_rec:
                self.release_rec = rec
                return 1
        return 0

    def init_positions(self, fset, dim=-1):
        if fset.dim != 2:
            raise ValueError("Dimension must be 2")
        if dim == 3:
            raise ValueError("ParticleSourceFromField only generates 2D positions, "
                             "it cannot be used with a 3D LagrangianParticleSet")
        m = fset.triangular_mesh
        rec = fset.record
        dens = np.asarray(fset._get_field_slice(fset._get_field_from_id(self.field_id_density),
                                                rec, -1))
        va = m.vertex_adjacency
        out = []
        for k in self.loc:
            if m.vertex_labels[k] != INTERN_REF:
                continue
            area = 0.0
            for itri in va[k]:
                if itri != -1:
                    area += abs(float(m.signed_area[itri])) / 3.
            density = float(dens[k]) / self.virtual_mass
            r0 = math.sqrt(area / np.pi)
            if density == 0.:
                continue
            n = max(1, int(density * area))
            x0, y0 = float(m.x[k]), float(m.y[k])
            p = np.zeros((n, 2))
            for j in range(n):
                r = r0 * math.sqrt(self.rng.uniform())
                a = 2. * np.pi * self.rng.uniform()
                p[j, 0] = x0 + r * np.cos(a)
                p[j, 1] = y0 + r * np.sin(a)
            out.append(p)
        return np.concatenate(out, axis=0) if out else np.zeros((0, 2))


# ---------------------------------------------------------------------------
# control sections (cylag/extra/control_shapes.pyx)
# ---------------------------------------------------------------------------
class ControlSection:
    """control_shapes.pyx:7-101: counts the particles whose step crosses the
    section.  As in the reference, ``nseg = poly.shape[1] - 1``, which for an
    (npoint, 2) polyline is 1: only the first segment poly[0] -> poly[1] is
    tested.  The counting itself runs in the GPU step."""

    def __init__(self, poly):
        self.poly = np.asarray(poly, dtype=np.float64)
        self.nseg = self.poly.shape[1] - 1

    def cross(self, pos_0, pos_1):
        for i in range(self.nseg):
            if segments_intersect(pos_0[0], pos_0[1], pos_1[0], pos_1[1],
                                  self.poly[i, 0], self.poly[i, 1],
                                  self.poly[i + 1, 0], self.poly[i + 1, 1]):
                return 1
        return 0


def _orientation(ax, ay, bx, by, cx, cy):
    """geom/utils.pyx:254-280: 0 collinear, 1 clockwise, 2 counter-clockwise."""
    d = (ay - by) * (cx - ax) - (ax - bx) * (cy - ay)
    return 0 if d == 0. else (1 if d > 0. else 2)


def _on_segment(ax, ay, bx, by, cx, cy):
    return min(ax, bx) <= cx <= max(ax, bx) and min(ay, by) <= cy <= max(ay, by)


def segments_intersect(p0x, p0y, p1x, p1y, s0x, s0y, s1x, s1y):
    """intersections.pyx:150-192: segment p0-p1 meets segment s0-s1."""
    o1 = _orientation(p0x, p0y, p1x, p1y, s0x, s0y)
    o2 = _orientation(p0x, p0y, p1x, p1y, s1x, s1y)
    o3 = _orientation(s0x, s0y, s1x, s1y, p0x, p0y)
    o4 = _orientation(s0x, s0y, s1x, s1y, p1x, p1y)
    if o1 != o2 and o3 != o4:
        return 1
    if o1 == 0 and _on_segment(p0x, p0y, p1x, p1y, s0x, s0y):
        return 1
    if o2 == 0 and _on_segment(p0x, p0y, p1x, p1y, s1x, s1y):
        return 1
    if o3 == 0 and _on_segment(s0x, s0y, s1x, s1y, p0x, p0y):
        return 1
    if o4 == 0 and _on_segment(s0x, s0y, s1x, s1y, p1x, p1y):
        return 1
    return 0


def section_segments(sections):
    """[ncsec, 4] {x0, y0, x1, y1} of each section's tested segment, for the
    GPU step; a section with no segment gets NaNs (never crosses)."""
    out = np.full((len(sections), 4), np.nan)
    for c, cs in enumerate(sections):
        poly = np.asarray(cs.poly, dtype=np.float64)
        nseg = poly.shape[1] - 1
        if nseg > 1:
            raise NotImplementedError(
                "control section polygon of shape (n, >2): the reference's nseg = "
                "poly.shape[1] - 1 would test rows as segments")
        if nseg == 1 and poly.shape[0] >= 2:
            out[c] = [poly[0, 0], poly[0, 1], poly[1, 0], poly[1, 1]]
    return out
