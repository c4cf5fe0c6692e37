"""Seeded synthetic meshes, fields and particle releases.

One module feeds both the GPU runs and the CPU oracle, so that every
comparison sees identical inputs.  All randomness comes from
``numpy.random.default_rng(seed)`` streams; nothing reads a file.

Workloads (the reference measures on none of its own data sets; these are
the named synthetic shapes):

* ``channel``: a structured rectangle, each quad split along a seeded random
  diagonal; optional vertex jitter (boundary vertices slide along the
  boundary only).
* ``fourier_velocity``: a sum of seeded random Fourier modes.
* ``keps_from_K``: nodal (k, eps) such that (Cmu/sigc) k^2/eps = K, the
  k-epsilon diffusivity of cylag/core/eulerian_field_set.pyx:1995-1997.
"""
from __future__ import annotations

import numpy as np

CMU = 0.09


def channel_mesh(lx: float, ly: float, nx: int, ny: int, seed: int = 0,
                 jitter: float = 0.0):
    """Vertices of an (nx x ny) grid on [0,lx]x[0,ly]; 2*(nx-1)*(ny-1)
    counter-clockwise triangles.  ``jitter`` is the +- fraction of the grid
    spacing by which vertices move (uniform, seeded)."""
    rng = np.random.default_rng(seed)
    xs = np.linspace(0.0, lx, nx)
    ys = np.linspace(0.0, ly, ny)
    X, Y = np.meshgrid(xs, ys, indexing="xy")  # [ny, nx]
    X = X.copy()
    Y = Y.copy()
    if jitter > 0.0:
        dx, dy = lx / (nx - 1), ly / (ny - 1)
        jx = rng.uniform(-jitter, jitter, size=X.shape) * dx
        jy = rng.uniform(-jitter, jitter, size=Y.shape) * dy
        jx[:, 0] = 0.0
        jx[:, -1] = 0.0
        jy[0, :] = 0.0
        jy[-1, :] = 0.0
        X += jx
        Y += jy
    x = X.reshape(-1)
    y = Y.reshape(-1)
    j, i = np.meshgrid(np.arange(ny - 1), np.arange(nx - 1), indexing="ij")
    j = j.reshape(-1)
    i = i.reshape(-1)
    v00 = j * nx + i
    v10 = v00 + 1
    v01 = v00 + nx
    v11 = v01 + 1
    diag = rng.integers(0, 2, size=v00.shape[0]).astype(bool)
    # diag False: split along v00-v11; True: along v10-v01 (both CCW)
    t1 = np.where(diag[:, None], np.stack([v00, v10, v01], 1), np.stack([v00, v10, v11], 1))
    t2 = np.where(diag[:, None], np.stack([v10, v11, v01], 1), np.stack([v00, v11, v01], 1))
    tri = np.empty((2 * len(v00), 3), dtype=np.int32)
    tri[0::2] = t1
    tri[1::2] = t2
    return x, y, tri


def fourier_velocity(x, y, seed: int, nmodes: int = 8, amplitude: float = 0.5,
                     lmin: float = 100.0, lmax: float = 1000.0):
    """Sum of ``nmodes`` modes, each of amplitude amplitude/nmodes, random
    wavelength in [lmin, lmax], random wave direction, phase and velocity
    direction."""
    rng = np.random.default_rng(seed)
    lam = rng.uniform(lmin, lmax, nmodes)
    th = rng.uniform(0.0, 2 * np.pi, nmodes)
    ph = rng.uniform(0.0, 2 * np.pi, nmodes)
    psi = rng.uniform(0.0, 2 * np.pi, nmodes)
    a = amplitude / nmodes
    u = np.zeros_like(x)
    v = np.zeros_like(x)
    for m in range(nmodes):
        k = 2 * np.pi / lam[m]
        c = a * np.cos(k * (x * np.cos(th[m]) + y * np.sin(th[m])) + ph[m])
        u += c * np.cos(psi[m])
        v += c * np.sin(psi[m])
    return u, v


def periodic_K(x, y):
    """K(x,y) = 0.01 + 0.09*(1 + sin(2 pi x/800) cos(2 pi y/400))/2  [m^2/s]."""
    return 0.01 + 0.09 * (1.0 + np.sin(2 * np.pi * x / 800.0) * np.cos(2 * np.pi * y / 400.0)) / 2.0


def keps_from_K(K, sigc: float = 0.72, eps: float = 1.0e-3):
    """Nodal (k, eps) with (Cmu/sigc)*k^2/eps == K (up to rounding)."""
    fac = CMU / sigc
    k = np.sqrt(K * eps / fac)
    return k, np.full_like(K, eps)


def uniform_in_box(n: int, x0, x1, y0, y1, seed: int):
    rng = np.random.default_rng(seed)
    return np.stack([rng.uniform(x0, x1, n), rng.uniform(y0, y1, n)], axis=1)


# ---------------------------------------------------------------------------
# named workloads
# ---------------------------------------------------------------------------

def couette_channel(npart: int = 10_000, seed: int = 0):
    """LSM1 2D plain FP64 case: channel 1000 m x 100 m, 101x11 vertices, random
    diagonals (2,000 triangles), depth 1 m, u = 0.1*(y/100), v = 0, constant
    K = 0.01, particles uniform in x in [400,600], y in [0,100]; dt = 1 s,
    1,000 steps."""
    x, y, tri = channel_mesh(1000.0, 100.0, 101, 11, seed=seed)
    u = 0.1 * (y / 100.0)
    v = np.zeros_like(y)
    pos = uniform_in_box(npart, 400.0, 600.0, 0.0, 100.0, seed=seed + 3)
    params = {"model": 1, "diffusion_model": 1, "horizontal_diffusivity": 0.01,
              "time_scheme": 1, "frozen_eulerian_fields": True,
              "time_step": 1.0, "final_time": 1000.0}
    return dict(x=x, y=y, triangles=tri, times=np.zeros(1),
                elevation=np.ones((1, len(x))), velocity_x=u[None, :],
                velocity_y=v[None, :], opt_fields=None, opt_fields_names=None,
                position=pos, parameters=params, nsteps=1000)


def keps_drift_channel(npart: int = 10_000_000, nx: int = 1001, ny: int = 251,
                       lx: float = 4000.0, ly: float = 1000.0, seed: int = 0,
                       nsteps: int = 2000, dt: float = 0.5, horizon: float = 1200.0):
    """LSM1 2D with diffusivity-gradient drift: 4 km x 1 km, 1001x251 jittered
    vertices (+-0.3 spacing), random diagonals (~5e5 triangles); frames A, B
    600 s apart, each a sum of 8 Fourier modes (amplitude 0.5 m/s,
    wavelengths 100-1000 m); the record sequence is A, B, A at t = 0, 600,
    1200 s so that the 1,000 s horizon never extrapolates (continued A, B,
    ... every 600 s up to `horizon` when a longer one is asked for); K(x,y)
    periodic, passed as nodal k-epsilon (eps = 1e-3, sigc = 0.72); particles
    uniform in the domain; dt = 0.5 s, 2,000 steps."""
    x, y, tri = channel_mesh(lx, ly, nx, ny, seed=seed, jitter=0.3)
    uA, vA = fourier_velocity(x, y, seed + 1)
    uB, vB = fourier_velocity(x, y, seed + 2)
    K = periodic_K(x, y)
    k, eps = keps_from_K(K)
    nrec = max(3, int(np.ceil(horizon / 600.0)) + 1)
    times = 600.0 * np.arange(nrec, dtype=np.float64)
    vx = np.stack([uA if r % 2 == 0 else uB for r in range(nrec)])
    vy = np.stack([vA if r % 2 == 0 else vB for r in range(nrec)])
    elev = np.ones((nrec, len(x)))
    opt = np.stack([np.stack([k] * nrec), np.stack([eps] * nrec)])
    pos = uniform_in_box(npart, 0.0, lx, 0.0, ly, seed=seed + 3)
    params = {"model": 1, "diffusion_model": 2, "time_scheme": 1,
              "schmidt_number": 0.72, "frozen_eulerian_fields": False,
              "time_step": dt, "final_time": nsteps * dt}
    return dict(x=x, y=y, triangles=tri, times=times, elevation=elev,
                velocity_x=vx, velocity_y=vy, opt_fields=opt,
                opt_fields_names=["TURBULENT ENERG.", "DISSIPATION"],
                position=pos, parameters=params, nsteps=nsteps)


# ---------------------------------------------------------------------------
# 3D prismatic (sigma-layer) cases
# ---------------------------------------------------------------------------
C0KOLM = 1.2
KAPPA = 0.41


def bathymetry(x, y, seed: int, hmin: float = 5.0, hmax: float = 30.0,
               lx: float = 2000.0, ly: float = 1000.0, nmodes: int = 4):
    """Smooth seeded depth field in [hmin, hmax]: 4 low-wavenumber modes."""
    rng = np.random.default_rng(seed)
    kx = rng.integers(1, 3, nmodes) * np.pi / lx
    ky = rng.integers(1, 3, nmodes) * np.pi / ly
    ph = rng.uniform(0, 2 * np.pi, (nmodes, 2))
    a = rng.uniform(0.5, 1.0, nmodes)
    s = np.zeros_like(x)
    for m in range(nmodes):
        s += a[m] * np.cos(kx[m] * x + ph[m, 0]) * np.cos(ky[m] * y + ph[m, 1])
    s = s / a.sum()                       # in [-1, 1]
    return hmin + (hmax - hmin) * 0.5 * (1.0 + s)


def sigma_elevation(zb, zs, nplanes: int):
    """Plane elevations z_l = zb + l (zs - zb)/(nplanes-1), flattened layer-major."""
    frac = np.arange(nplanes)[:, None] / (nplanes - 1.0)
    return (zb[None, :] + frac * (zs - zb)[None, :]).reshape(-1)


def loglaw_case(nx: int = 501, ny: int = 201, lx: float = 2000.0, ly: float = 1000.0,
                nplanes: int = 21, npart: int = 4_000_000, seed: int = 0,
                ustar: float = 0.05, z0: float = 0.001, angle_deg: float = 30.0):
    """Sigma-layer channel with a log-law current and parabolic K(z):
    u(z) = (u*/kappa) ln(max(z', z0)/z0) with z' the height above the bed,
    along angle_deg; K = kappa u* z' (1 - z'/h) floored at 1e-6; sigma_w =
    1.25 u*, T_L = K/sigma_w^2; passed as nodal k-epsilon with
    eps = 2K/(C0 T_L^2) and k = (0.5 + 0.75 C0) T_L eps."""
    x, y, tri = channel_mesh(lx, ly, nx, ny, seed=seed, jitter=0.3)
    h = bathymetry(x, y, seed + 7, lx=lx, ly=ly)
    zb = -h
    zs = np.zeros_like(zb)
    elev = sigma_elevation(zb, zs, nplanes)
    zr = elev - np.tile(zb, nplanes)                 # height above bed
    hh = np.tile(h, nplanes)
    speed = (ustar / KAPPA) * np.log(np.maximum(zr, z0) / z0)
    th = np.deg2rad(angle_deg)
    u, v, w = speed * np.cos(th), speed * np.sin(th), np.zeros_like(speed)
    K = np.maximum(KAPPA * ustar * zr * (1.0 - zr / hh), 1e-6)
    sw = 1.25 * ustar
    TL = K / sw ** 2
    eps = 2.0 * K / (C0KOLM * TL ** 2)
    k = (0.5 + 0.75 * C0KOLM) * TL * eps
    rng = np.random.default_rng(seed + 3)
    px = rng.uniform(0.0, lx, npart)
    py = rng.uniform(0.0, ly, npart)
    hp = bathymetry(px, py, seed + 7, lx=lx, ly=ly)
    pz = -hp * rng.uniform(0.02, 0.98, npart)
    return dict(x=x, y=y, triangles=tri, nlayers=nplanes, times=np.zeros(1),
                elevation=elev[None, :], velocity_x=u[None, :], velocity_y=v[None, :],
                velocity_z=w[None, :], opt_fields=np.stack([k[None, :], eps[None, :]]),
                opt_fields_names=["TURBULENT ENERG.", "DISSIPATION"],
                position=np.stack([px, py, pz], axis=1), bathymetry=h)


def lsm2_loglaw_workload(npart: int = 4_000_000, nx: int = 501, ny: int = 201,
                         nplanes: int = 21, seed: int = 0, nsteps: int = 5000, dt: float = 0.1):
    """LSM2 Langevin in the 3D log-law channel (2 km x 1 km, 2e5 triangles at
    the default grid, 21 sigma planes): k-epsilon velocity diffusion on all
    three components (diffusion_model 3, diffusion_lsm2_option 2), direct
    integrator (time_scheme 5), frozen fields; particles rho_p = 1000 kg/m3,
    d_p = 1e-4 m, uniform in the volume; dt = 0.1 s, 5,000 steps."""
    c = loglaw_case(nx=nx, ny=ny, nplanes=nplanes, npart=npart, seed=seed)
    c["dim"] = 3
    c["parameters"] = {"model": 2, "time_scheme": 5, "diffusion_model": 3,
                       "diffusion_lsm2_option": 2, "frozen_eulerian_fields": True,
                       "time_step": dt, "final_time": nsteps * dt}
    c["pset"] = {"particle_density": 1000., "particle_diameter": 1e-4}
    c["nsteps"] = nsteps
    return c


def stokes_diameter(ws, rhop: float = 2650., rho0: float = 1000., nu: float = 1.3e-6,
                    g: float = 9.80665):
    """Diameter whose Stokes settling velocity is ws: ws = (s-1) g d^2 / (18 nu)."""
    return np.sqrt(18.0 * nu * np.asarray(ws) / ((rhop / rho0 - 1.0) * g))


def lsm3_taylor_green_workload(npart: int = 10_000_000, nx: int = 501, ny: int = 201,
                               nplanes: int = 21, seed: int = 0, nsteps: int = 2000,
                               dt: float = 0.2, U0: float = 0.2, L: float = 200.0):
    """LSM3 polydisperse settling on the log-law channel's mesh and bathymetry:
    horizontal Taylor-Green vortex in every layer, u = -U0 sin(pi x/L)
    cos(pi y/L), v = U0 cos(pi x/L) sin(pi y/L), w = 0 (U0 = 0.2 m/s,
    L = 200 m); constant diffusivities K_h = 0.01, K_v = 1e-3 m2/s with
    T_L = 1 s (diffusion_model 1); direct integrator; quartz particles
    (2650 kg/m3) whose Stokes settling velocity is log-normal (median 1 mm/s,
    sigma_ln 0.8), i.e. diameters log-normal with median 3.80e-5 m and
    sigma_ln 0.4; released uniformly in the top 20% of the column;
    dt = 0.2 s, 2,000 steps.  The bed reflects, as in the reference."""
    lx, ly = 2000.0, 1000.0
    x, y, tri = channel_mesh(lx, ly, nx, ny, seed=seed, jitter=0.3)
    h = bathymetry(x, y, seed + 7, lx=lx, ly=ly)
    zb = -h
    zs = np.zeros_like(zb)
    elev = sigma_elevation(zb, zs, nplanes)
    u1 = -U0 * np.sin(np.pi * x / L) * np.cos(np.pi * y / L)
    v1 = U0 * np.cos(np.pi * x / L) * np.sin(np.pi * y / L)
    u, v = np.tile(u1, nplanes), np.tile(v1, nplanes)
    w = np.zeros_like(u)
    rng = np.random.default_rng(seed + 3)
    px = rng.uniform(0.0, lx, npart)
    py = rng.uniform(0.0, ly, npart)
    hp = bathymetry(px, py, seed + 7, lx=lx, ly=ly)
    pz = -hp * rng.uniform(0.0, 0.2, npart)
    ws = 1e-3 * np.exp(0.8 * rng.standard_normal(npart))
    diam = stokes_diameter(ws)
    params = {"model": 3, "time_scheme": 5, "diffusion_model": 1,
              "horizontal_diffusivity": 0.01, "vertical_diffusivity": 1e-3,
              "diffusion_lsm3_tl_horizontal": 1.0, "diffusion_lsm3_tl_vertical": 1.0,
              "frozen_eulerian_fields": True, "time_step": dt, "final_time": nsteps * dt}
    return dict(x=x, y=y, triangles=tri, nlayers=nplanes, dim=3, times=np.zeros(1),
                elevation=elev[None, :], velocity_x=u[None, :], velocity_y=v[None, :],
                velocity_z=w[None, :], position=np.stack([px, py, pz], axis=1),
                diameter=diam, parameters=params, pset={"particle_density": 2650.},
                nsteps=nsteps, bathymetry=h)
