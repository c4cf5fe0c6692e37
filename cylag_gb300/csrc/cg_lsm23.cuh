// cg_lsm23.cuh -- the LSM2 (particle velocity) and LSM3 (velocity seen)
// updates of the fused step, one particle per thread.
//
// Restates cylag/lsm/update_state_lsm2.pyx, update_state_lsm3.pyx,
// init_lsm2_fluctuations.pyx and init_lsm3_fluctuations.pyx in the same
// floating-point expression order, so that the plain form (compiled with
// -fmad=false) agrees with the reference to the rounding of libm
// transcendentals (exp, expm1, log, log1p, pow).  Included by cg_step.cuh
// after the Particle definition.
#pragma once

namespace cg {

// x**y (x > 0) as the compiled reference evaluates it: Cython gives
// double ** double a complex result, computed by the C library's complex
// power exp(y * log x) through the complex logarithm, whose real part is
// log1p((x-1)(x+1))/2 for 0.5 <= x < 2 and log(x) elsewhere.
__device__ __forceinline__ double cpow_re(double x, double y) {
    double L = (x >= 0.5 && x < 2.) ? log1p((x - 1.) * (x + 1.)) / 2. : log(x);
    return exp(y * L);
}

// lagrangian_particle_set.pyx:790-832
__device__ inline double drag_coefficient(const DevParams& p, double U, double dp) {
    double Re = fmax(EPSILON, U * dp / NU0);
    if (p.drag_model == 0) return p.drag_coef;
    if (p.drag_model == 1) {
        if (Re <= 1000.) return (24. / Re) * (1. + 0.15 * cpow_re(Re, 0.687));
        return 0.44;
    }
    if (p.drag_model == 2) {
        double phi1 = pow(24. / Re, 10.) + cpow_re(21. * cpow_re(Re, -0.67), 10.) +
                      cpow_re(4. * cpow_re(Re, -0.33), 10.) + pow(0.4, 10.);
        double phi2 = 1. / (cpow_re(0.148 * cpow_re(Re, 0.11), -10.) + pow(0.5, -10.));
        double phi3 = cpow_re(1.57 * cpow_re(Re, -1.625) * 1.e8, 10.);
        double phi4 = 1. / (cpow_re(6e-17 * cpow_re(Re, 2.63), -10.) + pow(0.2, -10.));
        return pow(1. / (1. / (phi1 + phi2) + 1. / phi3) + phi4, 1. / 10.);
    }
    return 0.44;
}

// ---------------------------------------------------------------------------
// LSM2 (cylag/lsm/update_state_lsm2.pyx)
// ---------------------------------------------------------------------------

// drag rate ((a1c*(1.5/dp))*Cd)*|slip| (update_state_lsm2.pyx:192-198)
__device__ __forceinline__ double lsm2_a1(const DevParams& p, int dim, double dp, double rx,
                                          double ry, double rz) {
    double unorm = dim == 2 ? sqrt(rx * rx + ry * ry) : sqrt(rx * rx + ry * ry + rz * rz);
    unorm = fmax(EPSILON_LSM2, unorm);
    double Cd = drag_coefficient(p, unorm, dp);
    return p.a1c * (1.5 / dp) * Cd * unorm;
}

template <int DIM, typename FT>
__device__ __forceinline__ void mean_fields(Particle<DIM, FT>& q, int k, int l, double px,
                                            double py, double pz, bool want_acc, double& ux,
                                            double& uy, double& uz, double& ax, double& ay,
                                            double& az) {
    q.velocity(k, l, px, py, pz, ux, uy, uz);
    ax = ay = az = 0.;
    if (want_acc) q.accel(k, l, px, py, pz, ux, uy, uz, ax, ay, az);
}

// update_state_lsm2.pyx:141-217
template <int DIM, typename FT>
__device__ void euler_lsm2(Particle<DIM, FT>& q, double dp) {
    const DevParams& p = q.p;
    double dt = p.dt, ux, uy, uz, ax, ay, az;
    double z = DIM == 3 ? q.x[2] : 0.;
    mean_fields(q, q.tri, q.ll, q.x[0], q.x[1], z, p.added_mass, ux, uy, uz, ax, ay, az);
    double a1 = lsm2_a1(p, DIM, dp, ux - q.up[0], uy - q.up[1], DIM == 3 ? uz - q.up[2] : 0.);
    q.us[0] = ux;
    q.us[1] = uy;
    q.up[0] += (ux - q.up[0]) * dt * a1 + ax * p.a2c * dt;
    q.up[1] += (uy - q.up[1]) * dt * a1 + ay * p.a2c * dt;
    q.x[0] += q.up[0] * dt;
    q.x[1] += q.up[1] * dt;
    if (DIM == 3) {
        q.us[2] = uz;
        q.up[2] += (uz - q.up[2]) * dt * a1 + az * p.a2c * dt - GRAV * p.a0c * dt;
        q.x[2] += q.up[2] * dt;
    }
}

// Runge-Kutta schemes of LSM2 (update_state_lsm2.pyx:219-1021).  Stage s
// evaluates U (and the added-mass acceleration) at the stage point, the
// slip against up + c f(s-1), k = (up + c f(s-1)) dt and
// f = (U - (up + c f(s-1))) dt a1 + a a2c dt [- g a0c dt].  A stage point
// that leaves the mesh (or the water column) ends the step with an Euler
// update from the stage just evaluated.  NST = 2, 3, 4.
template <int NST, int DIM, typename FT>
__device__ int rk_lsm2(Particle<DIM, FT>& q, double dp) {
    const DevParams& p = q.p;
    const double dt = p.dt;
    // stage-point and slip coefficients applied to k(s-1) and f(s-1)
    constexpr double c1 = NST == 3 ? 1. / 3. : 0.5;
    constexpr double c2 = NST == 3 ? 2. / 3. : 0.5;
    double kx[NST], ky[NST], kz[NST], fx[NST], fy[NST], fz[NST];
    int k = q.tri, l = q.ll;
    double xs = q.x[0], ys = q.x[1], zs = DIM == 3 ? q.x[2] : 0.;
    double ux = 0., uy = 0., uz = 0., ax = 0., ay = 0., az = 0., a1 = 0.;
#pragma unroll
    for (int st = 0; st < NST; ++st) {
        mean_fields(q, k, l, xs, ys, zs, p.added_mass, ux, uy, uz, ax, ay, az);
        const double cv = st == 0 ? 0. : (st == 1 ? c1 : (st == 2 ? c2 : 1.));
        double vx, vy, vz = 0.;
        if (st == 0) {
            a1 = lsm2_a1(p, DIM, dp, ux - q.up[0], uy - q.up[1], DIM == 3 ? uz - q.up[2] : 0.);
            vx = q.up[0];
            vy = q.up[1];
            if (DIM == 3) vz = q.up[2];
        } else {
            // (ux - up[0] - c*f)**2 ... evaluated left to right
            double sx = ux - q.up[0] - cv * fx[st - 1];
            double sy = uy - q.up[1] - cv * fy[st - 1];
            double sz = DIM == 3 ? uz - q.up[2] - cv * fz[st - 1] : 0.;
            a1 = lsm2_a1(p, DIM, dp, sx, sy, sz);
            vx = q.up[0] + cv * fx[st - 1];
            vy = q.up[1] + cv * fy[st - 1];
            if (DIM == 3) vz = q.up[2] + cv * fz[st - 1];
        }
        kx[st] = vx * dt;
        ky[st] = vy * dt;
        fx[st] = (ux - vx) * dt * a1 + ax * p.a2c * dt;
        fy[st] = (uy - vy) * dt * a1 + ay * p.a2c * dt;
        if (DIM == 3) {
            kz[st] = vz * dt;
            fz[st] = (uz - vz) * dt * a1 + az * p.a2c * dt - GRAV * p.a0c * dt;
        }
        if (st == NST - 1) break;
        // next stage point: x + c*k(st) (c = 1 for the last RK4 stage)
        const double cp = st == 0 ? c1 : (st == 1 ? c2 : 1.);
        double xt = q.x[0] + cp * kx[st], yt = q.x[1] + cp * ky[st];
        double zt = DIM == 3 ? q.x[2] + cp * kz[st] : 0.;
        int tt, tl = 0, bnd;
        q.ltri = q.tri;
        xy_localize(q.m, q.ltri, q.x0[0], q.x0[1], xt, yt, tt, bnd);
        if (DIM == 3) tl = q.z_localize(tt, xt, yt, zt);
        if (bnd != -1 || (DIM == 3 && (tl == -2 || tl == -3))) {
            // Euler step with this stage's U, a and a1 (update_state_lsm2.pyx:315-333)
            q.tri = tt;
            if (DIM == 3) q.ll = tl;
            q.us[0] = ux;
            q.us[1] = uy;
            q.up[0] += (ux - q.up[0]) * dt * a1 + ax * p.a2c * dt;
            q.up[1] += (uy - q.up[1]) * dt * a1 + ay * p.a2c * dt;
            if (DIM == 3) {
                q.us[2] = uz;
                q.up[2] += (uz - q.up[2]) * dt * a1 + az * p.a2c * dt - GRAV * p.a0c * dt;
            }
            q.x[0] += q.up[0] * dt;
            q.x[1] += q.up[1] * dt;
            if (DIM == 3) q.x[2] += q.up[2] * dt;
            return bnd;
        }
        // outside with no boundary crossing: the reference raises at the
        // next interpolation
        if (tt < 0) { q.err |= ERR_INTERP_OUTSIDE; return -1; }
        k = tt;
        l = tl;
        xs = xt;
        ys = yt;
        zs = zt;
    }
    q.us[0] = ux;
    q.us[1] = uy;
    if (DIM == 3) q.us[2] = uz;
    if constexpr (NST == 2) {
        q.up[0] += fx[1];
        q.up[1] += fy[1];
        q.x[0] += kx[1];
        q.x[1] += ky[1];
        if (DIM == 3) {
            q.up[2] += fz[1];
            q.x[2] += kz[1];
        }
    } else if constexpr (NST == 3) {
        q.up[0] += (0.25 * fx[0] + 0.75 * fx[2]);
        q.up[1] += (0.25 * fy[0] + 0.75 * fy[2]);
        q.x[0] += (0.25 * kx[0] + 0.75 * kx[2]);
        q.x[1] += (0.25 * ky[0] + 0.75 * ky[2]);
        if (DIM == 3) {
            q.up[2] += (0.25 * fz[0] + 0.75 * fz[2]);
            q.x[2] += (0.25 * kz[0] + 0.75 * kz[2]);
        }
    } else {
        q.up[0] += (1. / 6.) * (fx[0] + 2. * fx[1] + 2. * fx[2] + fx[3]);
        q.up[1] += (1. / 6.) * (fy[0] + 2. * fy[1] + 2. * fy[2] + fy[3]);
        q.x[0] += (1. / 6.) * (kx[0] + 2. * kx[1] + 2. * kx[2] + kx[3]);
        q.x[1] += (1. / 6.) * (ky[0] + 2. * ky[1] + 2. * ky[2] + ky[3]);
        if (DIM == 3) {
            q.up[2] += (1. / 6.) * (fz[0] + 2. * fz[1] + 2. * fz[2] + fz[3]);
            q.x[2] += (1. / 6.) * (kz[0] + 2. * kz[1] + 2. * kz[2] + kz[3]);
        }
    }
    return -1;
}

// B_k^2 terms of the k-epsilon LSM2 diffusion: T_L and (kt, eps) at the
// particle (update_state_lsm2.pyx:1161-1173)
template <int DIM, typename FT>
__device__ __forceinline__ double keps_tml(Particle<DIM, FT>& q, int k, int l, double px,
                                           double py, double pz, double& ep) {
    P1 f1 = p1_at(q.m, k, px, py);
    double kt;
    q.turb_q(f1, l, pz, kt, ep);
    ep = fmax(ep, EPSILON);
    return (kt / ep) / (0.5 + (3. / 4.) * C0KOLM);
}

// update_state_lsm2.pyx:1088-1230
template <int DIM, typename FT>
__device__ void euler_maruyama_lsm2_u(Particle<DIM, FT>& q, double dp) {
    const DevParams& p = q.p;
    double dt = p.dt, sqrtdt = p.sqrtdt, ux, uy, uz, ax, ay, az;
    const int diffmod = p.diffmod, nuopt = p.nuopt;
    double z = DIM == 3 ? q.x[2] : 0.;
    mean_fields(q, q.tri, q.ll, q.x[0], q.x[1], z, p.added_mass, ux, uy, uz, ax, ay, az);
    double a1 = lsm2_a1(p, DIM, dp, ux - q.up[0], uy - q.up[1], DIM == 3 ? uz - q.up[2] : 0.);
    double xix = 0., xiy = 0., xiz = 0., diffx = 0., diffy = 0., diffz = 0.;
    if (diffmod != 0) {
        rng_pair(q.rng, p.rng_method, q.z, xix, xiy);
        if (DIM == 3) xiz = rng_single(q.rng, p.rng_method, q.z);
    }
    if (diffmod == 2 || diffmod == 3) {
        double ep;
        double tml = keps_tml(q, q.tri, q.ll, q.x[0], q.x[1], z, ep);
        diffx = a1 * tml * sqrt(C0KOLM * ep) * sqrtdt;
        diffy = diffx;
        if (DIM == 3) {
            if (diffmod == 2) diffz = nuopt == 2 ? p.nuz * sqrtdt : a1 * sqrt(2. * p.nuz) * sqrtdt;
            else diffz = diffx;
        }
    } else if (nuopt == 2) {
        diffx = p.nux * sqrtdt;
        diffy = diffx;
        if (DIM == 3) diffz = p.nuz * sqrtdt;
    } else if (nuopt == 3) {
        diffx = a1 * sqrt(2. * p.nux) * sqrtdt;
        diffy = diffx;
        if (DIM == 3) diffz = a1 * sqrt(2. * p.nuz) * sqrtdt;
    }
    q.us[0] = ux;
    q.us[1] = uy;
    q.up[0] += (ux - q.up[0]) * dt * a1 + ax * p.a2c * dt + diffx * xix;
    q.up[1] += (uy - q.up[1]) * dt * a1 + ay * p.a2c * dt + diffy * xiy;
    q.x[0] += q.up[0] * dt;
    q.x[1] += q.up[1] * dt;
    if (DIM == 3) {
        q.us[2] = uz;
        q.up[2] += (uz - q.up[2]) * dt * a1 + az * p.a2c * dt - GRAV * p.a0c * dt + diffz * xiz;
        q.x[2] += q.up[2] * dt;
    }
}

// frozen-step coefficients of one LSM2 component (update_state_lsm2.pyx:1240-1327)
struct Lsm2Coef {
    double beta, D1, D2, force_x, q_uu, q_xu, q_xx;
};

__device__ inline bool lsm2_direct_coefficients(double a1, double dt, Lsm2Coef& c) {
    double r = a1 * dt;
    if (!isfinite(a1) || !isfinite(dt) || a1 < 0. || dt < 0. || !isfinite(r)) return false;
    c.beta = exp(-r);
    if (r < 0.1) {
        double phi1 = 1., phi2 = 0.5, term = 1.;
        for (int n = 1; n < 13; ++n) {
            term *= -r / (n + 1.);
            phi1 += term;
            phi2 += term / (n + 2.);
        }
        c.D1 = dt * phi1;
        c.D2 = dt * r * phi2;
        c.force_x = dt * dt * phi2;
    } else {
        c.D1 = -expm1(-r) / a1;
        c.D2 = dt - c.D1;
        c.force_x = c.D2 / a1;
    }
    c.q_uu = r == 0. ? dt : dt * (-expm1(-2. * r) / (2. * r));
    c.q_xu = 0.5 * c.D1 * c.D1;
    if (r < 1.) {
        double term = 1. / 6., power2 = 4., qxx = 1. / 3.;
        for (int n = 1; n < 24; ++n) {
            term *= -r / (n + 3.);
            power2 *= 2.;
            qxx += (power2 - 2.) * term;
        }
        c.q_xx = qxx * dt * dt * dt;
    } else {
        c.q_xx = ((dt - 2. * c.D1 + c.q_uu) / a1) / a1;
    }
    return true;
}

// update_state_lsm2.pyx:1329-1542 (diffmod 0, nux = nuz = 0, nuopt 2:
// di_ode_lsm2, 1232-1238)
template <int DIM, typename FT>
__device__ void di_lsm2(Particle<DIM, FT>& q, double dp, int diffmod, double nux, double nuz,
                        int nuopt) {
    const DevParams& p = q.p;
    const double dt = p.dt;
    double xp0[3], up0[3];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        xp0[d] = q.x[d];
        up0[d] = q.up[d];
    }
    double z0 = DIM == 3 ? xp0[2] : 0.;
    double ux, uy, uz, ax, ay, az;
    mean_fields(q, q.tri, q.ll, xp0[0], xp0[1], z0, p.added_mass, ux, uy, uz, ax, ay, az);
    double a1 = lsm2_a1(p, DIM, dp, ux - up0[0], uy - up0[1], DIM == 3 ? uz - up0[2] : 0.);
    Lsm2Coef c;
    if (!lsm2_direct_coefficients(a1, dt, c)) { q.err |= ERR_NONFINITE; return; }
    double um_beta = -expm1(-a1 * dt);
    double b2[3] = {0., 0., 0.};
    if (diffmod == 2 || diffmod == 3) {
        double ep;
        double tml = keps_tml(q, q.tri, q.ll, xp0[0], xp0[1], z0, ep);
        b2[0] = a1 * a1 * C0KOLM * ep * (tml * tml);
        b2[1] = b2[0];
        if (diffmod == 2) b2[2] = nuopt == 2 ? nuz * nuz : 2. * nuz * a1 * a1;
        else b2[2] = b2[0];
    } else if (diffmod != 0) {
        if (nuopt == 2) {
            b2[0] = nux * nux;
            b2[1] = b2[0];
            b2[2] = nuz * nuz;
        } else if (nuopt == 3) {
            b2[0] = 2. * nux * a1 * a1;
            b2[1] = b2[0];
            b2[2] = 2. * nuz * a1 * a1;
        }
    }
    const double mu[3] = {ux, uy, uz};
    const double Fp3[3] = {p.a2c * ax, p.a2c * ay, p.a2c * az - GRAV * p.a0c};
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        double u_k = mu[d];
        double Fp = Fp3[d];
        double up_mean = up0[d] * c.beta + u_k * um_beta + Fp * c.D1;
        double xp_mean = xp0[d] + up0[d] * c.D1 + u_k * c.D2 + Fp * c.force_x;
        q.us[d] = u_k;
        if (b2[d] == 0. || dt == 0.) {
            q.up[d] = up_mean;
            q.x[d] = xp_mean;
            continue;
        }
        double var_gp = b2[d] * c.q_uu, cov = b2[d] * c.q_xu, var_gx = b2[d] * c.q_xx;
        double L_pp = sqrt(fmax(0., var_gp));
        double L_xp = L_pp > 0. ? cov / L_pp : 0.;
        double L_xx = sqrt(fmax(0., var_gx - L_xp * L_xp));
        double xix, xiy;
        rng_pair(q.rng, p.rng_method, q.z, xix, xiy);
        q.up[d] = up_mean + L_pp * xix;
        q.x[d] = xp_mean + (L_xp * xix + L_xx * xiy);
    }
}

// update_state_lsm2.pyx:30-139; the final localization is unconditional
template <int DIM, typename FT>
__device__ int update_lsm2(Particle<DIM, FT>& q, double dp) {
    const DevParams& p = q.p;
    const int diffmod = p.diffmod, nuopt = p.nuopt;
    int bnd_j = -1;
    if (nuopt == 1 || (nuopt >= 2 && diffmod == 0)) {
        switch (p.time_scheme) {
            case 1: euler_lsm2(q, dp); break;
            case 2: bnd_j = rk_lsm2<2>(q, dp); break;
            case 3: bnd_j = rk_lsm2<3>(q, dp); break;
            case 4: bnd_j = rk_lsm2<4>(q, dp); break;
            case 5: di_lsm2(q, dp, 0, 0., 0., 2); break;
            default: q.err |= ERR_UNSUPPORTED; return -1;
        }
        if (diffmod != 0) q.diffusion_lsm1(p1_at(q.m, q.tri0, q.x0[0], q.x0[1]));
    } else if (p.time_scheme == 1) {
        euler_maruyama_lsm2_u(q, dp);
    } else if (p.time_scheme == 5) {
        di_lsm2(q, dp, diffmod, p.nux, p.nuz, nuopt);
    } else {
        q.err |= ERR_UNSUPPORTED;
        return -1;
    }
    (void)bnd_j;
    q.ltri = q.tri;
    xy_localize(q.m, q.ltri, q.x0[0], q.x0[1], q.x[0], q.x[1], q.tri, bnd_j);
    if (DIM == 3) q.ll = q.z_localize(q.tri, q.x[0], q.x[1], q.x[2]);
    return bnd_j;
}

// init_lsm2_fluctuations.pyx:28-129: stationary velocity fluctuation
template <int DIM, typename FT>
__device__ void lsm2_fluctuations(Particle<DIM, FT>& q, double dp, double* fl) {
    const DevParams& p = q.p;
    fl[0] = fl[1] = fl[2] = 0.;
    if (p.diffmod == 0) return;
    double unorm = EPSILON_LSM2;
    double Cd = drag_coefficient(p, unorm, dp);
    double a1 = p.a1c * (1.5 / dp) * Cd * unorm;
    if (a1 == 0.) {
        // the reference raises when an explicit amplitude B is nonzero
        if (p.nuopt == 2 && ((p.diffmod != 2 && p.diffmod != 3 && p.nux != 0.) ||
                             (DIM == 3 && p.diffmod != 3 && p.nuz != 0.)))
            q.err |= ERR_NONFINITE;
        return;
    }
    double b0, b1, b2;
    if (p.diffmod == 2 || p.diffmod == 3) {
        double ep;
        double tml = keps_tml(q, q.tri, q.ll, q.x[0], q.x[1], DIM == 3 ? q.x[2] : 0., ep);
        b0 = a1 * C0KOLM * ep * (tml * tml);
        b1 = b0;
        if (p.diffmod == 2) b2 = p.nuopt == 2 ? (p.nuz * p.nuz) / a1 : 2. * p.nuz * a1;
        else b2 = b0;
    } else if (p.nuopt == 2) {
        b0 = (p.nux * p.nux) / a1;
        b1 = b0;
        b2 = (p.nuz * p.nuz) / a1;
    } else {
        b0 = 2. * p.nux * a1;
        b1 = b0;
        b2 = 2. * p.nuz * a1;
    }
    if (b0 > 0.) {
        double xix, xiy;
        rng_pair(q.rng, p.rng_method, q.z, xix, xiy);
        fl[0] = sqrt(0.5 * b0) * xix;
        fl[1] = sqrt(0.5 * b1) * xiy;
    }
    if (DIM == 3 && b2 > 0.) fl[2] = sqrt(0.5 * b2) * rng_single(q.rng, p.rng_method, q.z);
}

// ---------------------------------------------------------------------------
// LSM3 (cylag/lsm/update_state_lsm3.pyx)
// ---------------------------------------------------------------------------

// frozen-step coefficients of one LSM3 component in state order (s, ur, x):
// phi (transition), q (unit-noise covariance), force, flow
struct Lsm3Coef {
    double phi[9], q[9], force[3], flow[3];
};

__device__ __forceinline__ double phi1_(double z) { return z == 0. ? 1. : expm1(z) / z; }
__device__ __forceinline__ double exp_divdiff(double x, double y) {
    return exp(-fmin(x, y)) * phi1_(-fabs(x - y));
}
__device__ __forceinline__ double phi2_(double z) {
    if (fabs(z) < 0.05)
        return 0.5 + z * (1. / 6. + z * (1. / 24. + z * (1. / 120. + z * (1. / 720. +
               z * (1. / 5040. + z * (1. / 40320. + z / 362880.))))));
    return (expm1(z) - z) / (z * z);
}

__device__ inline bool lsm3_check(double a, double a2, double tl, double dt, Lsm3Coef& c) {
    if (!isfinite(a) || !isfinite(a2) || !isfinite(tl) || !isfinite(dt) || a < 0. || tl <= 0. ||
        dt < 0.)
        return false;
    double b = 1. / tl;
    if (!isfinite(b) || !isfinite(a * dt) || !isfinite(b * dt) || !isfinite(a * (1. - a2) * dt))
        return false;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        c.phi[k] = 0.;
        c.q[k] = 0.;
    }
    c.phi[0] = c.phi[4] = c.phi[8] = 1.;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        c.force[k] = 0.;
        c.flow[k] = 0.;
    }
    return true;
}

__device__ inline bool lsm3_finite(const Lsm3Coef& c) {
#pragma unroll
    for (int k = 0; k < 9; ++k)
        if (!isfinite(c.phi[k]) || !isfinite(c.q[k])) return false;
    if (!isfinite(c.force[1]) || !isfinite(c.force[2])) return false;
#pragma unroll
    for (int k = 0; k < 3; ++k)
        if (!isfinite(c.flow[k])) return false;
    return true;
}

// update_state_lsm3.pyx:32-216 (lsm3_edge_opt = 1: normalized Taylor series
// at max(a h, b h) <= 1/2, then step doublings)
__device__ inline bool lsm3_direct_coefficients(double a, double a2, double tl, double dt,
                                                Lsm3Coef& c) {
    if (!lsm3_check(a, a2, tl, dt, c)) return false;
    if (dt == 0.) return true;
    double b = 1. / tl;
    double h = dt;
    int doublings = 0;
    while (h > 0. && fmax(a * h, b * h) > 0.5 && doublings < 2100) {
        h *= 0.5;
        doublings += 1;
    }
    double ah = a * h, bh = b * h, kh = a * (1. - a2) * h;
    double qb0 = 1., qb1 = 0., qb2 = 0., qb3 = 0., qb4 = 0., qb5 = 0., qb6 = 0., qb7 = 0.,
           qb8 = 0., qb9 = 0.;
    double tss = 1., tsp = 0., tsx = 0., tpp = 0., tpx = 0., txx = 0.;
    double tsi = 0., tpi = 0., txi = 0., tii = 0.;
    double s = 1., pp = 0., x = 0., si = 0.;
    double sum_p = 0., sum_x = 0., sum_si = 0., int_p = 0., int_x = 0., int_si = 0.;
    double beta_term = 1., phi1 = 1., phi2 = 0.5;
    for (int n = 1; n < 25; ++n) {
        double divisor = n + 1.;
        double nss = -2. * bh * tss / divisor;
        double nsp = (tss - (ah + bh) * tsp) / divisor;
        double nsx = (tsp - bh * tsx) / divisor;
        double npp = (2. * tsp - 2. * ah * tpp) / divisor;
        double npx = (tsx + tpp - ah * tpx) / divisor;
        double nxx = 2. * tpx / divisor;
        double nsi = (tss - bh * tsi) / divisor;
        double npi = (tsi + tsp - ah * tpi) / divisor;
        double nxi = (tpi + tsx) / divisor;
        double nii = 2. * tsi / divisor;
        tss = nss; tsp = nsp; tsx = nsx;
        tpp = npp; tpx = npx; txx = nxx;
        tsi = nsi; tpi = npi; txi = nxi; tii = nii;
        qb0 += tss; qb1 += tsp; qb2 += tsx; qb3 += tpp; qb4 += tpx;
        qb5 += txx; qb6 += tsi; qb7 += tpi; qb8 += txi; qb9 += tii;
        double sn = -bh * s / n, pn = (s - ah * pp) / n, xn = pp / n, sin_ = s / n;
        s = sn; pp = pn; x = xn; si = sin_;
        sum_p += pp; sum_x += x; sum_si += si;
        int_p += pp / (n + 1.); int_x += x / (n + 1.); int_si += si / (n + 1.);
        beta_term *= -ah / n;
        phi1 += beta_term / (n + 1.);
        phi2 += beta_term / ((n + 1.) * (n + 2.));
    }
    double* q = c.q;
    double* phi = c.phi;
    q[0] = h * qb0;
    q[1] = q[3] = h * kh * qb1;
    q[2] = q[6] = h * h * (kh * qb2 + a2 * qb6);
    q[4] = h * kh * kh * qb3;
    q[5] = q[7] = h * h * kh * (kh * qb4 + a2 * qb7);
    q[8] = h * h * h * (kh * kh * qb5 + 2. * kh * a2 * qb8 + a2 * a2 * qb9);
    phi[0] = exp(-bh);
    phi[3] = kh * sum_p;
    phi[4] = exp(-ah);
    phi[6] = h * (kh * sum_x + a2 * sum_si);
    phi[7] = h * phi1;
    c.force[1] = phi[7];
    c.force[2] = h * h * phi2;
    c.flow[0] = -expm1(-bh);
    c.flow[1] = kh * bh * int_p;
    c.flow[2] = h * bh * (kh * int_x + a2 * int_si);
    for (int n = 0; n < doublings; ++n) {
        // Q(2h) = Q(h) + Phi(h) Q(h) Phi(h)^T, symmetric by construction
        double work[9], qnew[9];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int cc = 0; cc < 3; ++cc) {
                double value = 0.;
#pragma unroll
                for (int k = 0; k < r + 1; ++k) value += phi[3 * r + k] * q[3 * k + cc];
                work[3 * r + cc] = value;
            }
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int cc = 0; cc < r + 1; ++cc) {
                double value = q[3 * r + cc];
#pragma unroll
                for (int k = 0; k < cc + 1; ++k) value += work[3 * r + k] * phi[3 * cc + k];
                qnew[3 * r + cc] = qnew[3 * cc + r] = value;
            }
#pragma unroll
        for (int k = 0; k < 9; ++k) q[k] = qnew[k];
        c.flow[2] = 2. * c.flow[2] + phi[6] * c.flow[0] + phi[7] * c.flow[1];
        c.flow[1] = (1. + phi[4]) * c.flow[1] + phi[3] * c.flow[0];
        c.flow[0] = -expm1(-2. * b * h);
        phi[6] = phi[6] * (1. + phi[0]) + phi[7] * phi[3];
        phi[3] *= phi[0] + phi[4];
        c.force[2] = 2. * c.force[2] + phi[7] * phi[7];
        phi[7] *= 1. + phi[4];
        c.force[1] = phi[7];
        h *= 2.;
        phi[0] = exp(-b * h);
        phi[4] = exp(-a * h);
    }
    return lsm3_finite(c);
}

// update_state_lsm3.pyx:235-264
__device__ inline void lsm3_closed_covariance(double a, double b, double a2, double h, double* q) {
    double d = a - b;
    double cc = a * (1. - a2) / d;
    double bb = (1. - a2) / d;
    double aa = (a2 + cc) / b;
    double sb = h * phi1_(-b * h), sa = h * phi1_(-a * h);
    double s2b = h * phi1_(-2. * b * h), s2a = h * phi1_(-2. * a * h);
    double sab = h * phi1_(-(a + b) * h);
    q[0] = s2b;
    q[1] = q[3] = cc * (s2b - sab);
    q[2] = q[6] = aa * (sb - s2b) - bb * (sb - sab);
    q[4] = cc * cc * (s2b - 2. * sab + s2a);
    q[5] = q[7] = cc * (aa * (sb - s2b - sa + sab) - bb * (sb - sab - sa + s2a));
    q[8] = (aa * aa * (h - 2. * sb + s2b) - 2. * aa * bb * (h - sb - sa + sab) +
            bb * bb * (h - 2. * sa + s2a));
}

// update_state_lsm3.pyx:266-307
__device__ inline void lsm3_clipped_covariance(double a, double b, double a2, double h, double* q) {
    double d = a - b, m = 0.5 * (a + b), x = m * h, delta;
    if (x > 1.) delta = fmin(0.5, LSM3_CLIP_STEP * sqrt(x)) / h;
    else delta = fmin(0.5, LSM3_CLIP_STEP / sqrt(x)) * m;
    if (fabs(d) >= delta) {
        lsm3_closed_covariance(a, b, a2, h, q);
    } else {
        double qp[9], qm[9];
        lsm3_closed_covariance(m + 0.5 * delta, m - 0.5 * delta, a2, h, qp);
        lsm3_closed_covariance(m - 0.5 * delta, m + 0.5 * delta, a2, h, qm);
        double w = 0.5 * (1. + d / delta);
#pragma unroll
        for (int k = 0; k < 9; ++k) q[k] = qm[k] + w * (qp[k] - qm[k]);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) q[4 * k] = fmax(q[4 * k], 0.);
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int cc = 0; cc < r; ++cc) {
            double bound = sqrt(q[4 * r] * q[4 * cc]);
            q[3 * r + cc] = q[3 * cc + r] = fmax(-bound, fmin(bound, q[3 * r + cc]));
        }
}

// update_state_lsm3.pyx:309-374 (lsm3_edge_opt = 2, the default)
__device__ inline bool lsm3_clipped_coefficients(double a, double a2, double tl, double dt,
                                                 Lsm3Coef& c) {
    if (!lsm3_check(a, a2, tl, dt, c)) return false;
    if (dt == 0.) return true;
    double b = 1. / tl;
    double ah = a * dt, bh = b * dt, k = a * (1. - a2);
    double alpha = exp(-bh), beta = exp(-ah);
    double divdiff = exp_divdiff(ah, bh);
    double ib = dt * phi1_(-bh), ia = dt * phi1_(-ah);
    c.phi[0] = alpha;
    c.phi[3] = k * dt * divdiff;
    c.phi[4] = beta;
    c.phi[6] = ib - (1. - a2) * dt * divdiff;
    c.phi[7] = ia;
    c.force[1] = ia;
    c.force[2] = dt * dt * phi2_(-ah);
    c.flow[0] = -expm1(-bh);
    c.flow[1] = k * dt * (phi1_(-ah) - divdiff);
    c.flow[2] = (a2 * (dt - ib) + (1. - a2) * (dt - ia - ib + dt * divdiff));
    lsm3_clipped_covariance(a, b, a2, dt, c.q);
    return lsm3_finite(c);
}

__device__ __forceinline__ bool lsm3_coefficients(double a, double a2, double tl, double dt,
                                                  int edge_opt, Lsm3Coef& c) {
    return edge_opt == 2 ? lsm3_clipped_coefficients(a, a2, tl, dt, c)
                         : lsm3_direct_coefficients(a, a2, tl, dt, c);
}

// update_state_lsm3.pyx:523-557 (strict: only roundoff-sized negative pivots clip)
__device__ inline bool lsm3_cholesky(const double* q, double* lower) {
#pragma unroll
    for (int k = 0; k < 9; ++k) lower[k] = 0.;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        double pivot = q[3 * r + r];
#pragma unroll
        for (int cc = 0; cc < r; ++cc) {
            double residual = q[3 * r + cc];
#pragma unroll
            for (int k = 0; k < cc; ++k) residual -= lower[3 * r + k] * lower[3 * cc + k];
            if (lower[3 * cc + cc] > 0.) {
                lower[3 * r + cc] = residual / lower[3 * cc + cc];
            } else {
                double tol = (128. * DBL_EPS * sqrt(fabs(q[3 * r + r])) * sqrt(fabs(q[3 * cc + cc])));
                if (fabs(residual) > tol) return false;
            }
            pivot -= lower[3 * r + cc] * lower[3 * r + cc];
        }
        if (pivot < 0.) {
            if (-pivot > 128. * DBL_EPS * fabs(q[3 * r + r])) return false;
            pivot = 0.;
        }
        lower[3 * r + r] = sqrt(pivot);
    }
    return true;
}

// update_state_lsm3.pyx:559-585
__device__ inline void lsm3_cholesky_clipped(const double* q, double* lower) {
#pragma unroll
    for (int k = 0; k < 9; ++k) lower[k] = 0.;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        double remaining = fmax(q[3 * r + r], 0.);
#pragma unroll
        for (int cc = 0; cc < r; ++cc) {
            if (lower[3 * cc + cc] > 0.) {
                double value = q[3 * r + cc];
#pragma unroll
                for (int k = 0; k < cc; ++k) value -= lower[3 * r + k] * lower[3 * cc + k];
                value /= lower[3 * cc + cc];
                if (value * value > remaining) value = copysign(sqrt(remaining), value);
                lower[3 * r + cc] = value;
                remaining -= value * value;
            }
        }
        lower[3 * r + r] = sqrt(fmax(remaining, 0.));
    }
}

// drag rate ((a1c*(1.5/dp))*unorm)*Cd (update_state_lsm3.pyx:728)
__device__ __forceinline__ double lsm3_a1(const DevParams& p, double dp, double unorm) {
    double Cd = drag_coefficient(p, unorm, dp);
    return p.a1c * (1.5 / dp) * unorm * Cd;
}

template <int DIM>
__device__ __forceinline__ double slip_norm(const double* us, const double* up) {
    double unorm = (us[0] - up[0]) * (us[0] - up[0]) + (us[1] - up[1]) * (us[1] - up[1]);
    if (DIM == 3) unorm += (us[2] - up[2]) * (us[2] - up[2]);
    return unorm;
}

// update_state_lsm3.pyx:664-820
template <int DIM, typename FT>
__device__ void euler_maruyama_lsm3(Particle<DIM, FT>& q, double dp) {
    const DevParams& p = q.p;
    double dt = p.dt, sqrtdt = p.sqrtdt, ux, uy, uz, ax, ay, az;
    const int diffmod = p.diffmod;
    double z = DIM == 3 ? q.x[2] : 0.;
    mean_fields(q, q.tri, q.ll, q.x[0], q.x[1], z, true, ux, uy, uz, ax, ay, az);
    double unorm = fmax(EPSILON_LSM2, sqrt(slip_norm<DIM>(q.us, q.up)));
    double a1 = lsm3_a1(p, dp, unorm);
    double xix, xiy, xiz = 0.;
    rng_pair(q.rng, p.rng_method, q.z, xix, xiy);
    if (DIM == 3) xiz = rng_single(q.rng, p.rng_method, q.z);
    double ep = 0., tml = 0., unstml, diffx;
    if (diffmod == 2 || diffmod == 3) {
        tml = keps_tml(q, q.tri, q.ll, q.x[0], q.x[1], z, ep);
        unstml = 1. / fmax(EPSILON_LSM3, tml);
        diffx = sqrt(C0KOLM * ep) * sqrtdt;
    } else {
        unstml = 1. / p.tl_h;
        diffx = sqrt(2. * p.nux) * sqrtdt / p.tl_h;
    }
    double diffy = diffx;
    double dusx = (ax + (ux - q.us[0]) * unstml) * dt + diffx * xix;
    double dusy = (ay + (uy - q.us[1]) * unstml) * dt + diffy * xiy;
    q.up[0] += (q.us[0] - q.up[0]) * dt * a1;
    q.up[1] += (q.us[1] - q.up[1]) * dt * a1;
    q.us[0] += dusx;
    q.us[1] += dusy;
    if (p.added_mass) {
        q.up[0] += p.a2c * dusx;
        q.up[1] += p.a2c * dusy;
    }
    q.x[0] += q.up[0] * dt;
    q.x[1] += q.up[1] * dt;
    if (DIM == 3) {
        double diffz;
        if (diffmod == 1 || diffmod == 2) {
            unstml = 1. / p.tl_v;
            diffz = sqrt(2. * p.nuz) * sqrtdt / p.tl_v;
        } else {
            unstml = 1. / fmax(EPSILON_LSM3, tml);
            diffz = sqrt(C0KOLM * ep) * sqrtdt;
        }
        double dusz = (az + (uz - q.us[2]) * unstml) * dt + diffz * xiz;
        q.up[2] += (q.us[2] - q.up[2]) * dt * a1 - GRAV * p.a0c * dt;
        q.us[2] += dusz;
        if (p.added_mass) q.up[2] += p.a2c * dusz;
        q.x[2] += q.up[2] * dt;
    }
}

// update_state_lsm3.pyx:822-996
template <int DIM, typename FT>
__device__ void di_lsm3(Particle<DIM, FT>& q, double dp) {
    const DevParams& p = q.p;
    const double dt = p.dt;
    if (dt == 0.) return;
    const int diffmod = p.diffmod, edge_opt = p.edge_opt;
    double xp0[3], up0[3], us0[3];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        xp0[d] = q.x[d];
        up0[d] = q.up[d];
        us0[d] = q.us[d];
    }
    double z0 = DIM == 3 ? xp0[2] : 0.;
    double ux, uy, uz, ax, ay, az, ep = 0., tml_ke = 0.;
    mean_fields(q, q.tri, q.ll, xp0[0], xp0[1], z0, true, ux, uy, uz, ax, ay, az);
    if (diffmod == 2 || diffmod == 3) tml_ke = keps_tml(q, q.tri, q.ll, xp0[0], xp0[1], z0, ep);
    double unorm = fmax(EPSILON_LSM2, sqrt(slip_norm<DIM>(us0, up0)));
    double a1 = lsm3_a1(p, dp, unorm);
    double a2 = p.added_mass ? p.a2c : 0.;
    double tl_h = p.tl_h, tl_v = p.tl_v, sigma_h, sigma_v = 0.;
    if (diffmod == 2 || diffmod == 3) {
        tl_h = fmax(EPSILON_LSM3, tml_ke);
        sigma_h = sqrt(C0KOLM * ep);
    } else {
        sigma_h = sqrt(2. * p.nux) / tl_h;
    }
    if (DIM == 3) {
        if (diffmod == 3) {
            tl_v = tl_h;
            sigma_v = sigma_h;
        } else {
            sigma_v = sqrt(2. * p.nuz) / tl_v;
        }
    }
    const double mean_flow[3] = {ux, uy, uz}, mean_acc[3] = {ax, ay, az};
    Lsm3Coef c;
    double lower[9];
    if (!lsm3_coefficients(a1, a2, tl_h, dt, edge_opt, c)) { q.err |= ERR_NONFINITE; return; }
    bool factored = false;
    double sigma_s = sigma_h;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        double tl_k = tl_h;
        if (d == 2) {
            tl_k = tl_v;
            sigma_s = sigma_v;
            if (tl_v != tl_h) {
                if (!lsm3_coefficients(a1, a2, tl_v, dt, edge_opt, c)) {
                    q.err |= ERR_NONFINITE;
                    return;
                }
                factored = false;
            }
        }
        double u_k = mean_flow[d];
        double Fp = d == 2 ? -GRAV * p.a0c : 0.;
        double ur0 = up0[d] - a2 * us0[d];
        double us_mean = (us0[d] * c.phi[0] + u_k * c.flow[0] + mean_acc[d] * tl_k * c.flow[0]);
        double ur_mean = (ur0 * c.phi[4] + us0[d] * c.phi[3] + u_k * c.flow[1] +
                          mean_acc[d] * tl_k * c.flow[1] + Fp * c.force[1]);
        double xp_mean = (xp0[d] + ur0 * c.force[1] + us0[d] * c.phi[6] + u_k * c.flow[2] +
                          mean_acc[d] * tl_k * c.flow[2] + Fp * c.force[2]);
        if (sigma_s > 0. && c.q[0] > 0.) {
            if (!factored) {
                if (edge_opt == 2) {
                    lsm3_cholesky_clipped(c.q, lower);
                } else if (!lsm3_cholesky(c.q, lower)) {
                    q.err |= ERR_NONFINITE;
                    return;
                }
                factored = true;
            }
            double xix, xiy, xiz;
            if (lower[4] > 0.) {
                rng_pair(q.rng, p.rng_method, q.z, xix, xiy);
            } else {
                xix = rng_single(q.rng, p.rng_method, q.z);
                xiy = 0.;
            }
            xiz = lower[8] > 0. ? rng_single(q.rng, p.rng_method, q.z) : 0.;
            us_mean += sigma_s * lower[0] * xix;
            ur_mean += sigma_s * (lower[3] * xix + lower[4] * xiy);
            xp_mean += sigma_s * (lower[6] * xix + lower[7] * xiy + lower[8] * xiz);
        }
        q.us[d] = us_mean;
        q.up[d] = ur_mean + a2 * us_mean;
        q.x[d] = xp_mean;
    }
}

// update_state_lsm3.pyx:587-662; the final localization is unconditional
template <int DIM, typename FT>
__device__ int update_lsm3(Particle<DIM, FT>& q, double dp) {
    if (q.p.time_scheme == 1) euler_maruyama_lsm3(q, dp);
    else if (q.p.time_scheme == 5) di_lsm3(q, dp);
    else { q.err |= ERR_UNSUPPORTED; return -1; }
    int bnd_j;
    q.ltri = q.tri;
    xy_localize(q.m, q.ltri, q.x0[0], q.x0[1], q.x[0], q.x[1], q.tri, bnd_j);
    if (DIM == 3) q.ll = q.z_localize(q.tri, q.x[0], q.x[1], q.x[2]);
    return bnd_j;
}

// init_lsm3_fluctuations.pyx:28-90: stationary seen-velocity fluctuation
template <int DIM, typename FT>
__device__ void lsm3_fluctuations(Particle<DIM, FT>& q, double* fl) {
    const DevParams& p = q.p;
    fl[0] = fl[1] = fl[2] = 0.;
    double sigma_h;
    if (p.diffmod == 2 || p.diffmod == 3) {
        double ep;
        double tml = keps_tml(q, q.tri, q.ll, q.x[0], q.x[1], DIM == 3 ? q.x[2] : 0., ep);
        tml = fmax(EPSILON_LSM3, tml);
        sigma_h = sqrt(0.5 * C0KOLM * ep * tml);
    } else {
        sigma_h = sqrt(p.nux / p.tl_h);
    }
    if (sigma_h > 0.) {
        double xix, xiy;
        rng_pair(q.rng, p.rng_method, q.z, xix, xiy);
        fl[0] = sigma_h * xix;
        fl[1] = sigma_h * xiy;
    }
    if (DIM == 3) {
        double sigma_v = p.diffmod == 3 ? sigma_h : sqrt(p.nuz / p.tl_v);
        if (sigma_v > 0.) fl[2] = sigma_v * rng_single(q.rng, p.rng_method, q.z);
    }
}

}  // namespace cg
