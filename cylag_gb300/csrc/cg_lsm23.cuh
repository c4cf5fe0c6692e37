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

#include <type_traits>

namespace cg {

// Arithmetic of the Langevin coefficients (drag law, direct-integrator
// transitions and covariances, Cholesky factors): FP64 in the plain form,
// FP32 in the mixed form (FP32 node records).  Written with R(...) literals
// so that the FP64 instantiation keeps the reference's expressions exactly.
template <typename FT> struct ArithOf { using type = double; };
template <> struct ArithOf<float> { using type = float; };


// lagrangian_particle_set.pyx:790-832.  The Almedeij powers overflow FP32
// at small Re: that law is evaluated in FP64 in both forms.
__device__ __forceinline__ double drag_almedeij(double Re) {
    double phi1 = pow(24. / Re, 10.) + cpow_re(21. * cpow_re(Re, -0.67), 10.) +
                  cpow_re(4. * cpow_re(Re, -0.33), 10.) + pow(0.4, 10.);
    double phi2 = 1. / (cpow_re(0.148 * cpow_re(Re, 0.11), -10.) + pow(0.5, -10.));
    double phi3 = cpow_re(1.57 * cpow_re(Re, -1.625) * 1.e8, 10.);
    double phi4 = 1. / (cpow_re(6e-17 * cpow_re(Re, 2.63), -10.) + pow(0.2, -10.));
    return pow(1. / (1. / (phi1 + phi2) + 1. / phi3) + phi4, 1. / 10.);
}

// DRAG >= 0: the drag law compiled in (the run's drag_coefficient_model)
template <typename R, int DRAG = -1>
__device__ __forceinline__ R drag_coefficient(const DevParams& p, R U, R dp) {
    const int dm = DRAG >= 0 ? DRAG : p.drag_model;
    R Re = fmax(R(EPSILON), U * dp / R(NU0));
    if (dm == 0) return par<R>(p.drag_coef, p.drag_coef32);
    if (dm == 1) {
        if (Re <= R(1000.)) return (R(24.) / Re) * (R(1.) + R(0.15) * cpow_re(Re, R(0.687)));
        return R(0.44);
    }
    if (dm == 2) return R(drag_almedeij((double)Re));
    return R(0.44);
}

// ---------------------------------------------------------------------------
// LSM2 (cylag/lsm/update_state_lsm2.pyx)
// ---------------------------------------------------------------------------

// drag rate ((a1c*(1.5/dp))*Cd)*|slip| (update_state_lsm2.pyx:192-198), in R
template <typename R>
__device__ __forceinline__ double lsm2_a1(const DevParams& p, int dim, double dp, double rx,
                                          double ry, double rz) {
    R x = R(rx), y = R(ry), z = R(rz), d = R(dp);
    R unorm = dim == 2 ? sqrt(x * x + y * y) : sqrt(x * x + y * y + z * z);
    unorm = fmax(R(EPSILON_LSM2), unorm);
    R Cd = drag_coefficient<R>(p, unorm, d);
    return double(par<R>(p.a1c, p.a1c32) * (R(1.5) / d) * Cd * unorm);
}

template <typename FT>
__host__ __device__ constexpr bool is_mixed() { return std::is_same<FT, float>::value; }

// mean velocity (and, when asked, acceleration) at (k, l, px, py, pz) in the
// arithmetic V: FP64 interpolation in the plain form, FP32 from the FP32
// records and barycentrics in the mixed form
// mixed: mean velocity (and acceleration) from the P1 factors P in FP32
template <int DIM, typename FT>
__device__ __forceinline__ void mean_fields32(Particle<DIM, FT>& q,
                                              const typename Particle<DIM, FT>::P1f& P, int l,
                                              float pz, bool want_acc, float& ux, float& uy,
                                              float& uz, float& ax, float& ay, float& az) {
    ax = ay = az = 0.f;
    q.velocity32(P, l, pz, ux, uy, uz);
    if (want_acc) q.accel32(P, l, pz, ux, uy, uz, ax, ay, az);
}

template <typename V, int DIM, typename FT>
__device__ __forceinline__ void mean_fields(Particle<DIM, FT>& q, int k, int l, double px,
                                            double py, double pz, bool want_acc, V& ux, V& uy,
                                            V& uz, V& ax, V& ay, V& az) {
    if constexpr (is_mixed<FT>()) {
        float u, v, w, a, b, c;
        mean_fields32(q, q.p1f_at(k, px, py), l, (float)pz, want_acc, u, v, w, a, b, c);
        ux = V(u); uy = V(v); uz = V(w);
        ax = V(a); ay = V(b); az = V(c);
    } else {
        double u, v, w, a = 0., b = 0., c = 0.;
        q.velocity(k, l, px, py, pz, u, v, w);
        if (want_acc) q.accel(k, l, px, py, pz, u, v, w, a, b, c);
        ux = V(u); uy = V(v); uz = V(w);
        ax = V(a); ay = V(b); az = V(c);
    }
}

// horizontal localization: the exact predicates in the plain form, the
// FP32-filtered ones (same decisions) in the mixed form; element -1 (the
// stage-exit quirk) takes the exact walk in both
template <int DIM, typename FT>
__device__ __forceinline__ void localize(Particle<DIM, FT>& q, int k, double p0x, double p0y,
                                         double x, double y, int& nk, int& bnd) {
    if constexpr (is_mixed<FT>()) xy_localize_filtered(q.m, k, p0x, p0y, x, y, nk, bnd);
    else xy_localize(q.m, k, p0x, p0y, x, y, nk, bnd);
}

template <int DIM, typename FT>
__device__ __forceinline__ int zloc(Particle<DIM, FT>& q, int k, double x, double y, double z) {
    if constexpr (is_mixed<FT>()) return q.z_localize32(k, x, y, z);
    else return q.z_localize(k, x, y, z);
}

// update_state_lsm2.pyx:141-217
template <int DIM, typename FT>
__device__ __forceinline__ void euler_lsm2(Particle<DIM, FT>& q, double dp) {
    const DevParams& p = q.p;
    double dt = p.dt, ux, uy, uz, ax, ay, az;
    double z = DIM == 3 ? q.x[2] : 0.;
    mean_fields<double>(q, q.tri, q.ll, q.x[0], q.x[1], z, p.added_mass, ux, uy, uz, ax, ay, az);
    double a1 = lsm2_a1<typename ArithOf<FT>::type>(p, DIM, dp, ux - q.up[0], uy - q.up[1], DIM == 3 ? uz - q.up[2] : 0.);
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
__device__ __forceinline__ int rk_lsm2(Particle<DIM, FT>& q, double dp) {
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
        mean_fields<double>(q, k, l, xs, ys, zs, p.added_mass, ux, uy, uz, ax, ay, az);
        const double cv = st == 0 ? 0. : (st == 1 ? c1 : (st == 2 ? c2 : 1.));
        double vx, vy, vz = 0.;
        if (st == 0) {
            a1 = lsm2_a1<typename ArithOf<FT>::type>(p, DIM, dp, ux - q.up[0], uy - q.up[1], DIM == 3 ? uz - q.up[2] : 0.);
            vx = q.up[0];
            vy = q.up[1];
            if (DIM == 3) vz = q.up[2];
        } else {
            // (ux - up[0] - c*f)**2 ... evaluated left to right
            double sx = ux - q.up[0] - cv * fx[st - 1];
            double sy = uy - q.up[1] - cv * fy[st - 1];
            double sz = DIM == 3 ? uz - q.up[2] - cv * fz[st - 1] : 0.;
            a1 = lsm2_a1<typename ArithOf<FT>::type>(p, DIM, dp, sx, sy, sz);
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
        localize(q, q.ltri, q.x0[0], q.x0[1], xt, yt, tt, bnd);
        if (DIM == 3) tl = zloc(q, tt, xt, yt, zt);
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

// T_L and eps at the particle from the FP32 records (mixed form)
template <int DIM, typename FT>
__device__ __forceinline__ float keps_tml32p(Particle<DIM, FT>& q,
                                             const typename Particle<DIM, FT>::P1f& P, int l,
                                             float pz, float& ep) {
    float kt;
    q.turb32(P, l, pz, kt, ep);
    ep = fmaxf(ep, (float)EPSILON);
    return (kt / ep) / (0.5f + 0.75f * (float)C0KOLM);
}
template <int DIM, typename FT>
__device__ __forceinline__ float keps_tml32(Particle<DIM, FT>& q, int k, int l, double px,
                                            double py, double pz, float& ep) {
    return keps_tml32p(q, q.p1f_at(k, px, py), l, (float)pz, ep);
}

// B_k^2 terms of the k-epsilon LSM2 diffusion: T_L and (kt, eps) at the
// particle (update_state_lsm2.pyx:1161-1173)
template <int DIM, typename FT>
__device__ __forceinline__ double keps_tml(Particle<DIM, FT>& q, int k, int l, double px,
                                           double py, double pz, double& ep) {
    if constexpr (is_mixed<FT>()) {
        float e;
        float t = keps_tml32(q, k, l, px, py, pz, e);
        ep = e;
        return t;
    }
    P1 f1 = p1_at(q.m, k, px, py);
    double kt;
    q.turb_q(f1, l, pz, kt, ep);
    ep = fmax(ep, EPSILON);
    return (kt / ep) / (0.5 + (3. / 4.) * C0KOLM);
}

// update_state_lsm2.pyx:1088-1230
template <int DIM, typename FT>
__device__ __forceinline__ void euler_maruyama_lsm2_u(Particle<DIM, FT>& q, double dp) {
    const DevParams& p = q.p;
    double dt = p.dt, sqrtdt = p.sqrtdt, ux, uy, uz, ax, ay, az;
    const int diffmod = p.diffmod, nuopt = p.nuopt;
    double z = DIM == 3 ? q.x[2] : 0.;
    mean_fields<double>(q, q.tri, q.ll, q.x[0], q.x[1], z, p.added_mass, ux, uy, uz, ax, ay, az);
    double a1 = lsm2_a1<typename ArithOf<FT>::type>(p, DIM, dp, ux - q.up[0], uy - q.up[1], DIM == 3 ? uz - q.up[2] : 0.);
    double xix = 0., xiy = 0., xiz = 0., diffx = 0., diffy = 0., diffz = 0.;
    if (diffmod != 0) {
        rng_pair_ol(q.rng, p.rng_method, q.z, xix, xiy);
        if (DIM == 3) xiz = rng_single_ol(q.rng, p.rng_method, q.z);
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
template <typename R>
struct Lsm2Coef {
    R beta, D1, D2, force_x, q_uu, q_xu, q_xx;
};

template <typename R>
__device__ __forceinline__ bool lsm2_direct_coefficients(R a1, R dt, Lsm2Coef<R>& c) {
    R r = a1 * dt;
    if (!isfinite(a1) || !isfinite(dt) || a1 < R(0.) || dt < R(0.) || !isfinite(r)) return false;
    c.beta = exp(-r);
    if (r < R(0.1)) {
        R phi1 = R(1.), phi2 = R(0.5), term = R(1.);
        for (int n = 1; n < 13; ++n) {
            term *= -r / (R(n) + R(1.));
            phi1 += term;
            phi2 += term / (R(n) + R(2.));
        }
        c.D1 = dt * phi1;
        c.D2 = dt * r * phi2;
        c.force_x = dt * dt * phi2;
    } else {
        c.D1 = -expm1(-r) / a1;
        c.D2 = dt - c.D1;
        c.force_x = c.D2 / a1;
    }
    c.q_uu = r == R(0.) ? dt : dt * (-expm1(R(-2.) * r) / (R(2.) * r));
    c.q_xu = R(0.5) * c.D1 * c.D1;
    if (r < R(1.)) {
        R term = R(1.) / R(6.), power2 = R(4.), qxx = R(1.) / R(3.);
        for (int n = 1; n < 24; ++n) {
            term *= -r / (R(n) + R(3.));
            power2 *= R(2.);
            qxx += (power2 - R(2.)) * term;
        }
        c.q_xx = qxx * dt * dt * dt;
    } else {
        c.q_xx = ((dt - R(2.) * c.D1 + c.q_uu) / a1) / a1;
    }
    return true;
}

// The mixed form's LSM2 direct integrator on FP32 state
// (update_state_lsm2.pyx:1329-1542): from the start point's P1 factors P0
// and height z0 (in q.ll), the particle velocity up (updated), the fluid
// velocity seen us (set) and the displacement dx.  False, with ERR_NONFINITE
// in q.err and nothing set, when the coefficients are not finite.
// DRAG, AM >= 0: the run's drag law and added mass compiled in (-1: from
// the parameters).
template <int DIM, typename FT, int DRAG = -1, int AM = -1>
__device__ __forceinline__ bool di_lsm2_32(Particle<DIM, FT>& q,
                                           const typename Particle<DIM, FT>::P1f& P0, float z0,
                                           float dp, int diffmod, int nuopt, float* up, float* us,
                                           float* dx) {
    const DevParams& p = q.p;
    float ux, uy, uz, ax, ay, az;
    mean_fields32(q, P0, q.ll, z0, AM >= 0 ? AM != 0 : p.added_mass, ux, uy, uz, ax, ay, az);
    const float sx = ux - up[0], sy = uy - up[1], sz = DIM == 3 ? uz - up[2] : 0.f;
    const float unorm = fmax(float(EPSILON_LSM2), sqrt(sx * sx + sy * sy + sz * sz));
    const float a1 =
        p.a1c32 * (1.5f / dp) * drag_coefficient<float, DRAG>(p, unorm, dp) * unorm;
    const float rdt = p.dt32;
    Lsm2Coef<float> c;
    if (!lsm2_direct_coefficients<float>(a1, rdt, c)) { q.err |= ERR_NONFINITE; return false; }
    const float um_beta = -expm1(-a1 * rdt);
    float b2[3] = {0.f, 0.f, 0.f};
    if (diffmod == 2 || diffmod == 3) {
        float ep;
        const float tml = keps_tml32p(q, P0, q.ll, z0, ep);
        const float rnuz = p.nuz32;
        b2[0] = a1 * a1 * float(C0KOLM) * ep * (tml * tml);
        b2[1] = b2[0];
        if (diffmod == 2) b2[2] = nuopt == 2 ? rnuz * rnuz : 2.f * rnuz * a1 * a1;
        else b2[2] = b2[0];
    } else if (diffmod != 0) {
        const float rnux = p.nux32, rnuz = p.nuz32;
        if (nuopt == 2) {
            b2[0] = rnux * rnux;
            b2[1] = b2[0];
            b2[2] = rnuz * rnuz;
        } else if (nuopt == 3) {
            b2[0] = 2.f * rnux * a1 * a1;
            b2[1] = b2[0];
            b2[2] = 2.f * rnuz * a1 * a1;
        }
    }
    const float mu[3] = {ux, uy, uz};
    const float acc[3] = {ax, ay, az};
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        const float u_k = mu[d];
        const float Fp = d == 2 ? p.a2c32 * acc[2] - float(GRAV) * p.a0c32 : p.a2c32 * acc[d];
        const float v0 = up[d];
        us[d] = u_k;
        float Gp = 0.f, Gx = 0.f;
        if (!(b2[d] == 0.f || rdt == 0.f)) {
            const float var_gp = b2[d] * c.q_uu, cov = b2[d] * c.q_xu, var_gx = b2[d] * c.q_xx;
            const float L_pp = sqrt(fmax(0.f, var_gp));
            const float L_xp = L_pp > 0.f ? cov / L_pp : 0.f;
            const float L_xx = sqrt(fmax(0.f, var_gx - L_xp * L_xp));
            float xix, xiy;
            pair32_ol(q.rng, p.rng_method, *q.z32, xix, xiy);   // FP32 draws
            Gp = L_pp * xix;
            Gx = L_xp * xix + L_xx * xiy;
        }
        up[d] = v0 * c.beta + u_k * um_beta + Fp * c.D1 + Gp;
        dx[d] = v0 * c.D1 + u_k * c.D2 + Fp * c.force_x + Gx;
    }
    return true;
}

// update_state_lsm2.pyx:1329-1542 (diffmod 0, nux = nuz = 0, nuopt 2:
// di_ode_lsm2, 1232-1238).  Mixed form: coefficients, means and increments
// in FP32, one FP64 add per position coordinate.
template <int DIM, typename FT>
__device__ __forceinline__ void di_lsm2(Particle<DIM, FT>& q, double dp, int diffmod, int nuopt) {
    using R = typename ArithOf<FT>::type;
    const DevParams& p = q.p;
    const double dt = p.dt;
    double xp0[3], up0[3];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        xp0[d] = q.x[d];
        up0[d] = q.up[d];
    }
    double z0 = DIM == 3 ? xp0[2] : 0.;
    if constexpr (!std::is_same<R, double>::value) {
        // mixed: the FP32 integrator, one FP64 add per position coordinate
        float up[3] = {0.f, 0.f, 0.f}, us[3], dx[3];
#pragma unroll
        for (int d = 0; d < DIM; ++d) up[d] = float(up0[d]);
        if (!di_lsm2_32(q, q.p1f_at(q.tri, xp0[0], xp0[1]), float(z0), float(dp), diffmod, nuopt,
                        up, us, dx))
            return;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            q.us[d] = double(us[d]);
            q.up[d] = double(up[d]);
            q.x[d] = xp0[d] + double(dx[d]);
        }
        return;
    }
    R ux, uy, uz, ax, ay, az;
    mean_fields<R>(q, q.tri, q.ll, xp0[0], xp0[1], z0, p.added_mass, ux, uy, uz, ax, ay, az);
    R a1 = lsm2_a1<R>(p, DIM, dp, ux - up0[0], uy - up0[1], DIM == 3 ? uz - up0[2] : 0.);
    const R rdt = par<R>(dt, p.dt32);
    Lsm2Coef<R> c;
    if (!lsm2_direct_coefficients<R>(a1, rdt, c)) { q.err |= ERR_NONFINITE; return; }
    R um_beta = -expm1(-a1 * rdt);
    R b2[3] = {R(0.), R(0.), R(0.)};
    if (diffmod == 2 || diffmod == 3) {
        R tml, ep;
        if constexpr (std::is_same<R, double>::value) {
            tml = keps_tml(q, q.tri, q.ll, xp0[0], xp0[1], z0, ep);
        } else {
            tml = keps_tml32(q, q.tri, q.ll, xp0[0], xp0[1], z0, ep);
        }
        const R rnuz = par<R>(p.nuz, p.nuz32);
        b2[0] = a1 * a1 * R(C0KOLM) * ep * (tml * tml);
        b2[1] = b2[0];
        if (diffmod == 2) b2[2] = nuopt == 2 ? rnuz * rnuz : R(2.) * rnuz * a1 * a1;
        else b2[2] = b2[0];
    } else if (diffmod != 0) {
        const R rnux = par<R>(p.nux, p.nux32), rnuz = par<R>(p.nuz, p.nuz32);
        if (nuopt == 2) {
            b2[0] = rnux * rnux;
            b2[1] = b2[0];
            b2[2] = rnuz * rnuz;
        } else if (nuopt == 3) {
            b2[0] = R(2.) * rnux * a1 * a1;
            b2[1] = b2[0];
            b2[2] = R(2.) * rnuz * a1 * a1;
        }
    }
    const R mu[3] = {ux, uy, uz};
    const R acc[3] = {ax, ay, az};
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        const R u_k = mu[d];
        const R a2c = par<R>(p.a2c, p.a2c32);
        const R Fp = d == 2 ? a2c * acc[2] - R(GRAV) * par<R>(p.a0c, p.a0c32) : a2c * acc[d];
        const R v0 = R(up0[d]);
        q.us[d] = double(mu[d]);
        R Gp = R(0.), Gx = R(0.);
        const bool noise = !(b2[d] == R(0.) || rdt == R(0.));
        if (noise) {
            R var_gp = b2[d] * c.q_uu, cov = b2[d] * c.q_xu, var_gx = b2[d] * c.q_xx;
            R L_pp = sqrt(fmax(R(0.), var_gp));
            R L_xp = L_pp > R(0.) ? cov / L_pp : R(0.);
            R L_xx = sqrt(fmax(R(0.), var_gx - L_xp * L_xp));
            R xix, xiy;
            if constexpr (std::is_same<R, double>::value) {
                rng_pair_ol(q.rng, p.rng_method, q.z, xix, xiy);
            } else {
                pair32_ol(q.rng, p.rng_method, *q.z32, xix, xiy);   // FP32 draws (mixed)
            }
            Gp = L_pp * xix;
            Gx = L_xp * xix + L_xx * xiy;
        }
        if constexpr (std::is_same<R, double>::value) {
            double up_mean = up0[d] * c.beta + u_k * um_beta + Fp * c.D1;
            double xp_mean = xp0[d] + up0[d] * c.D1 + u_k * c.D2 + Fp * c.force_x;
            q.up[d] = noise ? up_mean + Gp : up_mean;
            q.x[d] = noise ? xp_mean + Gx : xp_mean;
        } else {
            q.up[d] = double(v0 * c.beta + u_k * um_beta + Fp * c.D1 + Gp);
            q.x[d] = xp0[d] + double(v0 * c.D1 + u_k * c.D2 + Fp * c.force_x + Gx);
        }
    }
}

// update_state_lsm2.pyx:30-139; the final localization is unconditional.
// SCHEME: the time scheme, fixed per kernel instantiation
template <int SCHEME, int DIM, typename FT>
__device__ __forceinline__ int update_lsm2(Particle<DIM, FT>& q, double dp) {
    const DevParams& p = q.p;
    const int diffmod = p.diffmod, nuopt = p.nuopt;
    int bnd_j = -1;
    if (nuopt == 1 || (nuopt >= 2 && diffmod == 0)) {
        if constexpr (SCHEME == 1) euler_lsm2(q, dp);
        else if constexpr (SCHEME == 2) bnd_j = rk_lsm2<2>(q, dp);
        else if constexpr (SCHEME == 3) bnd_j = rk_lsm2<3>(q, dp);
        else if constexpr (SCHEME == 4) bnd_j = rk_lsm2<4>(q, dp);
        else di_lsm2(q, dp, 0, 2);
        if (diffmod != 0) {
            // K and its gradient at the start point only for the k-epsilon models
            P1 q0{};
            if (diffmod == 2 || diffmod == 3) q0 = p1_at(q.m, q.tri0, q.x0[0], q.x0[1]);
            q.diffusion_lsm1(q0);
        }
    } else if constexpr (SCHEME == 1) {
        euler_maruyama_lsm2_u(q, dp);
    } else if constexpr (SCHEME == 5) {
        di_lsm2(q, dp, diffmod, nuopt);
    } else {
        q.err |= ERR_UNSUPPORTED;
        return -1;
    }
    (void)bnd_j;
    q.ltri = q.tri;
    localize(q, q.ltri, q.x0[0], q.x0[1], q.x[0], q.x[1], q.tri, bnd_j);
    if (DIM == 3) q.ll = zloc(q, q.tri, q.x[0], q.x[1], q.x[2]);
    return bnd_j;
}

// init_lsm2_fluctuations.pyx:28-129: stationary velocity fluctuation
template <int DIM, typename FT>
__device__ __forceinline__ void lsm2_fluctuations(Particle<DIM, FT>& q, double dp, double* fl) {
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
        rng_pair_ol(q.rng, p.rng_method, q.z, xix, xiy);
        fl[0] = sqrt(0.5 * b0) * xix;
        fl[1] = sqrt(0.5 * b1) * xiy;
    }
    if (DIM == 3 && b2 > 0.) fl[2] = sqrt(0.5 * b2) * rng_single_ol(q.rng, p.rng_method, q.z);
}

// ---------------------------------------------------------------------------
// LSM3 (cylag/lsm/update_state_lsm3.pyx)
// ---------------------------------------------------------------------------

// frozen-step coefficients of one LSM3 component in state order (s, ur, x):
// phi (transition), q (unit-noise covariance), force, flow
// machine epsilon of the arithmetic type (DBL_EPSILON, FLT_EPSILON)
template <typename R> struct EpsOf { static constexpr double value = 2.220446049250313e-16; };
template <> struct EpsOf<float> { static constexpr float value = 1.1920928955078125e-7f; };

template <typename R>
struct Lsm3Coef {
    R phi[9], q[9], force[3], flow[3];
};

template <typename R>
__device__ __forceinline__ R phi1_(R z) { return z == R(0.) ? R(1.) : expm1(z) / z; }
template <typename R>
__device__ __forceinline__ R exp_divdiff(R x, R y) {
    return exp(-fmin(x, y)) * phi1_(-fabs(x - y));
}
template <typename R>
__device__ __forceinline__ R phi2_(R z) {
    if (fabs(z) < R(0.05))
        return R(0.5) + z * (R(1.) / R(6.) + z * (R(1.) / R(24.) + z * (R(1.) / R(120.) + z * (R(1.) / R(720.) +
               z * (R(1.) / R(5040.) + z * (R(1.) / R(40320.) + z / R(362880.)))))));
    return (expm1(z) - z) / (z * z);
}

template <typename R>
__device__ __forceinline__ bool lsm3_check(R a, R a2, R tl, R dt, Lsm3Coef<R>& c) {
    if (!isfinite(a) || !isfinite(a2) || !isfinite(tl) || !isfinite(dt) || a < R(0.) || tl <= R(0.) ||
        dt < R(0.))
        return false;
    R b = R(1.) / tl;
    if (!isfinite(b) || !isfinite(a * dt) || !isfinite(b * dt) || !isfinite(a * (R(1.) - a2) * dt))
        return false;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        c.phi[k] = R(0.);
        c.q[k] = R(0.);
    }
    c.phi[0] = c.phi[4] = c.phi[8] = R(1.);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        c.force[k] = R(0.);
        c.flow[k] = R(0.);
    }
    return true;
}

template <typename R>
__device__ __forceinline__ bool lsm3_finite(const Lsm3Coef<R>& c) {
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
template <typename R>
__device__ __forceinline__ bool lsm3_direct_coefficients(R a, R a2, R tl, R dt,
                                                Lsm3Coef<R>& c) {
    if (!lsm3_check(a, a2, tl, dt, c)) return false;
    if (dt == R(0.)) return true;
    R b = R(1.) / tl;
    R h = dt;
    int doublings = 0;
    while (h > R(0.) && fmax(a * h, b * h) > R(0.5) && doublings < 2100) {
        h *= R(0.5);
        doublings += 1;
    }
    R ah = a * h, bh = b * h, kh = a * (R(1.) - a2) * h;
    R qb0 = R(1.), qb1 = R(0.), qb2 = R(0.), qb3 = R(0.), qb4 = R(0.), qb5 = R(0.), qb6 = R(0.), qb7 = R(0.),
           qb8 = R(0.), qb9 = R(0.);
    R tss = R(1.), tsp = R(0.), tsx = R(0.), tpp = R(0.), tpx = R(0.), txx = R(0.);
    R tsi = R(0.), tpi = R(0.), txi = R(0.), tii = R(0.);
    R s = R(1.), pp = R(0.), x = R(0.), si = R(0.);
    R sum_p = R(0.), sum_x = R(0.), sum_si = R(0.), int_p = R(0.), int_x = R(0.), int_si = R(0.);
    R beta_term = R(1.), phi1 = R(1.), phi2 = R(0.5);
    for (int n = 1; n < 25; ++n) {
        R divisor = n + R(1.);
        R nss = -R(2.) * bh * tss / divisor;
        R nsp = (tss - (ah + bh) * tsp) / divisor;
        R nsx = (tsp - bh * tsx) / divisor;
        R npp = (R(2.) * tsp - R(2.) * ah * tpp) / divisor;
        R npx = (tsx + tpp - ah * tpx) / divisor;
        R nxx = R(2.) * tpx / divisor;
        R nsi = (tss - bh * tsi) / divisor;
        R npi = (tsi + tsp - ah * tpi) / divisor;
        R nxi = (tpi + tsx) / divisor;
        R nii = R(2.) * tsi / divisor;
        tss = nss; tsp = nsp; tsx = nsx;
        tpp = npp; tpx = npx; txx = nxx;
        tsi = nsi; tpi = npi; txi = nxi; tii = nii;
        qb0 += tss; qb1 += tsp; qb2 += tsx; qb3 += tpp; qb4 += tpx;
        qb5 += txx; qb6 += tsi; qb7 += tpi; qb8 += txi; qb9 += tii;
        R sn = -bh * s / n, pn = (s - ah * pp) / n, xn = pp / n, sin_ = s / n;
        s = sn; pp = pn; x = xn; si = sin_;
        sum_p += pp; sum_x += x; sum_si += si;
        int_p += pp / (n + R(1.)); int_x += x / (n + R(1.)); int_si += si / (n + R(1.));
        beta_term *= -ah / n;
        phi1 += beta_term / (n + R(1.));
        phi2 += beta_term / ((n + R(1.)) * (n + R(2.)));
    }
    R* q = c.q;
    R* phi = c.phi;
    q[0] = h * qb0;
    q[1] = q[3] = h * kh * qb1;
    q[2] = q[6] = h * h * (kh * qb2 + a2 * qb6);
    q[4] = h * kh * kh * qb3;
    q[5] = q[7] = h * h * kh * (kh * qb4 + a2 * qb7);
    q[8] = h * h * h * (kh * kh * qb5 + R(2.) * kh * a2 * qb8 + a2 * a2 * qb9);
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
        R work[9], qnew[9];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int cc = 0; cc < 3; ++cc) {
                R value = R(0.);
#pragma unroll
                for (int k = 0; k < r + 1; ++k) value += phi[3 * r + k] * q[3 * k + cc];
                work[3 * r + cc] = value;
            }
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int cc = 0; cc < r + 1; ++cc) {
                R value = q[3 * r + cc];
#pragma unroll
                for (int k = 0; k < cc + 1; ++k) value += work[3 * r + k] * phi[3 * cc + k];
                qnew[3 * r + cc] = qnew[3 * cc + r] = value;
            }
#pragma unroll
        for (int k = 0; k < 9; ++k) q[k] = qnew[k];
        c.flow[2] = R(2.) * c.flow[2] + phi[6] * c.flow[0] + phi[7] * c.flow[1];
        c.flow[1] = (R(1.) + phi[4]) * c.flow[1] + phi[3] * c.flow[0];
        c.flow[0] = -expm1(-R(2.) * b * h);
        phi[6] = phi[6] * (R(1.) + phi[0]) + phi[7] * phi[3];
        phi[3] *= phi[0] + phi[4];
        c.force[2] = R(2.) * c.force[2] + phi[7] * phi[7];
        phi[7] *= R(1.) + phi[4];
        c.force[1] = phi[7];
        h *= R(2.);
        phi[0] = exp(-b * h);
        phi[4] = exp(-a * h);
    }
    return lsm3_finite(c);
}

// update_state_lsm3.pyx:235-264
template <typename R>
__device__ __forceinline__ void lsm3_closed_covariance(R a, R b, R a2, R h, R* q) {
    R d = a - b;
    R cc = a * (R(1.) - a2) / d;
    R bb = (R(1.) - a2) / d;
    R aa = (a2 + cc) / b;
    R sb = h * phi1_(-b * h), sa = h * phi1_(-a * h);
    R s2b = h * phi1_(-R(2.) * b * h), s2a = h * phi1_(-R(2.) * a * h);
    R sab = h * phi1_(-(a + b) * h);
    q[0] = s2b;
    q[1] = q[3] = cc * (s2b - sab);
    q[2] = q[6] = aa * (sb - s2b) - bb * (sb - sab);
    q[4] = cc * cc * (s2b - R(2.) * sab + s2a);
    q[5] = q[7] = cc * (aa * (sb - s2b - sa + sab) - bb * (sb - sab - sa + s2a));
    q[8] = (aa * aa * (h - R(2.) * sb + s2b) - R(2.) * aa * bb * (h - sb - sa + sab) +
            bb * bb * (h - R(2.) * sa + s2a));
}

// update_state_lsm3.pyx:266-307
template <typename R>
__device__ __forceinline__ void lsm3_clipped_covariance(R a, R b, R a2, R h, R* q) {
    R d = a - b, m = R(0.5) * (a + b), x = m * h, delta;
    if (x > R(1.)) delta = fmin(R(0.5), R(LSM3_CLIP_STEP) * sqrt(x)) / h;
    else delta = fmin(R(0.5), R(LSM3_CLIP_STEP) / sqrt(x)) * m;
    if (fabs(d) >= delta) {
        lsm3_closed_covariance(a, b, a2, h, q);
    } else {
        R qp[9], qm[9];
        lsm3_closed_covariance(m + R(0.5) * delta, m - R(0.5) * delta, a2, h, qp);
        lsm3_closed_covariance(m - R(0.5) * delta, m + R(0.5) * delta, a2, h, qm);
        R w = R(0.5) * (R(1.) + d / delta);
#pragma unroll
        for (int k = 0; k < 9; ++k) q[k] = qm[k] + w * (qp[k] - qm[k]);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) q[4 * k] = fmax(q[4 * k], R(0.));
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int cc = 0; cc < r; ++cc) {
            R bound = sqrt(q[4 * r] * q[4 * cc]);
            q[3 * r + cc] = q[3 * cc + r] = fmax(-bound, fmin(bound, q[3 * r + cc]));
        }
}

// update_state_lsm3.pyx:309-374 (lsm3_edge_opt = 2, the default)
template <typename R>
__device__ __forceinline__ bool lsm3_clipped_coefficients(R a, R a2, R tl, R dt,
                                                 Lsm3Coef<R>& c) {
    if (!lsm3_check(a, a2, tl, dt, c)) return false;
    if (dt == R(0.)) return true;
    R b = R(1.) / tl;
    R ah = a * dt, bh = b * dt, k = a * (R(1.) - a2);
    R alpha = exp(-bh), beta = exp(-ah);
    R divdiff = exp_divdiff(ah, bh);
    R ib = dt * phi1_(-bh), ia = dt * phi1_(-ah);
    c.phi[0] = alpha;
    c.phi[3] = k * dt * divdiff;
    c.phi[4] = beta;
    c.phi[6] = ib - (R(1.) - a2) * dt * divdiff;
    c.phi[7] = ia;
    c.force[1] = ia;
    c.force[2] = dt * dt * phi2_(-ah);
    c.flow[0] = -expm1(-bh);
    c.flow[1] = k * dt * (phi1_(-ah) - divdiff);
    c.flow[2] = (a2 * (dt - ib) + (R(1.) - a2) * (dt - ia - ib + dt * divdiff));
    lsm3_clipped_covariance(a, b, a2, dt, c.q);
    return lsm3_finite(c);
}

// out of line: called for the horizontal and (when T_L differs) the
// vertical time scale, one copy of the code; the coefficients come back by
// value (no caller state needs an address)
template <typename R>
struct Lsm3CoefOut {
    Lsm3Coef<R> c;
    bool ok;
};

template <typename R>
__device__ __noinline__ Lsm3CoefOut<R> lsm3_coefficients_ol(R a, R a2, R tl, R dt, int edge_opt) {
    Lsm3CoefOut<R> o;
    o.ok = edge_opt == 2 ? lsm3_clipped_coefficients(a, a2, tl, dt, o.c)
                         : lsm3_direct_coefficients(a, a2, tl, dt, o.c);
    return o;
}

template <typename R>
__device__ __forceinline__ bool lsm3_coefficients(R a, R a2, R tl, R dt, int edge_opt,
                                                  Lsm3Coef<R>& c) {
    const Lsm3CoefOut<R> o = lsm3_coefficients_ol<R>(a, a2, tl, dt, edge_opt);
    c = o.c;
    return o.ok;
}

// update_state_lsm3.pyx:523-557 (strict: only roundoff-sized negative pivots clip)
template <typename R>
__device__ __forceinline__ bool lsm3_cholesky(const R* q, R* lower) {
#pragma unroll
    for (int k = 0; k < 9; ++k) lower[k] = R(0.);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        R pivot = q[3 * r + r];
#pragma unroll
        for (int cc = 0; cc < r; ++cc) {
            R residual = q[3 * r + cc];
#pragma unroll
            for (int k = 0; k < cc; ++k) residual -= lower[3 * r + k] * lower[3 * cc + k];
            if (lower[3 * cc + cc] > R(0.)) {
                lower[3 * r + cc] = residual / lower[3 * cc + cc];
            } else {
                R tol = (R(128.) * EpsOf<R>::value * sqrt(fabs(q[3 * r + r])) * sqrt(fabs(q[3 * cc + cc])));
                if (fabs(residual) > tol) return false;
            }
            pivot -= lower[3 * r + cc] * lower[3 * r + cc];
        }
        if (pivot < R(0.)) {
            if (-pivot > R(128.) * EpsOf<R>::value * fabs(q[3 * r + r])) return false;
            pivot = R(0.);
        }
        lower[3 * r + r] = sqrt(pivot);
    }
    return true;
}

// update_state_lsm3.pyx:559-585
template <typename R>
__device__ __forceinline__ void lsm3_cholesky_clipped(const R* q, R* lower) {
#pragma unroll
    for (int k = 0; k < 9; ++k) lower[k] = R(0.);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        R remaining = fmax(q[3 * r + r], R(0.));
#pragma unroll
        for (int cc = 0; cc < r; ++cc) {
            if (lower[3 * cc + cc] > R(0.)) {
                R value = q[3 * r + cc];
#pragma unroll
                for (int k = 0; k < cc; ++k) value -= lower[3 * r + k] * lower[3 * cc + k];
                value /= lower[3 * cc + cc];
                if (value * value > remaining) value = copysign(sqrt(remaining), value);
                lower[3 * r + cc] = value;
                remaining -= value * value;
            }
        }
        lower[3 * r + r] = sqrt(fmax(remaining, R(0.)));
    }
}

// drag rate ((a1c*(1.5/dp))*unorm)*Cd (update_state_lsm3.pyx:728)
template <typename R, int DRAG = -1>
__device__ __forceinline__ R lsm3_a1(const DevParams& p, R dp, R unorm) {
    R Cd = drag_coefficient<R, DRAG>(p, unorm, dp);
    return par<R>(p.a1c, p.a1c32) * (R(1.5) / dp) * unorm * Cd;
}

template <int DIM>
__device__ __forceinline__ double slip_norm(const double* us, const double* up) {
    double unorm = (us[0] - up[0]) * (us[0] - up[0]) + (us[1] - up[1]) * (us[1] - up[1]);
    if (DIM == 3) unorm += (us[2] - up[2]) * (us[2] - up[2]);
    return unorm;
}

// update_state_lsm3.pyx:664-820
template <int DIM, typename FT>
__device__ __forceinline__ void euler_maruyama_lsm3(Particle<DIM, FT>& q, double dp) {
    const DevParams& p = q.p;
    double dt = p.dt, sqrtdt = p.sqrtdt, ux, uy, uz, ax, ay, az;
    const int diffmod = p.diffmod;
    double z = DIM == 3 ? q.x[2] : 0.;
    mean_fields<double>(q, q.tri, q.ll, q.x[0], q.x[1], z, true, ux, uy, uz, ax, ay, az);
    using R = typename ArithOf<FT>::type;
    const double unorm = fmax(EPSILON_LSM2, sqrt(slip_norm<DIM>(q.us, q.up)));
    const double a1 = double(lsm3_a1<R>(p, R(dp), R(unorm)));
    double xix, xiy, xiz = 0.;
    rng_pair_ol(q.rng, p.rng_method, q.z, xix, xiy);
    if (DIM == 3) xiz = rng_single_ol(q.rng, p.rng_method, q.z);
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

// The mixed form's LSM3 direct integrator on FP32 state
// (update_state_lsm3.pyx:822-996): from the start point's P1 factors P0 and
// height z0 (in q.ll), the particle velocity up and fluid velocity seen us
// (both updated) and the displacement dx.  False, with ERR_NONFINITE in
// q.err and nothing set, when a coefficient or factor is not finite.
// DRAG, KEPS, EDGE2, AM >= 0: the run's drag law, k-epsilon diffusion
// (diffusion model 2 or 3) or not, lsm3_edge_opt 2 or not and added mass or
// not compiled in (-1: from the parameters).
template <int DIM, typename FT, int DRAG = -1, int KEPS = -1, int EDGE2 = -1, int AM = -1>
__device__ __forceinline__ bool di_lsm3_32(Particle<DIM, FT>& q,
                                           const typename Particle<DIM, FT>::P1f& P0, float z0,
                                           float dp, float* up, float* us, float* dx) {
    const DevParams& p = q.p;
    // (a form without k-epsilon diffusion: only "not 2 or 3" matters)
    const int diffmod = KEPS == 0 ? 1 : p.diffmod, edge_opt = EDGE2 == 1 ? 2 : p.edge_opt;
    float ux, uy, uz, ax, ay, az, ep = 0.f, tml_ke = 0.f;
    mean_fields32(q, P0, q.ll, z0, true, ux, uy, uz, ax, ay, az);
    if (diffmod == 2 || diffmod == 3) tml_ke = keps_tml32p(q, P0, q.ll, z0, ep);
    const float sx = us[0] - up[0], sy = us[1] - up[1], sz = DIM == 3 ? us[2] - up[2] : 0.f;
    const float unorm = fmax(float(EPSILON_LSM2), sqrt(sx * sx + sy * sy + sz * sz));
    const float a1 = lsm3_a1<float, DRAG>(p, dp, unorm);
    const float a2 = AM == 0 ? 0.f : (AM == 1 || p.added_mass ? p.a2c32 : 0.f);
    float tl_h = p.tl_h32, tl_v = p.tl_v32, sigma_h, sigma_v = 0.f;
    if (diffmod == 2 || diffmod == 3) {
        tl_h = fmax(float(EPSILON_LSM3), tml_ke);
        sigma_h = sqrt(float(C0KOLM) * ep);
    } else {
        sigma_h = sqrt(2.f * p.nux32) / tl_h;
    }
    if (DIM == 3) {
        if (diffmod == 3) {
            tl_v = tl_h;
            sigma_v = sigma_h;
        } else {
            sigma_v = sqrt(2.f * p.nuz32) / tl_v;
        }
    }
    const float mean_flow[3] = {ux, uy, uz}, mean_acc[3] = {ax, ay, az};
    Lsm3Coef<float> c;
    float lower[9];
    const float rdt = p.dt32;
    if (!lsm3_coefficients<float>(a1, a2, tl_h, rdt, edge_opt, c)) {
        q.err |= ERR_NONFINITE;
        return false;
    }
    float nus[3], nup[3], ndx[3];
    bool factored = false;
    float sigma_s = sigma_h;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        float tl_k = tl_h;
        if (d == 2) {
            tl_k = tl_v;
            sigma_s = sigma_v;
            if (tl_v != tl_h) {
                if (!lsm3_coefficients<float>(a1, a2, tl_v, rdt, edge_opt, c)) {
                    q.err |= ERR_NONFINITE;
                    return false;
                }
                factored = false;
            }
        }
        const float u_k = mean_flow[d], acc = mean_acc[d];
        const float Fp = d == 2 ? -float(GRAV) * p.a0c32 : 0.f;
        const float s0 = us[d];
        const float ur0 = up[d] - a2 * s0;
        float us_mean = (s0 * c.phi[0] + u_k * c.flow[0] + acc * tl_k * c.flow[0]);
        float ur_mean = (ur0 * c.phi[4] + s0 * c.phi[3] + u_k * c.flow[1] +
                         acc * tl_k * c.flow[1] + Fp * c.force[1]);
        // the position's mean without x0 (added by the caller)
        float xp_mean = (ur0 * c.force[1] + s0 * c.phi[6] + u_k * c.flow[2] +
                         acc * tl_k * c.flow[2] + Fp * c.force[2]);
        if (sigma_s > 0.f && c.q[0] > 0.f) {
            if (!factored) {
                if (edge_opt == 2) {
                    lsm3_cholesky_clipped<float>(c.q, lower);
                } else if (!lsm3_cholesky<float>(c.q, lower)) {
                    q.err |= ERR_NONFINITE;
                    return false;
                }
                factored = true;
            }
            float xix, xiy = 0.f, xiz = 0.f;   // FP32 draws
            if (lower[4] > 0.f) pair32_ol(q.rng, p.rng_method, *q.z32, xix, xiy);
            else xix = single32_ol(q.rng, p.rng_method, *q.z32);
            if (lower[8] > 0.f) xiz = single32_ol(q.rng, p.rng_method, *q.z32);
            us_mean += sigma_s * lower[0] * xix;
            ur_mean += sigma_s * (lower[3] * xix + lower[4] * xiy);
            xp_mean += sigma_s * (lower[6] * xix + lower[7] * xiy + lower[8] * xiz);
        }
        nus[d] = us_mean;
        nup[d] = ur_mean + a2 * us_mean;
        ndx[d] = xp_mean;
    }
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        us[d] = nus[d];
        up[d] = nup[d];
        dx[d] = ndx[d];
    }
    return true;
}

// update_state_lsm3.pyx:822-996.  Mixed form: coefficients, Cholesky factor,
// means and increments in FP32, one FP64 add per position coordinate.
template <int DIM, typename FT>
__device__ __forceinline__ void di_lsm3(Particle<DIM, FT>& q, double dp) {
    using R = typename ArithOf<FT>::type;
    constexpr bool exact = std::is_same<R, double>::value;
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
    if constexpr (!exact) {
        // mixed: the FP32 integrator, one FP64 add per position coordinate
        float up[3] = {0.f, 0.f, 0.f}, us[3] = {0.f, 0.f, 0.f}, dx[3];
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            up[d] = float(up0[d]);
            us[d] = float(us0[d]);
        }
        if (!di_lsm3_32(q, q.p1f_at(q.tri, xp0[0], xp0[1]), float(z0), float(dp), up, us, dx))
            return;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            q.us[d] = double(us[d]);
            q.up[d] = double(up[d]);
            q.x[d] = xp0[d] + double(dx[d]);
        }
        return;
    }
    R ux, uy, uz, ax, ay, az, ep = R(0.), tml_ke = R(0.);
    mean_fields<R>(q, q.tri, q.ll, xp0[0], xp0[1], z0, true, ux, uy, uz, ax, ay, az);
    if (diffmod == 2 || diffmod == 3) {
        if constexpr (exact) tml_ke = keps_tml(q, q.tri, q.ll, xp0[0], xp0[1], z0, ep);
        else tml_ke = keps_tml32(q, q.tri, q.ll, xp0[0], xp0[1], z0, ep);
    }
    R unorm;
    if constexpr (exact) {
        unorm = fmax(EPSILON_LSM2, sqrt(slip_norm<DIM>(us0, up0)));
    } else {
        R sx = R(us0[0]) - R(up0[0]), sy = R(us0[1]) - R(up0[1]);
        R sz = DIM == 3 ? R(us0[2]) - R(up0[2]) : R(0.);
        unorm = fmax(R(EPSILON_LSM2), sqrt(sx * sx + sy * sy + sz * sz));
    }
    const R a1 = lsm3_a1<R>(p, R(dp), unorm);
    const R a2 = p.added_mass ? par<R>(p.a2c, p.a2c32) : R(0.);
    R tl_h = par<R>(p.tl_h, p.tl_h32), tl_v = par<R>(p.tl_v, p.tl_v32), sigma_h, sigma_v = R(0.);
    if (diffmod == 2 || diffmod == 3) {
        tl_h = fmax(R(EPSILON_LSM3), tml_ke);
        sigma_h = sqrt(R(C0KOLM) * ep);
    } else {
        sigma_h = sqrt(R(2.) * par<R>(p.nux, p.nux32)) / tl_h;
    }
    if (DIM == 3) {
        if (diffmod == 3) {
            tl_v = tl_h;
            sigma_v = sigma_h;
        } else {
            sigma_v = sqrt(R(2.) * par<R>(p.nuz, p.nuz32)) / tl_v;
        }
    }
    const R mean_flow[3] = {ux, uy, uz}, mean_acc[3] = {ax, ay, az};
    Lsm3Coef<R> c;
    R lower[9];
    const R rdt = par<R>(dt, p.dt32);
    if (!lsm3_coefficients<R>(a1, a2, tl_h, rdt, edge_opt, c)) { q.err |= ERR_NONFINITE; return; }
    bool factored = false;
    R sigma_s = sigma_h;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        R tl_k = tl_h;
        if (d == 2) {
            tl_k = tl_v;
            sigma_s = sigma_v;
            if (tl_v != tl_h) {
                if (!lsm3_coefficients<R>(a1, a2, tl_v, rdt, edge_opt, c)) {
                    q.err |= ERR_NONFINITE;
                    return;
                }
                factored = false;
            }
        }
        const R u_k = mean_flow[d], acc = mean_acc[d];
        const R Fp = d == 2 ? -R(GRAV) * par<R>(p.a0c, p.a0c32) : R(0.);
        const R s0 = R(us0[d]);
        const R ur0 = exact ? R(up0[d] - a2 * us0[d]) : R(up0[d]) - a2 * s0;
        R us_mean = (s0 * c.phi[0] + u_k * c.flow[0] + acc * tl_k * c.flow[0]);
        R ur_mean = (ur0 * c.phi[4] + s0 * c.phi[3] + u_k * c.flow[1] +
                     acc * tl_k * c.flow[1] + Fp * c.force[1]);
        // position: the mean without x0 in the mixed form (added in FP64 below)
        R xp_mean;
        if constexpr (exact)
            xp_mean = (xp0[d] + ur0 * c.force[1] + s0 * c.phi[6] + u_k * c.flow[2] +
                       acc * tl_k * c.flow[2] + Fp * c.force[2]);
        else
            xp_mean = (ur0 * c.force[1] + s0 * c.phi[6] + u_k * c.flow[2] +
                       acc * tl_k * c.flow[2] + Fp * c.force[2]);
        if (sigma_s > R(0.) && c.q[0] > R(0.)) {
            if (!factored) {
                if (edge_opt == 2) {
                    lsm3_cholesky_clipped<R>(c.q, lower);
                } else if (!lsm3_cholesky<R>(c.q, lower)) {
                    q.err |= ERR_NONFINITE;
                    return;
                }
                factored = true;
            }
            R xix, xiy = R(0.), xiz = R(0.);
            if constexpr (exact) {
                if (lower[4] > R(0.)) rng_pair_ol(q.rng, p.rng_method, q.z, xix, xiy);
                else xix = rng_single_ol(q.rng, p.rng_method, q.z);
                if (lower[8] > R(0.)) xiz = rng_single_ol(q.rng, p.rng_method, q.z);
            } else {   // FP32 draws (mixed)
                if (lower[4] > R(0.)) pair32_ol(q.rng, p.rng_method, *q.z32, xix, xiy);
                else xix = single32_ol(q.rng, p.rng_method, *q.z32);
                if (lower[8] > R(0.)) xiz = single32_ol(q.rng, p.rng_method, *q.z32);
            }
            us_mean += sigma_s * lower[0] * xix;
            ur_mean += sigma_s * (lower[3] * xix + lower[4] * xiy);
            xp_mean += sigma_s * (lower[6] * xix + lower[7] * xiy + lower[8] * xiz);
        }
        q.us[d] = double(us_mean);
        q.up[d] = double(ur_mean + a2 * us_mean);
        q.x[d] = exact ? double(xp_mean) : xp0[d] + double(xp_mean);
    }
}

// update_state_lsm3.pyx:587-662; the final localization is unconditional
template <int SCHEME, int DIM, typename FT>
__device__ __forceinline__ int update_lsm3(Particle<DIM, FT>& q, double dp) {
    if constexpr (SCHEME == 1) euler_maruyama_lsm3(q, dp);
    else if constexpr (SCHEME == 5) di_lsm3(q, dp);
    else { q.err |= ERR_UNSUPPORTED; return -1; }
    int bnd_j;
    q.ltri = q.tri;
    localize(q, q.ltri, q.x0[0], q.x0[1], q.x[0], q.x[1], q.tri, bnd_j);
    if (DIM == 3) q.ll = zloc(q, q.tri, q.x[0], q.x[1], q.x[2]);
    return bnd_j;
}

// init_lsm3_fluctuations.pyx:28-90: stationary seen-velocity fluctuation
template <int DIM, typename FT>
__device__ __forceinline__ void lsm3_fluctuations(Particle<DIM, FT>& q, double* fl) {
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
        rng_pair_ol(q.rng, p.rng_method, q.z, xix, xiy);
        fl[0] = sigma_h * xix;
        fl[1] = sigma_h * xiy;
    }
    if (DIM == 3) {
        double sigma_v = p.diffmod == 3 ? sigma_h : sqrt(p.nuz / p.tl_v);
        if (sigma_v > 0.) fl[2] = sigma_v * rng_single_ol(q.rng, p.rng_method, q.z);
    }
}

}  // namespace cg
