// cg_step.cuh -- the fused per-particle step (one thread per particle).
//
// One launch replaces the body of the particle loop of Solver.forward
// (cylag/core/solver.pyx:459-524): the LSM update (advection scheme,
// diffusion with k-epsilon drift, buoyancy), re-localization by path walk,
// and the boundary conditions (wall rebound, open exit, bed/surface
// reflection, deletion).  Everything for one particle stays in registers;
// the only global traffic is the particle's own state and the gathers of
// its element's mesh and node data (L2-resident for meshes up to ~1e6
// triangles).
#pragma once

#include "cg_device.cuh"

namespace cg {

// ziggurat tables in global memory: blocks copy them to shared memory with
// coalesced loads (constant memory would serialize the 128 distinct indices)
__device__ const ZigTables g_zig = {CG_ZIG_KN_INIT, CG_ZIG_WN_INIT, CG_ZIG_FN_INIT};

template <int DIM, typename FT>
struct Particle {
    const DevMesh& m;
    const DevFields<FT>& f;
    const DevParams& p;
    const ZigTables& z;
    Rng rng;
    double x[3];      // position
    double x0[3];     // position at step start (last_position)
    double up[3];     // velocity
    double us[3];     // fluid velocity seen
    int tri, tri0, ltri, ll, ll0;
    int pidx = 0, pstep = 0;   // caller's particle index and step (stranding records)
    const Zig32* z32 = nullptr;   // FP32 tables (mixed LSM2/LSM3 direct integrators)
    uint32_t err;
    bool deleted;
    bool defer;       // in: 2D final localization may be deferred to the walk queue
    bool deferred;    // out: the particle left its start triangle, queue it

    __device__ Particle(const DevMesh& m_, const DevFields<FT>& f_, const DevParams& p_,
                        const ZigTables& z_)
        : m(m_), f(f_), p(p_), z(z_), err(0), deleted(false), defer(false), deferred(false) {}

    // ---- field interpolation -------------------------------------------------
    // eulerian_field_set.pyx:1057-1115 (2D) and 1289-1394 (3D, zlocalize=0)
    __device__ void velocity(int k, int l, double px, double py, double pz, double& ux,
                             double& uy, double& uz) {
        P1 q = p1_at(m, k, px, py);
        velocity_q(q, l, pz, ux, uy, uz);
    }

    __device__ void velocity_q(const P1& q, int l, double pz, double& ux, double& uy,
                               double& uz) {
        using S = Slots<DIM>;
        if (DIM == 2) {
            ux = p1_eval<DIM>(f.cur, 0, q, S::UX);
            uy = p1_eval<DIM>(f.cur, 0, q, S::UY);
            uz = 0.;
        } else if (f.dim == 2) {
            // 3D particle on 2D fields: depth-averaged velocity with the
            // pseudo-3D corrections (update_state_lsm1.pyx:144-163)
            ux = p1_eval<DIM>(f.cur, 0, q, S::UX);
            uy = p1_eval<DIM>(f.cur, 0, q, S::UY);
            uz = 0.;
            double w, hor;
            pseudo_3d_corrections(q, pz, ux, uy, w, hor);
            uz += w;
            ux *= hor;
            uy *= hor;
        } else {
            if (l == PART_LOC_B || l == PART_LOC_A) { err |= ERR_INTERP_OUTSIDE; ux = uy = uz = 0.; return; }
            l = (int)CG_IDX(m, l, f.nlayers - 1);
        int jl = l * f.npoints, ju = (l + 1) * f.npoints;
            double zlp = p1_eval<DIM>(f.cur, jl, q, S::ZS);
            double zup = p1_eval<DIM>(f.cur, ju, q, S::ZS);
            double dz = zlp - zup;
            if (fabs(dz) < EPSILON) { err |= ERR_DEGENERATE_LAYER; ux = uy = uz = 0.; return; }
            double zf0 = (pz - zup) / dz;
            double zf1 = (zlp - pz) / dz;
            ux = zf0 * p1_eval<DIM>(f.cur, jl, q, S::UX) + zf1 * p1_eval<DIM>(f.cur, ju, q, S::UX);
            uy = zf0 * p1_eval<DIM>(f.cur, jl, q, S::UY) + zf1 * p1_eval<DIM>(f.cur, ju, q, S::UY);
            uz = zf0 * p1_eval<DIM>(f.cur, jl, q, Slots<3>::UZ) +
                 zf1 * p1_eval<DIM>(f.cur, ju, q, Slots<3>::UZ);
        }
    }

    // eulerian_field_set.pyx:1957-1993: friction coefficient of the depth h
    __device__ double friction_calc(double h) {
        const double fc = p.friction_coef;
        if (p.friction_model == 0) return 2. * GRAV / (fc * fc);   // Chezy
        if (p.friction_model == 1)                                  // Strickler
            return 2. * GRAV / (fc * fc) / cpow_re(fmax(EPSILON, h), 1. / 3.);
        if (p.friction_model == 2)                                  // Manning
            return 2. * GRAV * (fc * fc) / cpow_re(fmax(EPSILON, h), 1. / 3.);
        double aux = h * 11.036 / fc;                               // Nikuradse
        if (!(aux > 1.001)) aux = 1.001;
        const double r = log(aux) / KAPPA;
        return 2. / (r * r);
    }

    // eulerian_field_set.pyx:1887-1955 (with 1581-1642 for dzs/dt): the
    // vertical velocity w that keeps the relative elevation of a particle
    // advected by the log-law velocity, and the log-law factor of the
    // depth-averaged velocity at height pz (3D particle, 2D fields)
    __device__ void pseudo_3d_corrections(const P1& q, double pz, double ux, double uy,
                                          double& w, double& hor) {
        using S = Slots<3>;
        const double zs = p1_eval<DIM>(f.cur, 0, q, S::ZS);
        const double zb = p1_eval<DIM>(f.cur, 0, q, S::ZB);
        const double h = fmax(EPSILON, zs - zb);
        const double sigma = fmin(1., fmax(0., (pz - zb) / h));
        const double Cf = friction_calc(h);
        const double z0 = fmax(EPSILON, h * exp(-(1. + KAPPA / sqrt(Cf / 2.))));
        hor = (pz - zb <= z0) ? 0.0 : log((pz - zb) / z0) / (log(h / z0) - 1.);
        const double uc = ux * hor, vc = uy * hor;
        const double dzsdx = p1_gx<DIM>(f.cur, 0, q, S::ZS), dzsdy = p1_gy<DIM>(f.cur, 0, q, S::ZS);
        const double dzbdx = p1_gx<DIM>(f.cur, 0, q, S::ZB), dzbdy = p1_gy<DIM>(f.cur, 0, q, S::ZB);
        // frozen fields or the first interpolation: no previous surface
        double dzsdt = 0.;
        if (f.prev_valid) dzsdt = (zs - p1_eval<DIM>(f.prev, 0, q, S::ZS)) / p.dt;
        w = (1. - sigma) * (uc * dzbdx + vc * dzbdy) + sigma * (dzsdt + uc * dzsdx + vc * dzsdy);
    }

    // eulerian_field_set.pyx:1117-1182; 2D fields (pseudo-3D): the bed is
    // the BOTTOM field and the point is in layer 0 unless outside the column
    __device__ int z_localize(int k, double px, double py, double pz) {
        if (k == -1) return PART_LOC_O;
        P1 q = p1_at(m, k, px, py);
        int nl = f.nlayers;
        double zbp, zsp;
        int l;
        if (DIM == 3 && f.dim == 2) {
            zbp = p1_eval<DIM>(f.cur, 0, q, Slots<3>::ZB);
            zsp = p1_eval<DIM>(f.cur, 0, q, Slots<DIM>::ZS);
            l = 0;
        } else {
            zbp = p1_eval<DIM>(f.cur, 0, q, Slots<DIM>::ZS);
            zsp = p1_eval<DIM>(f.cur, (nl - 1) * f.npoints, q, Slots<DIM>::ZS);
            l = lower_layer_index(nl, zsp, zbp, pz);
        }
        if (pz < zbp) l = PART_LOC_B;
        else if (pz > zsp) l = PART_LOC_A;
        return l;
    }

    // eulerian_field_set.pyx:994-1055 (zs at layer l)
    __device__ double zs_at(int k, int l, double px, double py) {
        P1 q = p1_at(m, k, px, py);
        return p1_eval<DIM>(f.cur, l * f.npoints, q, Slots<DIM>::ZS);
    }

    // bed elevation: the bottom layer's elevation, or on 2D fields the
    // BOTTOM field (solver.pyx:284-297)
    __device__ double zb_at(int k, double px, double py) {
        if (DIM == 3 && f.dim == 2) {
            P1 q = p1_at(m, k, px, py);
            return p1_eval<DIM>(f.cur, 0, q, Slots<3>::ZB);
        }
        return zs_at(k, 0, px, py);
    }

    // eulerian_field_set.pyx:1644-1763
    __device__ void diffusivity_q(const P1& q, int l, double pz, double& K, double& dKdx,
                                  double& dKdy, double& dKdz) {
        using S = Slots<DIM>;
        if (DIM == 2 || f.dim == 2) {
            double kn0 = nodev<DIM>(f.cur, q.i0, S::K), kn1 = nodev<DIM>(f.cur, q.i1, S::K),
                   kn2 = nodev<DIM>(f.cur, q.i2, S::K);
            double Kp = kn0 * q.f0 + kn1 * q.f1 + kn2 * q.f2;
            dKdx = kn0 * q.gx0 + kn1 * q.gx1 + kn2 * q.gx2;
            dKdy = kn0 * q.gy0 + kn1 * q.gy1 + kn2 * q.gy2;
            dKdz = 0.;
            K = fmax(0., Kp);
            return;
        }
        if (l == PART_LOC_B || l == PART_LOC_A) { err |= ERR_INTERP_OUTSIDE; K = dKdx = dKdy = dKdz = 0.; return; }
        l = (int)CG_IDX(m, l, f.nlayers - 1);
        int jl = l * f.npoints, ju = (l + 1) * f.npoints;
        double Kl = p1_eval<DIM>(f.cur, jl, q, S::K);
        double gxl = p1_gx<DIM>(f.cur, jl, q, S::K);
        double gyl = p1_gy<DIM>(f.cur, jl, q, S::K);
        double zlp = p1_eval<DIM>(f.cur, jl, q, S::ZS);
        double zlx = p1_gx<DIM>(f.cur, jl, q, S::ZS);
        double zly = p1_gy<DIM>(f.cur, jl, q, S::ZS);
        double Ku = p1_eval<DIM>(f.cur, ju, q, S::K);
        double gxu = p1_gx<DIM>(f.cur, ju, q, S::K);
        double gyu = p1_gy<DIM>(f.cur, ju, q, S::K);
        double zup = p1_eval<DIM>(f.cur, ju, q, S::ZS);
        double zux = p1_gx<DIM>(f.cur, ju, q, S::ZS);
        double zuy = p1_gy<DIM>(f.cur, ju, q, S::ZS);
        double dz = zup - zlp;
        if (fabs(dz) < EPSILON) { err |= ERR_DEGENERATE_LAYER; K = dKdx = dKdy = dKdz = 0.; return; }
        double s = (pz - zlp) / dz;
        double Kp = (1. - s) * Kl + s * Ku;
        dKdz = (Ku - Kl) / dz;
        dKdx = (1. - s) * gxl + s * gxu - dKdz * ((1. - s) * zlx + s * zux);
        dKdy = (1. - s) * gyl + s * gyu - dKdz * ((1. - s) * zly + s * zuy);
        K = fmax(0., Kp);
    }

    // lagrangian_particle_set.pyx:834-890 (model_hr = 0)
    __device__ double buoyancy_velocity(double dp) {
        if (p.buoy_model == 0) return p.buoy_wb;
        double s = p.density / p.rho0, wb;
        if (dp < 1.e-4) {
            wb = fabs(s - 1.) * (GRAV * (dp * dp)) / (18. * NU0);
        } else if (dp > 1.e-3) {
            wb = sqrt(fabs(s - 1.) * (4. * dp * GRAV) / (3. * p.drag_coef));
        } else {
            wb = (10. * NU0 / dp) * (sqrt(1. + fabs(s - 1.) * GRAV * pow(dp, 3.0) / (100. * (NU0 * NU0))) - 1.);
        }
        if (s > 1.) wb *= -1.;
        return wb;
    }

    // ---- fields of the LSM2/LSM3 updates -----------------------------------------
    // turbulent energy and dissipation: 2D P1 (eulerian_field_set.pyx:994-1055),
    // 3D prism with the layer given (1184-1287)
    __device__ void turb_q(const P1& q, int l, double pz, double& kt, double& ep) {
        const FT* t = f.turb;
        if (DIM == 2) {
            kt = (double)t[2 * q.i0] * q.f0 + (double)t[2 * q.i1] * q.f1 + (double)t[2 * q.i2] * q.f2;
            ep = (double)t[2 * q.i0 + 1] * q.f0 + (double)t[2 * q.i1 + 1] * q.f1 +
                 (double)t[2 * q.i2 + 1] * q.f2;
            return;
        }
        if (l == PART_LOC_B || l == PART_LOC_A) { err |= ERR_INTERP_OUTSIDE; kt = ep = 0.; return; }
        l = (int)CG_IDX(m, l, f.nlayers - 1);
        int jl = l * f.npoints, ju = (l + 1) * f.npoints;
        double zlp = p1_eval<DIM>(f.cur, jl, q, Slots<DIM>::ZS);
        double zup = p1_eval<DIM>(f.cur, ju, q, Slots<DIM>::ZS);
        double dz = zlp - zup;
        if (fabs(dz) < EPSILON) { err |= ERR_DEGENERATE_LAYER; kt = ep = 0.; return; }
        double zf0 = (pz - zup) / dz;
        double zf1 = (zlp - pz) / dz;
        const FT* tl = t + 2 * (size_t)jl;
        const FT* tu = t + 2 * (size_t)ju;
        double ktl = (double)tl[2 * q.i0] * q.f0 + (double)tl[2 * q.i1] * q.f1 + (double)tl[2 * q.i2] * q.f2;
        double ktu = (double)tu[2 * q.i0] * q.f0 + (double)tu[2 * q.i1] * q.f1 + (double)tu[2 * q.i2] * q.f2;
        double epl = (double)tl[2 * q.i0 + 1] * q.f0 + (double)tl[2 * q.i1 + 1] * q.f1 +
                     (double)tl[2 * q.i2 + 1] * q.f2;
        double epu = (double)tu[2 * q.i0 + 1] * q.f0 + (double)tu[2 * q.i1 + 1] * q.f1 +
                     (double)tu[2 * q.i2 + 1] * q.f2;
        kt = zf0 * ktl + zf1 * ktu;
        ep = zf0 * epl + zf1 * epu;
    }

    // value and gradient of a nodal prism field (eulerian_field_set.pyx:1999-2023)
    __device__ void prism_vg(const FT* fld, int jl, int ju, int slot, const P1& q, double s_,
                             double dz, double zlx, double zly, double zux, double zuy,
                             double& val, double& ddx, double& ddy, double& ddz) {
        double a0 = nodev<DIM>(fld, jl + q.i0, slot), a1 = nodev<DIM>(fld, jl + q.i1, slot),
               a2 = nodev<DIM>(fld, jl + q.i2, slot);
        double b0 = nodev<DIM>(fld, ju + q.i0, slot), b1 = nodev<DIM>(fld, ju + q.i1, slot),
               b2 = nodev<DIM>(fld, ju + q.i2, slot);
        double fl = a0 * q.f0 + a1 * q.f1 + a2 * q.f2;
        double fu = b0 * q.f0 + b1 * q.f1 + b2 * q.f2;
        double gxl = a0 * q.gx0 + a1 * q.gx1 + a2 * q.gx2;
        double gyl = a0 * q.gy0 + a1 * q.gy1 + a2 * q.gy2;
        double gxu = b0 * q.gx0 + b1 * q.gx1 + b2 * q.gx2;
        double gyu = b0 * q.gy0 + b1 * q.gy1 + b2 * q.gy2;
        double dfdz = (fu - fl) / dz;
        val = (1. - s_) * fl + s_ * fu;
        ddx = (1. - s_) * gxl + s_ * gxu - dfdz * ((1. - s_) * zlx + s_ * zux);
        ddy = (1. - s_) * gyl + s_ * gyu - dfdz * ((1. - s_) * zly + s_ * zuy);
        ddz = dfdz;
    }

    // dU/dt along a path, Ua = (ua, va, wa): eulerian_field_set.pyx:1396-1454
    // (2D) and 1456-1579 (3D); the Eulerian time derivative from the previous
    // interpolation when it is valid (never for frozen fields)
    __device__ void accel(int k, int l, double px, double py, double pz, double ua, double va,
                          double wa, double& ax, double& ay, double& az) {
        P1 q = p1_at(m, k, px, py);
        double dt = p.dt;
        if (DIM == 2) {
            using S = Slots<2>;
            double u0 = nodev<DIM>(f.cur, q.i0, S::UX), u1 = nodev<DIM>(f.cur, q.i1, S::UX),
                   u2 = nodev<DIM>(f.cur, q.i2, S::UX);
            double v0 = nodev<DIM>(f.cur, q.i0, S::UY), v1 = nodev<DIM>(f.cur, q.i1, S::UY),
                   v2 = nodev<DIM>(f.cur, q.i2, S::UY);
            double dudx = u0 * q.gx0 + u1 * q.gx1 + u2 * q.gx2;
            double dudy = u0 * q.gy0 + u1 * q.gy1 + u2 * q.gy2;
            double dvdx = v0 * q.gx0 + v1 * q.gx1 + v2 * q.gx2;
            double dvdy = v0 * q.gy0 + v1 * q.gy1 + v2 * q.gy2;
            double dudt = 0., dvdt = 0.;
            if (f.prev_valid) {
                double pu0 = nodev<DIM>(f.prev, q.i0, S::UX), pu1 = nodev<DIM>(f.prev, q.i1, S::UX),
                       pu2 = nodev<DIM>(f.prev, q.i2, S::UX);
                double pv0 = nodev<DIM>(f.prev, q.i0, S::UY), pv1 = nodev<DIM>(f.prev, q.i1, S::UY),
                       pv2 = nodev<DIM>(f.prev, q.i2, S::UY);
                dudt = ((u0 - pu0) * q.f0 + (u1 - pu1) * q.f1 + (u2 - pu2) * q.f2) / dt;
                dvdt = ((v0 - pv0) * q.f0 + (v1 - pv1) * q.f1 + (v2 - pv2) * q.f2) / dt;
            }
            ax = dudt + ua * dudx + va * dudy;
            ay = dvdt + ua * dvdx + va * dvdy;
            az = 0.;
            return;
        }
        using S = Slots<3>;
        if (l == PART_LOC_B || l == PART_LOC_A) { err |= ERR_INTERP_OUTSIDE; ax = ay = az = 0.; return; }
        l = (int)CG_IDX(m, l, f.nlayers - 1);
        int jl = l * f.npoints, ju = (l + 1) * f.npoints;
        double e0 = nodev<DIM>(f.cur, jl + q.i0, S::ZS), e1 = nodev<DIM>(f.cur, jl + q.i1, S::ZS),
               e2 = nodev<DIM>(f.cur, jl + q.i2, S::ZS);
        double h0 = nodev<DIM>(f.cur, ju + q.i0, S::ZS), h1 = nodev<DIM>(f.cur, ju + q.i1, S::ZS),
               h2 = nodev<DIM>(f.cur, ju + q.i2, S::ZS);
        double zlp = e0 * q.f0 + e1 * q.f1 + e2 * q.f2;
        double zup = h0 * q.f0 + h1 * q.f1 + h2 * q.f2;
        double dz = zup - zlp;
        if (fabs(dz) < EPSILON) { err |= ERR_DEGENERATE_LAYER; ax = ay = az = 0.; return; }
        double s_ = (pz - zlp) / dz;
        double zlx = e0 * q.gx0 + e1 * q.gx1 + e2 * q.gx2;
        double zly = e0 * q.gy0 + e1 * q.gy1 + e2 * q.gy2;
        double zux = h0 * q.gx0 + h1 * q.gx1 + h2 * q.gx2;
        double zuy = h0 * q.gy0 + h1 * q.gy1 + h2 * q.gy2;
        double un, dudx, dudy, dudz, vn, dvdx, dvdy, dvdz, wn, dwdx, dwdy, dwdz, t0, t1, t2, t3;
        prism_vg(f.cur, jl, ju, S::UX, q, s_, dz, zlx, zly, zux, zuy, un, dudx, dudy, dudz);
        prism_vg(f.cur, jl, ju, S::UY, q, s_, dz, zlx, zly, zux, zuy, vn, dvdx, dvdy, dvdz);
        prism_vg(f.cur, jl, ju, S::UZ, q, s_, dz, zlx, zly, zux, zuy, wn, dwdx, dwdy, dwdz);
        double dudt = 0., dvdt = 0., dwdt = 0.;
        if (f.prev_valid) {
            prism_vg(f.prev, jl, ju, S::UX, q, s_, dz, zlx, zly, zux, zuy, t0, t1, t2, t3);
            dudt = (un - t0) / dt;
            prism_vg(f.prev, jl, ju, S::UY, q, s_, dz, zlx, zly, zux, zuy, t0, t1, t2, t3);
            dvdt = (vn - t0) / dt;
            prism_vg(f.prev, jl, ju, S::UZ, q, s_, dz, zlx, zly, zux, zuy, t0, t1, t2, t3);
            dwdt = (wn - t0) / dt;
        }
        ax = dudt + ua * dudx + va * dudy + wa * dudz;
        ay = dvdt + ua * dvdx + va * dvdy + wa * dvdz;
        az = dwdt + ua * dwdx + va * dwdy + wa * dwdz;
    }

    // ---- FP32 field access of the mixed LSM2/LSM3 form ------------------------------
    // P1 weights from the FP32 offset to the triangle's anchor vertex and the
    // FP32 gradients of its packed record (no FP64 arithmetic).
    struct P1f {
        int i0, i1, i2;
        float f0, f1, f2, gx0, gx1, gx2, gy0, gy1, gy2;
    };
    __device__ P1f p1f_at(int k, double px, double py) const {
        Tri32 t = load_tri32(m, k);
        return p1f_of(t, bary32(t, px, py));
    }
    template <typename T>   // Tri32 or Tri32S (the same vertex ids and gradients)
    __device__ P1f p1f_of(const T& t, const Bary& b) const {
        P1f r;
        r.i0 = t.tv.x; r.i1 = t.tv.y; r.i2 = t.tv.z;
        r.f0 = b.l0; r.f1 = b.l1; r.f2 = b.l2;
        r.gx0 = t.g0.x; r.gx1 = t.g0.y; r.gx2 = t.g0.z;
        r.gy0 = t.g0.w; r.gy1 = t.g1.x; r.gy2 = t.g1.y;
        return r;
    }
    __device__ float nf(const FT* fld, int node, int slot) const {
        return (float)fld[(size_t)node * Slots<DIM>::NF + slot];
    }
    __device__ float ev(const FT* fld, int off, const P1f& q, int slot) const {
        return nf(fld, off + q.i0, slot) * q.f0 + nf(fld, off + q.i1, slot) * q.f1 +
               nf(fld, off + q.i2, slot) * q.f2;
    }
    // 2D / prism velocity (eulerian_field_set.pyx:1057-1115, 1289-1394)
    __device__ void velocity32(const P1f& q, int l, float pz, float& ux, float& uy, float& uz) {
        using S = Slots<DIM>;
        if (DIM == 2) {
            ux = ev(f.cur, 0, q, S::UX);
            uy = ev(f.cur, 0, q, S::UY);
            uz = 0.f;
            return;
        }
        if (l == PART_LOC_B || l == PART_LOC_A) { err |= ERR_INTERP_OUTSIDE; ux = uy = uz = 0.f; return; }
        l = (int)CG_IDX(m, l, f.nlayers - 1);
        int jl = l * f.npoints, ju = (l + 1) * f.npoints;
        float zlp = ev(f.cur, jl, q, S::ZS), zup = ev(f.cur, ju, q, S::ZS);
        float dz = zlp - zup;
        if (!(fabsf(dz) >= (float)EPSILON)) { err |= ERR_DEGENERATE_LAYER; ux = uy = uz = 0.f; return; }
        float zf0 = (pz - zup) / dz, zf1 = (zlp - pz) / dz;
        ux = zf0 * ev(f.cur, jl, q, S::UX) + zf1 * ev(f.cur, ju, q, S::UX);
        uy = zf0 * ev(f.cur, jl, q, S::UY) + zf1 * ev(f.cur, ju, q, S::UY);
        uz = zf0 * ev(f.cur, jl, q, Slots<3>::UZ) + zf1 * ev(f.cur, ju, q, Slots<3>::UZ);
    }
    // k and eps (2D P1, 3D prism)
    __device__ void turb32(const P1f& q, int l, float pz, float& kt, float& ep) {
        const FT* t = f.turb;
        auto tv = [&](int off, int c) {
            return (float)t[2 * (size_t)(off + q.i0) + c] * q.f0 +
                   (float)t[2 * (size_t)(off + q.i1) + c] * q.f1 +
                   (float)t[2 * (size_t)(off + q.i2) + c] * q.f2;
        };
        if (DIM == 2) {
            kt = tv(0, 0);
            ep = tv(0, 1);
            return;
        }
        if (l == PART_LOC_B || l == PART_LOC_A) { err |= ERR_INTERP_OUTSIDE; kt = ep = 0.f; return; }
        l = (int)CG_IDX(m, l, f.nlayers - 1);
        int jl = l * f.npoints, ju = (l + 1) * f.npoints;
        float zlp = ev(f.cur, jl, q, Slots<DIM>::ZS), zup = ev(f.cur, ju, q, Slots<DIM>::ZS);
        float dz = zlp - zup;
        if (!(fabsf(dz) >= (float)EPSILON)) { err |= ERR_DEGENERATE_LAYER; kt = ep = 0.f; return; }
        float zf0 = (pz - zup) / dz, zf1 = (zlp - pz) / dz;
        kt = zf0 * tv(jl, 0) + zf1 * tv(ju, 0);
        ep = zf0 * tv(jl, 1) + zf1 * tv(ju, 1);
    }
    __device__ void prism_vg32(const FT* fld, int jl, int ju, int slot, const P1f& q, float s_,
                               float dz, float zlx, float zly, float zux, float zuy, float& val,
                               float& ddx, float& ddy, float& ddz) {
        float a0 = nf(fld, jl + q.i0, slot), a1 = nf(fld, jl + q.i1, slot), a2 = nf(fld, jl + q.i2, slot);
        float b0 = nf(fld, ju + q.i0, slot), b1 = nf(fld, ju + q.i1, slot), b2 = nf(fld, ju + q.i2, slot);
        float fl = a0 * q.f0 + a1 * q.f1 + a2 * q.f2;
        float fu = b0 * q.f0 + b1 * q.f1 + b2 * q.f2;
        float gxl = a0 * q.gx0 + a1 * q.gx1 + a2 * q.gx2, gyl = a0 * q.gy0 + a1 * q.gy1 + a2 * q.gy2;
        float gxu = b0 * q.gx0 + b1 * q.gx1 + b2 * q.gx2, gyu = b0 * q.gy0 + b1 * q.gy1 + b2 * q.gy2;
        float dfdz = (fu - fl) / dz;
        val = (1.f - s_) * fl + s_ * fu;
        ddx = (1.f - s_) * gxl + s_ * gxu - dfdz * ((1.f - s_) * zlx + s_ * zux);
        ddy = (1.f - s_) * gyl + s_ * gyu - dfdz * ((1.f - s_) * zly + s_ * zuy);
        ddz = dfdz;
    }
    // dU/dt along a path (eulerian_field_set.pyx:1396-1579) in FP32
    __device__ void accel32(const P1f& q, int l, float pz, float ua, float va, float wa,
                            float& ax, float& ay, float& az) {
        const float dt = (float)p.dt;
        if (DIM == 2) {
            using S = Slots<2>;
            float u0 = nf(f.cur, q.i0, S::UX), u1 = nf(f.cur, q.i1, S::UX), u2 = nf(f.cur, q.i2, S::UX);
            float v0 = nf(f.cur, q.i0, S::UY), v1 = nf(f.cur, q.i1, S::UY), v2 = nf(f.cur, q.i2, S::UY);
            float dudx = u0 * q.gx0 + u1 * q.gx1 + u2 * q.gx2, dudy = u0 * q.gy0 + u1 * q.gy1 + u2 * q.gy2;
            float dvdx = v0 * q.gx0 + v1 * q.gx1 + v2 * q.gx2, dvdy = v0 * q.gy0 + v1 * q.gy1 + v2 * q.gy2;
            float dudt = 0.f, dvdt = 0.f;
            if (f.prev_valid) {
                dudt = ((u0 - nf(f.prev, q.i0, S::UX)) * q.f0 + (u1 - nf(f.prev, q.i1, S::UX)) * q.f1 +
                        (u2 - nf(f.prev, q.i2, S::UX)) * q.f2) / dt;
                dvdt = ((v0 - nf(f.prev, q.i0, S::UY)) * q.f0 + (v1 - nf(f.prev, q.i1, S::UY)) * q.f1 +
                        (v2 - nf(f.prev, q.i2, S::UY)) * q.f2) / dt;
            }
            ax = dudt + ua * dudx + va * dudy;
            ay = dvdt + ua * dvdx + va * dvdy;
            az = 0.f;
            return;
        }
        using S = Slots<3>;
        if (l == PART_LOC_B || l == PART_LOC_A) { err |= ERR_INTERP_OUTSIDE; ax = ay = az = 0.f; return; }
        l = (int)CG_IDX(m, l, f.nlayers - 1);
        int jl = l * f.npoints, ju = (l + 1) * f.npoints;
        float e0 = nf(f.cur, jl + q.i0, S::ZS), e1 = nf(f.cur, jl + q.i1, S::ZS), e2 = nf(f.cur, jl + q.i2, S::ZS);
        float h0 = nf(f.cur, ju + q.i0, S::ZS), h1 = nf(f.cur, ju + q.i1, S::ZS), h2 = nf(f.cur, ju + q.i2, S::ZS);
        float zlp = e0 * q.f0 + e1 * q.f1 + e2 * q.f2, zup = h0 * q.f0 + h1 * q.f1 + h2 * q.f2;
        float dz = zup - zlp;
        if (!(fabsf(dz) >= (float)EPSILON)) { err |= ERR_DEGENERATE_LAYER; ax = ay = az = 0.f; return; }
        float s_ = (pz - zlp) / dz;
        float zlx = e0 * q.gx0 + e1 * q.gx1 + e2 * q.gx2, zly = e0 * q.gy0 + e1 * q.gy1 + e2 * q.gy2;
        float zux = h0 * q.gx0 + h1 * q.gx1 + h2 * q.gx2, zuy = h0 * q.gy0 + h1 * q.gy1 + h2 * q.gy2;
        float un, dudx, dudy, dudz, vn, dvdx, dvdy, dvdz, wn, dwdx, dwdy, dwdz, t0, t1, t2, t3;
        prism_vg32(f.cur, jl, ju, S::UX, q, s_, dz, zlx, zly, zux, zuy, un, dudx, dudy, dudz);
        prism_vg32(f.cur, jl, ju, S::UY, q, s_, dz, zlx, zly, zux, zuy, vn, dvdx, dvdy, dvdz);
        prism_vg32(f.cur, jl, ju, S::UZ, q, s_, dz, zlx, zly, zux, zuy, wn, dwdx, dwdy, dwdz);
        float dudt = 0.f, dvdt = 0.f, dwdt = 0.f;
        if (f.prev_valid) {
            prism_vg32(f.prev, jl, ju, S::UX, q, s_, dz, zlx, zly, zux, zuy, t0, t1, t2, t3);
            dudt = (un - t0) / dt;
            prism_vg32(f.prev, jl, ju, S::UY, q, s_, dz, zlx, zly, zux, zuy, t0, t1, t2, t3);
            dvdt = (vn - t0) / dt;
            prism_vg32(f.prev, jl, ju, S::UZ, q, s_, dz, zlx, zly, zux, zuy, t0, t1, t2, t3);
            dwdt = (wn - t0) / dt;
        }
        ax = dudt + ua * dudx + va * dudy + wa * dudz;
        ay = dvdt + ua * dvdx + va * dvdy + wa * dvdz;
        az = dwdt + ua * dwdx + va * dwdy + wa * dwdz;
    }
    // layer of (px, py, pz) in element k from FP32 bed/surface elevations
    // (eulerian_field_set.pyx:1117-1182)
    __device__ int z_localize32(int k, double px, double py, double pz) {
        if (k == -1) return PART_LOC_O;
        return z_localize32_q(p1f_at(k, px, py), (float)pz);
    }
    __device__ int z_localize32_q(const P1f& q, float z) {
        int nl = f.nlayers;
        float zbp = ev(f.cur, 0, q, Slots<DIM>::ZS);
        float zsp = ev(f.cur, (nl - 1) * f.npoints, q, Slots<DIM>::ZS);
        int l = 0;
        if (nl > 1) {
            float hl = (zsp - zbp) / (float)(nl - 1);
            if (hl > 0.f) {
                float fi = floorf((z - zbp) / hl);
                l = !(fi >= 0.f) ? 0 : (!(fi <= (float)(nl - 2)) ? nl - 2 : (int)fi);
            }
        }
        if (z < zbp) l = PART_LOC_B;
        else if (z > zsp) l = PART_LOC_A;
        return l;
    }

    // ---- LSM1 (cylag/lsm/update_state_lsm1.pyx) ----------------------------------
    __device__ void set_up_us(double ux, double uy, double uz) {
        up[0] = ux; up[1] = uy; us[0] = ux; us[1] = uy;
        if (DIM == 3) { up[2] = uz; us[2] = uz; }
    }

    // update_state_lsm1.pyx:228-248; true when the scheme stops at this stage
    __device__ bool stage_locate(double xt, double yt, double zt, int& tt, int& tl, int& bnd) {
        ltri = tri;
        xy_localize(m, ltri, x0[0], x0[1], xt, yt, tt, bnd);
        tl = 0;
        if (DIM == 3) tl = z_localize(tt, xt, yt, zt);
        if (bnd != -1 || (DIM == 3 && (tl == -2 || tl == -3))) {
            tri = tt;
            if (DIM == 3) ll = tl;
            x[0] += up[0] * p.dt;
            x[1] += up[1] * p.dt;
            if (DIM == 3) x[2] += up[2] * p.dt;
            return true;
        }
        // outside the mesh with no boundary crossing found: the reference
        // raises at the next interpolation; flag it and stop the step
        if (tt < 0) { err |= ERR_INTERP_OUTSIDE; tri = tt; return true; }
        return false;
    }

    // update_state_lsm1.pyx:135-656; q0: P1 factors at the step-start point
    __device__ int advect_lsm1(const P1& q0) {
        double dt = p.dt, ux, uy, uz;
        velocity_q(q0, ll, DIM == 3 ? x[2] : 0., ux, uy, uz);
        set_up_us(ux, uy, uz);
        if (p.time_scheme == 1) {  // 135-177
            x[0] += ux * dt;
            x[1] += uy * dt;
            if (DIM == 3) x[2] += uz * dt;
            return -1;
        }
        int tt, tl, bnd;
        double xt, yt, zt = 0.;
        if (p.time_scheme == 2) {  // 179-274
            xt = x[0] + 0.5 * ux * dt;
            yt = x[1] + 0.5 * uy * dt;
            if (DIM == 3) zt = x[2] + 0.5 * uz * dt;
            if (stage_locate(xt, yt, zt, tt, tl, bnd)) return bnd;
            velocity(tt, tl, xt, yt, zt, ux, uy, uz);
            x[0] += ux * dt;
            x[1] += uy * dt;
            if (DIM == 3) x[2] += uz * dt;
            return -1;
        }
        double k1x = ux * dt, k1y = uy * dt, k1z = DIM == 3 ? uz * dt : 0.;
        if (p.time_scheme == 3) {  // 276-432
            xt = x[0] + (1. / 3.) * k1x;
            yt = x[1] + (1. / 3.) * k1y;
            zt = DIM == 3 ? x[2] + (1. / 3.) * k1z : 0.;
            if (stage_locate(xt, yt, zt, tt, tl, bnd)) return bnd;
            velocity(tt, tl, xt, yt, zt, ux, uy, uz);
            double k2x = ux * dt, k2y = uy * dt, k2z = DIM == 3 ? uz * dt : 0.;
            xt = x[0] + (2. / 3.) * k2x;
            yt = x[1] + (2. / 3.) * k2y;
            zt = DIM == 3 ? x[2] + (2. / 3.) * k2z : 0.;
            if (stage_locate(xt, yt, zt, tt, tl, bnd)) return bnd;
            velocity(tt, tl, xt, yt, zt, ux, uy, uz);
            double k3x = ux * dt, k3y = uy * dt, k3z = DIM == 3 ? uz * dt : 0.;
            x[0] += (0.25 * k1x + 0.75 * k3x);
            x[1] += (0.25 * k1y + 0.75 * k3y);
            if (DIM == 3) x[2] += (0.25 * k1z + 0.75 * k3z);
            return -1;
        }
        // time_scheme 4, 434-656
        xt = x[0] + 0.5 * k1x;
        yt = x[1] + 0.5 * k1y;
        zt = DIM == 3 ? x[2] + 0.5 * k1z : 0.;
        if (stage_locate(xt, yt, zt, tt, tl, bnd)) return bnd;
        velocity(tt, tl, xt, yt, zt, ux, uy, uz);
        double k2x = ux * dt, k2y = uy * dt, k2z = DIM == 3 ? uz * dt : 0.;
        xt = x[0] + 0.5 * k2x;
        yt = x[1] + 0.5 * k2y;
        zt = DIM == 3 ? x[2] + 0.5 * k2z : 0.;
        if (stage_locate(xt, yt, zt, tt, tl, bnd)) return bnd;
        velocity(tt, tl, xt, yt, zt, ux, uy, uz);
        double k3x = ux * dt, k3y = uy * dt, k3z = DIM == 3 ? uz * dt : 0.;
        xt = x[0] + k3x;
        yt = x[1] + k3y;
        zt = DIM == 3 ? x[2] + k3z : 0.;
        if (stage_locate(xt, yt, zt, tt, tl, bnd)) return bnd;
        velocity(tt, tl, xt, yt, zt, ux, uy, uz);
        double k4x = ux * dt, k4y = uy * dt, k4z = DIM == 3 ? uz * dt : 0.;
        x[0] += (k1x + 2. * k2x + 2. * k3x + k4x) / 6.;
        x[1] += (k1y + 2. * k2y + 2. * k3y + k4y) / 6.;
        if (DIM == 3) x[2] += (k1z + 2. * k2z + 2. * k3z + k4z) / 6.;
        return -1;
    }

    // update_state_lsm1.pyx:658-726 (K at the start point, same factors q0)
    __device__ void diffusion_lsm1(const P1& q0) {
        double dt = p.dt;
        double xix = 0., xiy = 0., xiz = 0.;
        double diffx, diffy, diffz = 0.;
        double driftx = 0., drifty = 0., driftz = 0.;
        if (p.diffmod == 2 || p.diffmod == 3) {
            double Kp, dKdx, dKdy, dKdz;
            diffusivity_q(q0, ll0, DIM == 3 ? x0[2] : 0., Kp, dKdx, dKdy, dKdz);
            diffx = sqrt(2. * Kp) * p.sqrtdt;
            diffy = diffx;
            driftx = dKdx * dt;
            drifty = dKdy * dt;
            if (DIM == 3) {
                if (p.diffmod == 2) {
                    diffz = p.diffz_const;
                } else {
                    diffz = diffx;
                    driftz = dKdz * dt;
                }
            }
        } else {
            diffx = p.diffx_const;
            diffy = diffx;
            if (DIM == 3) diffz = p.diffz_const;
        }
        if (diffx != 0.) rng_pair(rng, p.rng_method, z, xix, xiy);
        if (DIM == 3 && diffz != 0.) xiz = rng_single(rng, p.rng_method, z);
        x[0] += driftx + diffx * xix;
        x[1] += drifty + diffy * xiy;
        if (DIM == 3) x[2] += driftz + diffz * xiz;
    }

    // update_state_lsm1.pyx:30-133
    __device__ int update_lsm1(double dp) {
        P1 q0 = p1_at(m, tri0, x0[0], x0[1]);
        int bnd_j = advect_lsm1(q0);
        if (p.diffmod != 0) diffusion_lsm1(q0);
        if (DIM == 3) {
            double wb = buoyancy_velocity(dp);
            x[2] += wb * p.dt;
            up[2] += wb;
        }
        if (bnd_j == -1) {
            ltri = tri;
            if (DIM == 2 && defer) {
                // xylocalizer.pyx:65-70 here, the path walk in walk_kernel
                if (!in_tri(m, ltri, x[0], x[1])) deferred = true;
                return -1;
            }
            xy_localize(m, ltri, x0[0], x0[1], x[0], x[1], tri, bnd_j);
            if (DIM == 3) ll = z_localize(tri, x[0], x[1], x[2]);
        }
        return bnd_j;
    }

    // end of the step (solver.pyx:505-524): state write-back; deletion per
    // lagrangian_particle_set.pyx:766-788, the tag recording the iteration
    // for the host-side retag (maxtag+1, ... in iteration then index order)
    // last_velocity (aux >= 2) is the velocity the state held at the step's
    // start, read here before the new one overwrites it
    __device__ void store(DevState& s, int i, int aux, int step_index) {
        const int D = DIM;
        const int a = aux_index(s, i);   // slot of the per-particle arrays outside the sort
        const int iv = widx(s, i, a, W_VEL), iu = widx(s, i, a, W_FVS | W_AUXW);
        const int il = widx(s, i, a, W_LAYER), id = widx(s, i, a, W_DIAM);
        const int ix = widx(s, i, a, W_AUXW);
        // the mixed LSM2/LSM3 form keeps its velocities as FP32 values,
        // whether the state is FP32 working copies or the caller's arrays
        const bool v32 = std::is_same<FT, float>::value && p.model >= 2;
        const bool two = (s.work & W_VEL2) != 0;   // (the write-back gives fvs, last_velocity)
        if (deleted) {
#pragma unroll
            for (int d = 0; d < D; ++d) {
                s.pos[(size_t)i * D + d] = 0.;
                vel_st(s, (size_t)iv * D + d, 0.);
                s.last_pos[(size_t)ix * D + d] = 0.;
                if (!two) {
                    fvs_st(s, (size_t)iu * D + d, 0.);
                    s.last_vel[(size_t)ix * D + d] = 0.;
                }
            }
            s.diameter[id] = 0.;
            if (s.depth) s.depth[a] = 0.;
            s.tri[i] = -1;
            s.last_tri[ix] = -1;
            s.lowerlayer[il] = 0;
            s.tag[i] = -2 - step_index;
            s.rng[i] = rng.state;
            return;
        }
        if (DIM == 2 && (s.work & W_SPLIT)) {
            reinterpret_cast<float4*>(s.pos)[i] = split_pos(x[0], x[1]);
        } else {
#pragma unroll
            for (int d = 0; d < D; ++d) s.pos[(size_t)i * D + d] = x[d];
        }
        s.tri[i] = tri;
        if (DIM == 3) s.lowerlayer[il] = ll;
        s.rng[i] = rng.state;
        double lastv[3] = {0., 0., 0.};
        if (aux >= 2 && !two) {
#pragma unroll
            for (int d = 0; d < D; ++d) {
                const double v = vel_ld(s, (size_t)iv * D + d);
                lastv[d] = v32 ? (double)(float)v : v;
            }
        }
        if (p.model >= 2 || aux >= 1) {
#pragma unroll
            for (int d = 0; d < D; ++d)
                vel_st(s, (size_t)iv * D + d, v32 ? (double)(float)up[d] : up[d]);
        }
        if ((p.model == 3 || aux >= 1) && !two) {
#pragma unroll
            for (int d = 0; d < D; ++d)
                fvs_st(s, (size_t)iu * D + d, v32 ? (double)(float)us[d] : us[d]);
        }
        if (aux >= 2) {
#pragma unroll
            for (int d = 0; d < D; ++d) {
                s.last_pos[(size_t)ix * D + d] = x0[d];
                if (!two) s.last_vel[(size_t)ix * D + d] = lastv[d];
            }
            s.last_tri[ix] = ltri;
        }
    }


    // ---- boundary conditions (compute_bc.pyx:35-395) ----------------------------
    // compute_bc.pyx:190-240 (normal2u utils.pyx:99-119)
    __device__ void reflect(double* v, double ex0, double ey0, double ex1, double ey1,
                            bool damp_vel) {
        double norm = sqrt((ex1 - ex0) * (ex1 - ex0) + (ey1 - ey0) * (ey1 - ey0));
        double nx = (ey0 - ey1) / norm;
        double ny = (ex1 - ex0) / norm;
        if (p.bc_type == 2 && p.roughness > 0.) {
            double max_theta = 85.0 * DEG_TO_RAD;
            double theta = rng_single(rng, p.rng_method, z) * p.roughness;
            theta = fmax(-max_theta, fmin(max_theta, theta));
            double ct = cos(theta), st = sin(theta);
            double nnx = nx * ct - ny * st;
            double nny = nx * st + ny * ct;
            nx = nnx; ny = nny;
        }
        double u0 = v[0];
        v[0] = u0 * nx + v[1] * ny;
        v[1] = -u0 * ny + v[1] * nx;
        v[0] = -1. * v[0];
        u0 = v[0];
        v[0] = u0 * nx - v[1] * ny;
        v[1] = u0 * ny + v[1] * nx;
        if (damp_vel) {
            v[0] *= 1. - p.damp;
            v[1] *= 1. - p.damp;
            if (DIM == 3) v[2] *= 1. - p.damp;
        }
    }

    __device__ void count_open(int* stats, int label) {
        if (p.bnd_statistics && stats) atomicAdd(&stats[label - 1], 1);
    }

    __device__ void compute_bc(int bnd_j, int* stats) {
        double damp = p.damp;
        bool strand_condition = false;
        if (bnd_j != -1) {
            int lab = __ldg(&m.elabel[CG_IDX(m, bnd_j, m.ne)]);
            if (lab == BND_WALL_REF && p.strand > 0.) strand_condition = rng_uniform(rng) < p.strand;
            if (strand_condition) record_strand(p, pstep, pidx, x[0], x[1], DIM == 3 ? x[2] : 0.);
            if (lab == BND_WALL_REF && !strand_condition) {
                int bnd_jj = bnd_j;
                for (int rc = 0; tri == PART_LOC_O && rc < p.max_rebounds; ++rc) {
                    int4 e = __ldg(&m.edge[CG_IDX(m, bnd_jj, m.ne)]);
                    double2 a = __ldg(&m.xy[CG_IDX(m, e.x, m.nv)]), b = __ldg(&m.xy[CG_IDX(m, e.y, m.nv)]);
                    // intersections.pyx:27-62
                    double coef = 1. - damp / 2.;
                    double nx = a.y - b.y, ny = b.x - a.x;
                    double norm2 = nx * nx + ny * ny;
                    double dist = (x[0] - a.x) * nx + (x[1] - a.y) * ny;
                    double px = x[0] - 2. * ((dist * coef) / norm2) * nx;
                    double py = x[1] - 2. * ((dist * coef) / norm2) * ny;
                    x[0] = px;
                    x[1] = py;
                    // the mixed form's filtered tests (same decisions, FP64
                    // only inside the rounding bands); 2D only: in the 3D
                    // kernels they cost more registers than they save
                    if constexpr (std::is_same<FT, float>::value && DIM == 2)
                        xy_localize_filtered(m, ltri, x0[0], x0[1], px, py, tri, bnd_jj);
                    else
                        xy_localize(m, ltri, x0[0], x0[1], px, py, tri, bnd_jj);
                    if (tri == PART_LOC_O && bnd_jj != -1) {
                        int lj = __ldg(&m.elabel[CG_IDX(m, bnd_jj, m.ne)]);
                        if (lj >= BND_OPEN_REF) {
                            count_open(stats, lj);
                            deleted = true;
                            break;
                        }
                    }
                    if (p.model == 0 || p.model >= 2) reflect(up, a.x, a.y, b.x, b.y, true);
                    if (p.model == 3) reflect(us, a.x, a.y, b.x, b.y, false);
                    if (tri == PART_LOC_O && bnd_jj == -1) break;
                }
                if (DIM == 3 && !deleted && tri != PART_LOC_O) ll = z_localize(tri, x[0], x[1], x[2]);
            }
            if (lab >= BND_OPEN_REF) {
                if (!deleted) count_open(stats, lab);
                deleted = true;
            }
        }
        if (deleted) return;
        // compute_bc.pyx:287-374
        if (DIM == 3) {
            for (int side = 0; side < 2; ++side) {
                int want = side == 0 ? PART_LOC_B : PART_LOC_A;
                if (!(ll == want && tri != PART_LOC_O)) continue;
                double zbp = zb_at(tri, x[0], x[1]);
                double zsp = zs_at(tri, f.nlayers - 1, x[0], x[1]);
                double hp = fmax(0., zsp - zbp);
                if (side == 0) {
                    double dz = fabs(zbp - x[2]);
                    x[2] = fmin(zbp + (1. - damp) * dz, zbp + 0.5 * hp);
                } else {
                    double dz = fabs(x[2] - zsp);
                    x[2] = fmax(zsp - (1. - damp) * dz, zsp - 0.5 * hp);
                }
                ll = lower_layer_index(f.nlayers, zsp, zbp, x[2]);
                double sg = side == 0 ? 1. : -1.;
                if (p.model >= 2) up[2] = sg * fabs(up[2]) * (1. - damp);
                if (p.model == 3) us[2] = sg * fabs(us[2]) * (1. - damp);
            }
        }
        // compute_bc.pyx:378-395
        if (tri == PART_LOC_O || ll == PART_LOC_B || ll == PART_LOC_A) deleted = true;
    }
};

}  // namespace cg

#include "cg_lsm23.cuh"

namespace cg {

// ziggurat tables into shared memory
__device__ __forceinline__ void load_zig(ZigTables& zt) {
    for (int t = threadIdx.x; t < 128; t += blockDim.x) {
        zt.kn[t] = g_zig.kn[t];
        zt.wn[t] = g_zig.wn[t];
        zt.fn[t] = g_zig.fn[t];
    }
    __syncthreads();
}

// aux: 0 = state only; 1 = also write velocity / fluid velocity seen;
//      2 = also write last_position / last_velocity / last_tri (the last
//      step of a batch, so that every public array is current afterwards).
// q.e != nullptr (2D): particles leaving their start triangle are queued
// for walk_kernel instead of walking here.
// One particle of the step (the body of the particle loop).
template <int DIM, typename FT, int MODEL, int SCHEME = 0>
__device__ __forceinline__ void step_particle(const DevMesh& m, const DevFields<FT>& f,
                                              const DevParams& p, DevState& s,
                                              const WalkQueue& wq, int aux, int step_index,
                                              int* __restrict__ stats,
                                              uint32_t* __restrict__ err_word,
                                              const ZigTables& zt, int i,
                                              const Zig32* z32 = nullptr) {
    int tri = s.tri[i];
    if (tri < 0) return;  // inactive (-1) or awaiting initialization (-2)

    Particle<DIM, FT> q(m, f, p, zt);
    q.z32 = z32;
    q.tri = tri;
    q.tri0 = tri;
    q.ltri = tri;
    const int ai = aux_index(s, i);
    q.ll = DIM == 3 ? s.lowerlayer[widx(s, i, ai, W_LAYER)] : 0;
    q.ll0 = q.ll;
    q.defer = (DIM == 2) && (wq.e != nullptr) && MODEL == 1;
    const int D = DIM;
#pragma unroll
    for (int d = 0; d < D; ++d) {
        q.x[d] = s.pos[(size_t)i * D + d];
        q.x0[d] = q.x[d];
    }
    const double sx = q.x[0], sy = q.x[1];   // last_position of the step
    // mixed LSM2/LSM3: velocities as FP32 values (see Particle::store)
    constexpr bool v32 = std::is_same<FT, float>::value && MODEL >= 2;
    if (MODEL >= 2) {
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const double v = vel_ld(s, (size_t)widx(s, i, ai, W_VEL) * D + d);
            q.up[d] = v32 ? (double)(float)v : v;
        }
    }
    if (MODEL == 3) {
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const double v = fvs_ld(s, (size_t)widx(s, i, ai, W_FVS) * D + d);
            q.us[d] = v32 ? (double)(float)v : v;
        }
    }
    q.rng.state = s.rng[i];
    q.rng.inc = ((uint64_t)(uint32_t)s.tag[i] << 1) | 1ULL;
    q.rng.err = 0;
    double dp = (DIM == 3 || MODEL >= 2) ? s.diameter[widx(s, i, ai, W_DIAM)] : 0.;

    int bnd_j = -1;
    if constexpr (MODEL == 1) bnd_j = q.update_lsm1(dp);
    else if constexpr (MODEL == 2) bnd_j = update_lsm2<SCHEME>(q, dp);
    else bnd_j = update_lsm3<SCHEME>(q, dp);

    uint32_t e = q.err | q.rng.err;
    if (e) atomicOr(err_word, e);
    if (q.deferred) {
        int slot = queue_slot(wq);
        WalkEntry w;
        w.xn = q.x[0];
        w.yn = q.x[1];
        w.rng = q.rng.state;
        w.i = i;
        w.tri0 = q.tri0;
        wq.e[slot] = w;
        return;
    }
    if (p.bc_on) {
        q.pidx = ai + s.base;
        q.pstep = step_index;
        q.compute_bc(bnd_j, stats);
    } else if (q.tri == PART_LOC_O || q.ll == PART_LOC_B || q.ll == PART_LOC_A) {
        q.deleted = true;
    }
    e = q.err | q.rng.err;
    if (e) atomicOr(err_word, e);
    q.store(s, i, aux, step_index);
    if (p.ncsec) {
        const bool del = q.deleted;
        count_sections(p, stats, del ? 0. : sx, del ? 0. : sy, del ? 0. : q.x[0],
                       del ? 0. : q.x[1]);
    }
}

// aux: 0 = state only; 1 = also write velocity / fluid velocity seen;
//      2 = also write last_position / last_velocity / last_tri (the last
//      step of a batch, so that every public array is current afterwards).
// wq.e != nullptr (2D): particles leaving their start triangle are queued
// for walk_kernel instead of walking here.  Persistent grid (one wave of
// resident blocks) striding over the particles.
// MODEL: 1, 2 or 3 (LSM1/2/3); SCHEME: the LSM2/LSM3 time scheme.  One
// instantiation per combination, so that each kernel holds one integrator
// inlined (no particle state in local memory) and the LSM1 kernels keep
// their register budget.
// Resident blocks of 256 per SM that a step kernel's register budget is set
// for: two for the mixed LSM2/LSM3 kernels (at most 128 registers; at one
// block per SM their dependent loads stall with nothing to hide them), one
// otherwise.
template <typename FT, int MODEL>
constexpr int step_min_blocks() {
    return (MODEL >= 2 && std::is_same<FT, float>::value) ? 2 : 1;
}

template <int DIM, typename FT, int MODEL = 1, int SCHEME = 0>
__global__ void __launch_bounds__(256, step_min_blocks<FT, MODEL>())
    step_kernel(DevMesh m, DevFields<FT> f, DevParams p,
                                                   DevState s, WalkQueue wq, int aux,
                                                   int step_index, int* __restrict__ stats,
                                                   uint32_t* __restrict__ err_word) {
    reset_next_queue(wq);
    __shared__ ZigTables zt;
    // the mixed LSM2/LSM3 direct integrators draw from FP32 tables
    constexpr bool z32_on = std::is_same<FT, float>::value && MODEL >= 2;
    __shared__ Zig32 z32[1];
    if constexpr (z32_on) {
        for (int t = threadIdx.x; t < 128; t += blockDim.x) {
            z32[0].kn[t] = g_zig.kn[t];
            z32[0].wn[t] = (float)g_zig.wn[t];
            z32[0].fn[t] = (float)g_zig.fn[t];
        }
    }
    load_zig(zt);   // ends with __syncthreads
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < s.n; i += gridDim.x * blockDim.x)
        step_particle<DIM, FT, MODEL, SCHEME>(m, f, p, s, wq, aux, step_index, stats, err_word,
                                               zt, i, z32_on ? &z32[0] : nullptr);
}

// blocks of one wave of resident blocks of `kernel` (persistent grid)
template <typename K>
inline int resident_blocks(K kernel, int bs) {
    int dev = 0, nsm = 152, per = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, bs, 0);
    return nsm * (per < 1 ? 1 : per);
}

// step_kernel<DIM, FT, 1> (LSM1) over every particle on a persistent grid
template <int DIM, typename FT>
void launch_lsm1_kernel(const DevMesh& m, const DevFields<FT>& f, const DevParams& p,
                        const DevState& s, const WalkQueue& wq, int aux, int step_index,
                        int* stats, uint32_t* err, cudaStream_t st) {
    const int bs = 256;
    const int need = (s.n + bs - 1) / bs;
    if (need == 0) return;
    static int wave = 0;
    if (!wave) wave = resident_blocks(step_kernel<DIM, FT, 1>, bs);
    step_kernel<DIM, FT, 1><<<need < wave ? need : wave, bs, 0, st>>>(m, f, p, s, wq, aux,
                                                                      step_index, stats, err);
}

// step_kernel<DIM, FT, model, time scheme> for LSM2/LSM3 runs (instantiated
// in cg_lsm23_plain.cu / cg_lsm23_mixed.cu)
template <int DIM, typename FT>
void launch_lsm23_kernel(const DevMesh& m, const DevFields<FT>& f, const DevParams& p,
                         const DevState& s, int aux, int step_index, int* stats, uint32_t* err,
                         cudaStream_t st) {
    const int bs = 256;
    const int need = (s.n + bs - 1) / bs;
    if (need == 0) return;
    static int wave[7] = {0, 0, 0, 0, 0, 0, 0};
    const WalkQueue none{nullptr, nullptr};
    auto go = [&](auto kernel, int idx) {
        if (!wave[idx]) wave[idx] = resident_blocks(kernel, bs);
        int nb = need < wave[idx] ? need : wave[idx];
        kernel<<<nb, bs, 0, st>>>(m, f, p, s, none, aux, step_index, stats, err);
    };
    const int ts = p.time_scheme;
    if (p.model == 2 && ts == 1) go(step_kernel<DIM, FT, 2, 1>, 0);
    else if (p.model == 2 && ts == 2) go(step_kernel<DIM, FT, 2, 2>, 1);
    else if (p.model == 2 && ts == 3) go(step_kernel<DIM, FT, 2, 3>, 2);
    else if (p.model == 2 && ts == 4) go(step_kernel<DIM, FT, 2, 4>, 3);
    else if (p.model == 2) go(step_kernel<DIM, FT, 2, 5>, 4);
    else if (ts == 1) go(step_kernel<DIM, FT, 3, 1>, 5);
    else go(step_kernel<DIM, FT, 3, 5>, 6);
}

// walk kernel launch shape: blocks of 64, 32 per SM (grid-stride beyond)
constexpr int WALK_BLOCK = 64, WALK_BLOCKS_PER_SM = 32;

// Second half of the step for queued (2D) particles: path walk from the
// start triangle (xylocalizer.pyx:338-435, then the global fallback) and the
// boundary conditions.  Grid-stride over the entries of this step.
template <typename FT, bool MIXED>
__global__ void __launch_bounds__(WALK_BLOCK) walk_kernel(DevMesh m, DevFields<FT> f, DevParams p,
                                                   DevState s, WalkQueue wq, int aux,
                                                   int step_index, int* __restrict__ stats,
                                                   uint32_t* __restrict__ err_word) {
    // launched as a programmatic dependent of the step kernel (mixed form):
    // wait until that grid has finished and its writes are visible (a no-op
    // for an ordinary launch)
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const int count = *wq.count;
    // blocks beyond the queue leave before loading the tables (the grid is
    // sized for any count; most steps queue few particles)
    if ((long long)blockIdx.x * blockDim.x >= count) return;
    __shared__ ZigTables zt;
    load_zig(zt);
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < count; j += gridDim.x * blockDim.x) {
        WalkEntry w = wq.e[j];
        int i = (int)CG_IDX(m, w.i, s.n);
        Particle<2, FT> q(m, f, p, zt);
        const int tri0 = w.tri0;   // s.tri[i], carried in the entry: the first record load need not wait for it
        double2 x0 = (s.work & W_SPLIT) ? join_pos(reinterpret_cast<const float4*>(s.pos)[i])
                                        : reinterpret_cast<const double2*>(s.pos)[i];
        q.tri0 = tri0;
        q.ltri = tri0;
        q.ll = q.ll0 = 0;
        q.x[0] = w.xn;
        q.x[1] = w.yn;
        q.x0[0] = x0.x;
        q.x0[1] = x0.y;
        q.rng.state = w.rng;
        q.rng.inc = ((uint64_t)(uint32_t)s.tag[i] << 1) | 1ULL;
        q.rng.err = 0;
        if (aux >= 1 || p.model >= 2) {
            // LSM1: up = us = U(x0) (update_state_lsm1.pyx:144-163)
            double ux, uy, uz;
            q.velocity(tri0, 0, x0.x, x0.y, 0., ux, uy, uz);
            q.up[0] = q.us[0] = ux;
            q.up[1] = q.us[1] = uy;
        }
        int nk, bnd;
        if (MIXED) path_walk_mixed(m, tri0, x0.x, x0.y, w.xn, w.yn, nk, bnd);
        else path_walk(m, tri0, x0.x, x0.y, w.xn, w.yn, nk, bnd);
        if (nk == -1 && bnd == -1) nk = grid_locate(m, w.xn, w.yn);
        q.tri = nk;
        q.pidx = aux_index(s, i) + s.base;
        q.pstep = step_index;
        if (p.bc_on) q.compute_bc(bnd, stats);
        else if (q.tri == PART_LOC_O) q.deleted = true;
        uint32_t e = q.err | q.rng.err;
        if (e) atomicOr(err_word, e);
        q.store(s, i, aux, step_index);
        if (p.ncsec) {
            const bool del = q.deleted;
            count_sections(p, stats, del ? 0. : x0.x, del ? 0. : x0.y, del ? 0. : q.x[0],
                           del ? 0. : q.x[1]);
        }
    }
}

}  // namespace cg
