// cg_step_mixed.cuh -- the mixed-precision form of the fused step (LSM1 2D).
//
// FP64 is kept only where stability needs it: particle positions and their
// accumulation, the in-element test and the edge-crossing tests that decide
// localization, simulated time (host).  Node fields are stored in FP32 and
// interpolated, differentiated and integrated in FP32; random normals are
// FP32 ziggurat draws from the same per-particle PCG32 stream.
//
// In-element test: barycentric coordinates are evaluated in FP32 from the
// FP64 offset to vertex a, with a rounding bound per coordinate.  Points
// certainly inside (every coordinate above its bound) or certainly outside
// (one below minus its bound) are decided there; the thin band in between
// is decided by the exact FP64 predicate of the plain form.  So the mixed
// form takes the same localization decision as the plain form for the same
// position; only the positions themselves differ (FP32 increments).
#pragma once

#include "cg_step.cuh"

namespace cg {

// xylocalizer.pyx:27-124 method 3, first test through the FP32 filter
__device__ __forceinline__ void xy_localize_mixed(const DevMesh& m, const Tri32& t, int k,
                                                  double p0x, double p0y, double x, double y,
                                                  int& new_k, int& bnd) {
    bnd = -1;
    if (in_tri_mixed(m, t, k, x, y)) { new_k = k; return; }
    path_walk_mixed(m, k, p0x, p0y, x, y, new_k, bnd);
    if (new_k == -1 && bnd == -1) new_k = grid_locate(m, x, y);
}

// FP32 P1 interpolation of the packed node record {ux, uy, K, zs}
struct Node4 {
    float4 n0, n1, n2;
};

template <typename T>
__device__ __forceinline__ Node4 load_nodes(const float4* __restrict__ f, const T& t) {
    Node4 r;
    r.n0 = __ldg(&f[t.tv.x]);
    r.n1 = __ldg(&f[t.tv.y]);
    r.n2 = __ldg(&f[t.tv.z]);
    return r;
}

// The FP32 arithmetic that reaches the particle state (here, the Euler
// increment and the samplers) is written with explicitly rounded operations
// (__fmul_rn, __fmaf_rn, ...), so that every compiled form of the step
// (per-call outputs or not, configuration forms) rounds the same way and a
// run's results do not depend on how its steps are split into calls.
__device__ __forceinline__ void vel32(const Node4& n, const Bary& b, float& ux, float& uy) {
    ux = __fmaf_rn(b.l2, n.n2.x, __fmaf_rn(b.l1, n.n1.x, __fmul_rn(b.l0, n.n0.x)));
    uy = __fmaf_rn(b.l2, n.n2.y, __fmaf_rn(b.l1, n.n1.y, __fmul_rn(b.l0, n.n0.y)));
}

// Runge-Kutta stages of update_state_lsm1.pyx:179-656 in the mixed form:
// each stage point is localized from (tri0, x0); a stage leaving the domain
// stops the scheme with an Euler step.  Kept out of line (cold path); the
// particle's values go in and out by value, so none of the caller's locals
// takes an address (they stay in registers).
struct RkOut {
    double xn, yn;
    int tri, bnd;
};

static __device__ __noinline__ RkOut rk_mixed(const DevMesh& m, const float4* __restrict__ cur,
                                              const DevParams& p, int tri0, double x0x,
                                              double x0y, float ux, float uy) {
    const Tri32 t0 = load_tri32(m, tri0);
    RkOut o{x0x, x0y, tri0, -1};
    const float dt = p.dt32;
    const float up0 = ux, up1 = uy;
    const int ns = p.time_scheme == 2 ? 1 : (p.time_scheme == 3 ? 2 : 3);
    float kx[4], ky[4];
    kx[0] = ux * dt;
    ky[0] = uy * dt;
    for (int st = 0; st < ns; ++st) {
        float cst;
        if (p.time_scheme == 2) cst = 0.5f;
        else if (p.time_scheme == 3) cst = st == 0 ? (1.f / 3.f) : (2.f / 3.f);
        else cst = st < 2 ? 0.5f : 1.f;
        float fx = (p.time_scheme == 2) ? 0.5f * ux * dt : cst * kx[st];
        float fy = (p.time_scheme == 2) ? 0.5f * uy * dt : cst * ky[st];
        double xt = x0x + (double)fx, yt = x0y + (double)fy;
        int tt, bnd;
        xy_localize_mixed(m, t0, tri0, x0x, x0y, xt, yt, tt, bnd);
        if (bnd != -1) {
            o.tri = tt;
            o.xn = x0x + (double)(up0 * dt);
            o.yn = x0y + (double)(up1 * dt);
            o.bnd = bnd;
            return o;
        }
        Tri32 ts = load_tri32(m, tt);
        Node4 ns4 = load_nodes(cur, ts);
        float sx, sy;
        vel32(ns4, bary32(ts, xt, yt), sx, sy);
        kx[st + 1] = sx * dt;
        ky[st + 1] = sy * dt;
    }
    float dxs, dys;
    if (p.time_scheme == 2) { dxs = kx[1]; dys = ky[1]; }
    else if (p.time_scheme == 3) { dxs = 0.25f * kx[0] + 0.75f * kx[2]; dys = 0.25f * ky[0] + 0.75f * ky[2]; }
    else { dxs = (kx[0] + 2.f * kx[1] + 2.f * kx[2] + kx[3]) / 6.f; dys = (ky[0] + 2.f * ky[1] + 2.f * ky[2] + ky[3]) / 6.f; }
    o.xn += (double)dxs;
    o.yn += (double)dys;
    return o;
}

// Boundary conditions (compute_bc.pyx:35-395) with the FP64 mirror and the
// exact walk of the plain form.  Out of line (cold path), values in and out.
struct BcOut {
    double xn, yn;
    uint64_t rng;
    uint32_t err;
    int tri;
    bool deleted;
};

static __device__ __noinline__ BcOut bc_mixed(const DevMesh& m, const DevFields<float>& f,
                                              const DevParams& p, const ZigTables& z64,
                                              uint64_t rng_state, uint64_t rng_inc, double x0x,
                                              double x0y, float up0, float up1, int tri0, int ltri,
                                              int bnd_j, int* stats, double xn, double yn, int tri,
                                              int pidx, int pstep) {
    Particle<2, float> q(m, f, p, z64);
    q.pidx = pidx;
    q.pstep = pstep;
    q.rng.state = rng_state;
    q.rng.inc = rng_inc;
    q.rng.err = 0;
    q.x[0] = xn; q.x[1] = yn;
    q.x0[0] = x0x; q.x0[1] = x0y;
    q.up[0] = up0; q.up[1] = up1;
    q.us[0] = up0; q.us[1] = up1;
    q.tri = tri; q.tri0 = tri0; q.ltri = ltri; q.ll = 0; q.ll0 = 0;
    if (p.bc_on) q.compute_bc(bnd_j, stats);
    else if (q.tri == PART_LOC_O) q.deleted = true;
    BcOut o;
    o.rng = q.rng.state;
    o.err = q.rng.err | q.err;
    o.xn = q.x[0];
    o.yn = q.x[1];
    o.tri = q.tri;
    o.deleted = q.deleted;
    return o;
}

// The walk's first hops for a split end position, decided in FP32 where the
// signs are certain.  From the start triangle (start point certainly
// inside) the segment crosses exactly the edge the end point is certainly
// beyond, as one_hop argues; in each triangle entered, a straight segment
// that came in through one edge and ends certainly beyond exactly one other
// edge (and certainly inside the third's half-plane) leaves through that
// edge, the only one the reference's walk finds there
// (xylocalizer.pyx:375-415).  After each crossing the walk's test of the end
// point in the new triangle is made here (exact in the rounding band).
// Returns the triangle holding the end point within HOPS crossings, else -1
// (the walk kernel decides: more hops, boundary edges, uncertain signs).
template <int HOPS>
__device__ __forceinline__ int hop_walk_split(const DevMesh& m, const Tri32S& t0, const Bary& bs,
                                              const Bary& be, float4 pn) {
    if (!(bs.l0 > bs.e0 && bs.l1 > bs.e1 && bs.l2 > bs.e2)) return -1;
    // neighbours of the current triangle, from its record
    int n0 = t0.tv.w, n1 = __float_as_int(t0.g1.z), n2 = __float_as_int(t0.g1.w);
    Bary b = be;
#pragma unroll 1
    for (int h = 0; h < HOPS; ++h) {
        const int j = single_exit(b);
        if (j < 0) return -1;
        const int kn = j == 0 ? n0 : (j == 1 ? n1 : n2);
        if (kn < 0) return -1;   // boundary edge: the walk kernel applies the conditions
        const Tri32S tn = load_tri32s(m, kn);
        const float2 r = split_offset(tn, pn);
        b = bary32_off(tn, r.x, r.y);
        const int d = decide32(b);
        if (d == 1) return kn;
        if (d < 0) {
            const double2 x = join_pos(pn);
            return in_tri(m, kn, x.x, x.y) ? kn : -1;
        }
        n0 = tn.tv.w;
        n1 = __float_as_int(tn.g1.z);
        n2 = __float_as_int(tn.g1.w);
    }
    return -1;
}

#ifndef MIXED_HOPS
#define MIXED_HOPS 3
#endif

// the per-particle state the mixed LSM1 step streams in
struct MixedIn {
    int tri;
    int tag;
    uint64_t rng;
    float4 pos;   // split pair (W_SPLIT) or the bits of the FP64 pair
};

__device__ __forceinline__ MixedIn load_mixed_in(const DevState& s, int i) {
    MixedIn in;
    in.tri = __ldcs(&s.tri[i]);
    in.pos = __ldcs(reinterpret_cast<const float4*>(s.pos) + i);
    in.rng = __ldcs(reinterpret_cast<const unsigned long long*>(s.rng) + i);
    in.tag = __ldcs(&s.tag[i]);
    return in;
}

__device__ __forceinline__ double2 double2_from_bits(float4 r) {
    return make_double2(__hiloint2double(__float_as_int(r.y), __float_as_int(r.x)),
                        __hiloint2double(__float_as_int(r.w), __float_as_int(r.z)));
}

// LSM1 2D, mixed precision.  update_state_lsm1.pyx:30-133 (schemes 135-656,
// diffusion 658-726) with the boundary conditions of compute_bc.pyx.
// SPLIT: the working position is a split pair (W_SPLIT); the Euler step then
// runs without FP64 arithmetic outside the rounding bands, the walk and the
// boundary conditions (which work on its FP64 value).
// EQ: the Euler scheme with a walk queue (the caller guarantees both): every
// particle that does not end in a triangle reached here goes to the queue,
// so this form has no out-of-line calls and no deletions.
// TWO: the working copies have two velocity arrays (W_VEL2); a step writes
// its velocity alone and the write-back gives the fluid velocity seen and the
// last velocity.  Only the steps with per-call outputs (aux >= 1) differ.
// DC >= 0: a form compiled for one run configuration, for runs without
// control sections: DC the diffusion class (0 none, 1 constant diffusivity,
// 2 k-epsilon: diffusion_model 2 or 3), RM the random number method.  -1:
// read from the parameters.
template <bool SPLIT, bool EQ = false, bool TWO = false, int DC = -1, int RM = -1>
__device__ __forceinline__ void step_mixed_particle(const DevMesh& m, const DevFields<float>& f,
                                                    const DevParams& p, DevState& s,
                                                    const WalkQueue& wq, int aux, int step_index,
                                                    int* __restrict__ stats,
                                                    uint32_t* __restrict__ err_word,
                                                    const Zig32& z32, const MixedIn& in, int i) {
    // particle state streams through L2 once per step (evict-first loads and
    // stores): the mesh and node records stay in L2
    const int tri0 = in.tri;
    if (tri0 < 0) return;
    const float4* __restrict__ cur = reinterpret_cast<const float4*>(f.cur);
    float4 xs = make_float4(0.f, 0.f, 0.f, 0.f);   // SPLIT: the start position
    double2 x0 = make_double2(0., 0.);
    if constexpr (SPLIT) xs = in.pos;
    else x0 = double2_from_bits(in.pos);
    Rng rng;
    rng.state = in.rng;
    rng.inc = ((uint64_t)(uint32_t)in.tag << 1) | 1ULL;
    rng.err = 0;
    double2 lastv = make_double2(0., 0.);
    if (aux >= 2 && !TWO)
        lastv = reinterpret_cast<const double2*>(s.vel)[widx(s, i, aux_index(s, i), W_VEL)];

    const float dt = p.dt32;
    const bool euler = EQ || p.time_scheme == 1;
    // start record and offset to its vertex a
    Tri32 t0;
    Tri32S t0s;
    float rx0, ry0;
    Node4 n0;
    Bary b0;
    if constexpr (SPLIT) {
        t0s = load_tri32s(m, tri0);
        const float2 r = split_offset(t0s, xs);
        rx0 = r.x;
        ry0 = r.y;
        n0 = load_nodes(cur, t0s);
        b0 = bary32_off(t0s, rx0, ry0);
        if (!euler) x0 = join_pos(xs);   // the Runge-Kutta stages work on the FP64 value
    } else {
        t0 = load_tri32(m, tri0);
        rx0 = (float)(x0.x - t0.a.x);
        ry0 = (float)(x0.y - t0.a.y);
        n0 = load_nodes(cur, t0);
        b0 = bary32_off(t0, rx0, ry0);
    }
    float ux, uy;
    vel32(n0, b0, ux, uy);
    float up0 = ux, up1 = uy;   // velocity = fluid velocity seen = U(x0)
    double xn = x0.x, yn = x0.y;
    int tri = tri0, ltri = tri0, bnd_j = -1;
    // Euler: the whole step's increment is accumulated in FP32 and added to
    // the position once
    float dx = 0.f, dy = 0.f;
    if (euler) {
        dx = __fmul_rn(ux, dt);
        dy = __fmul_rn(uy, dt);
    } else if constexpr (!EQ) {
        const RkOut r = rk_mixed(m, cur, p, tri0, x0.x, x0.y, ux, uy);
        xn = r.xn;
        yn = r.yn;
        tri = r.tri;
        bnd_j = r.bnd;
    }

    // diffusion (update_state_lsm1.pyx:658-726), K at the start point
    constexpr bool CONF = DC >= 0;
    const bool diff_on = CONF ? DC != 0 : p.diffmod != 0;
    const bool diff_k = CONF ? DC == 2 : (p.diffmod == 2 || p.diffmod == 3);
    const int rng_method = RM > 0 ? RM : p.rng_method;
    const int ncsec = CONF ? 0 : p.ncsec;
    if (diff_on) {
        float diffx, driftx = 0.f, drifty = 0.f;
        if (diff_k) {
            float4 g0, g1;
            if constexpr (SPLIT) {
                g0 = t0s.g0;
                g1 = t0s.g1;
            } else {
                g0 = t0.g0;
                g1 = t0.g1;
            }
            float K = __fmaf_rn(b0.l2, n0.n2.z, __fmaf_rn(b0.l1, n0.n1.z, __fmul_rn(b0.l0, n0.n0.z)));
            float dKdx = __fmaf_rn(n0.n2.z, g0.z, __fmaf_rn(n0.n1.z, g0.y, __fmul_rn(n0.n0.z, g0.x)));
            float dKdy = __fmaf_rn(n0.n2.z, g1.y, __fmaf_rn(n0.n1.z, g1.x, __fmul_rn(n0.n0.z, g0.w)));
            K = fmaxf(0.f, K);
            diffx = __fmul_rn(sqrtf(__fmul_rn(2.f, K)), p.sqrtdt32);
            driftx = __fmul_rn(dKdx, dt);
            drifty = __fmul_rn(dKdy, dt);
        } else {
            diffx = p.diffx32;
        }
        float xix = 0.f, xiy = 0.f;
        if (diffx != 0.f) pair32(rng, rng_method, z32, xix, xiy);
        if (euler) {
            dx = __fadd_rn(dx, __fmaf_rn(diffx, xix, driftx));
            dy = __fadd_rn(dy, __fmaf_rn(diffx, xiy, drifty));
        } else {
            xn += (double)__fmaf_rn(diffx, xix, driftx);
            yn += (double)__fmaf_rn(diffx, xiy, drifty);
        }
    }
    float4 xe = xs;   // SPLIT: the end position
    if (euler) {
        if constexpr (SPLIT) {
            xe = split_add(xs, dx, dy);
        } else {
            xn = x0.x + (double)dx;
            yn = x0.y + (double)dy;
        }
    } else if constexpr (SPLIT) {
        xe = split_pos(xn, yn);
    }
    // SPLIT: FP64 values of the start and end positions, formed where needed
    bool have64 = !SPLIT || !euler;
    auto need64 = [&]() {
        if constexpr (SPLIT) {
            if (!have64) {
                x0 = join_pos(xs);
                const double2 e = join_pos(xe);
                xn = e.x;
                yn = e.y;
                have64 = true;
            }
        }
    };

    if (bnd_j == -1) {
        ltri = tri0;
        if (EQ || wq.e != nullptr) {
            // leaves the start triangle: one hop here, else walk + boundary
            // conditions in walk_kernel
            int kn;
            if constexpr (SPLIT) {
                const Bary be = euler ? bary32_moved(t0s, rx0, ry0, dx, dy)
                                      : [&] {
                                            const float2 r = split_offset(t0s, xe);
                                            return bary32_off(t0s, r.x, r.y);
                                        }();
                int d = decide32(be);
                if (d < 0) {
                    need64();
                    d = in_tri(m, tri0, xn, yn) ? 1 : 0;
                }
                kn = d ? tri0 : hop_walk_split<MIXED_HOPS>(m, t0s, b0, be, xe);
            } else {
                const Bary be = euler ? bary32_moved(t0, rx0, ry0, dx, dy) : bary32(t0, xn, yn);
                const bool inside = in_tri_decide(m, be, tri0, xn, yn);
                kn = inside ? tri0 : one_hop(m, tri0, b0, be, xn, yn);
            }
            if (kn < 0) {
                need64();
                if (rng.err) atomicOr(err_word, rng.err);
                int slot = queue_slot(wq);
                WalkEntry w;
                w.xn = xn;
                w.yn = yn;
                w.rng = rng.state;
                w.i = i;
                w.tri0 = tri0;
                wq.e[slot] = w;
                return;
            }
            tri = kn;
        } else {
            need64();
            if constexpr (SPLIT) t0 = load_tri32(m, tri0);
            xy_localize_mixed(m, t0, tri0, x0.x, x0.y, xn, yn, tri, bnd_j);
        }
    }

    bool deleted = false;
    if (!EQ && (bnd_j != -1 || tri == PART_LOC_O)) {
        need64();
        const BcOut o = bc_mixed(m, f, p, g_zig, rng.state, rng.inc, x0.x, x0.y, up0, up1, tri0,
                                 ltri, bnd_j, stats, xn, yn, tri, aux_index(s, i) + s.base,
                                 step_index);
        rng.state = o.rng;
        rng.err |= o.err;
        xn = o.xn;
        yn = o.yn;
        tri = o.tri;
        deleted = o.deleted;
        if constexpr (SPLIT) xe = split_pos(xn, yn);
    }
    if (rng.err) atomicOr(err_word, rng.err);

    if (deleted) {
        const int a = aux_index(s, i);
        const int ix = widx(s, i, a, W_AUXW);
        reinterpret_cast<double2*>(s.pos)[i] = make_double2(0., 0.);
        reinterpret_cast<double2*>(s.vel)[widx(s, i, a, W_VEL)] = make_double2(0., 0.);
        reinterpret_cast<double2*>(s.last_pos)[ix] = make_double2(0., 0.);
        if (!TWO) {   // (TWO: the write-back zeroes them)
            reinterpret_cast<double2*>(s.fvs)[widx(s, i, a, W_FVS | W_AUXW)] = make_double2(0., 0.);
            reinterpret_cast<double2*>(s.last_vel)[ix] = make_double2(0., 0.);
        }
        s.diameter[widx(s, i, a, W_DIAM)] = 0.;
        s.tri[i] = -1;
        s.last_tri[ix] = -1;
        s.lowerlayer[a] = 0;
        s.tag[i] = -2 - step_index;
        s.rng[i] = rng.state;
        if (ncsec) count_sections(p, stats, 0., 0., 0., 0.);
        return;
    }
    if (ncsec) {
        need64();
        count_sections(p, stats, x0.x, x0.y, xn, yn);
    }
    if constexpr (SPLIT) __stcs(reinterpret_cast<float4*>(s.pos) + i, xe);
    else __stcs(reinterpret_cast<double2*>(s.pos) + i, make_double2(xn, yn));
    __stcs(&s.tri[i], tri);
    __stcs(reinterpret_cast<unsigned long long*>(s.rng) + i, (unsigned long long)rng.state);
    if (aux >= 1) {
        const int a = aux_index(s, i);
        // TWO: the velocity alone (it is the fluid velocity seen; the other
        // array holds the last velocity)
        reinterpret_cast<double2*>(s.vel)[widx(s, i, a, W_VEL)] = make_double2(up0, up1);
        if (!TWO)
            reinterpret_cast<double2*>(s.fvs)[widx(s, i, a, W_FVS | W_AUXW)] = make_double2(up0, up1);
        if (aux >= 2) {
            if constexpr (SPLIT) {
                if (!have64) x0 = join_pos(xs);
            }
            const int ix = widx(s, i, a, W_AUXW);
            reinterpret_cast<double2*>(s.last_pos)[ix] = x0;
            if (!TWO) reinterpret_cast<double2*>(s.last_vel)[ix] = lastv;
            s.last_tri[ix] = ltri;
        }
    }
}

// Persistent grid (one wave of resident blocks) striding over the particles.
// MINB: resident blocks of 256 per SM the register budget is set for.
// DC, RM: the form compiled for one run configuration (step_mixed_particle);
// with DC >= 0 and not TWO, the form of the steps without per-call outputs
// (aux 0).
template <int MINB, bool SPLIT = false, bool EQ = false, bool TWO = false, int DC = -1,
          int RM = -1>
__global__ void __launch_bounds__(256, MINB) step_mixed2d_kernel(DevMesh m, DevFields<float> f,
                                                                DevParams p, DevState s,
                                                                WalkQueue wq, int aux,
                                                                int step_index,
                                                                int* __restrict__ stats,
                                                                uint32_t* __restrict__ err_word) {
    // every block of this one-wave grid is resident: let the walk kernel
    // that follows be set up now (it waits for this grid's completion)
    asm volatile("griddepcontrol.launch_dependents;");
    reset_next_queue(wq);
    __shared__ Zig32 z32;
    for (int t = threadIdx.x; t < 128; t += blockDim.x) {
        z32.kn[t] = g_zig.kn[t];
        z32.wn[t] = (float)g_zig.wn[t];
        z32.fn[t] = (float)g_zig.fn[t];
    }
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < s.n; i += gridDim.x * blockDim.x)
        step_mixed_particle<SPLIT, EQ, TWO, DC, RM>(m, f, p, s, wq,
                                                    (DC >= 0 && !TWO) ? 0 : aux, step_index,
                                                    stats, err_word, z32, load_mixed_in(s, i),
                                                    i);
}

}  // namespace cg
