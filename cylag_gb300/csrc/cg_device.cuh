// cg_device.cuh -- device-side building blocks of the fused particle step.
//
// Every function restates one piece of CyLag's per-particle step (the file
// and lines are cited at each function) in the same floating-point
// expression order, so that the plain form, compiled with -fmad=false,
// rounds exactly as the reference's C does.
#pragma once

#include <climits>

#include <cstdint>
#include <cuda_runtime.h>

#include "ziggurat_tables.h"

namespace cg {

// cylag/core/constants.pyx:1-75
constexpr double EPSILON = 1.e-16;
constexpr double EPSILON_LSM2 = 1.e-8;
constexpr double EPSILON_LSM3 = 1.e-8;
constexpr double EPSILON_REBOUND = 1.e-8;
constexpr double LSM3_CLIP_STEP = 1.e-4;
constexpr double DBL_EPS = 2.220446049250313e-16;   // DBL_EPSILON
constexpr double DEG_TO_RAD = 0.017453292519943295;
constexpr double TWO_SQRT3 = 3.4641016151377544;
constexpr double GRAV = 9.80665;
constexpr double NU0 = 1.3e-6;
constexpr double C0KOLM = 1.2;
constexpr double CMU = 0.09;
constexpr double KAPPA = 0.41;
constexpr int BND_WALL_REF = 0;
constexpr int BND_OPEN_REF = 1;
constexpr int PART_LOC_O = -1;
constexpr int PART_LOC_B = -2;
constexpr int PART_LOC_A = -3;
constexpr int NITER_MAX = 50;            // xylocalizer.pyx:362
constexpr int RNG_MAX_TRIES = 1 << 16;   // bound on every rejection loop

// error flags (mirror CG_ERR_* in cylag_gpu.h)
constexpr uint32_t ERR_INTERP_OUTSIDE = 1;
constexpr uint32_t ERR_DEGENERATE_LAYER = 2;
constexpr uint32_t ERR_RNG_LIMIT = 4;
constexpr uint32_t ERR_UNSUPPORTED = 8;
constexpr uint32_t ERR_NONFINITE = 16;   // LSM2/LSM3 coefficients the reference rejects
constexpr uint32_t ERR_BOUNDS = 32;      // bounds-checked builds: a gather index out of range

// ---------------------------------------------------------------------------
// device views
// ---------------------------------------------------------------------------
struct DevMesh {
    int nv, nt, ne;
    const double2* __restrict__ xy;     // [nv]
    // [6*nt]: vertices a, b, c, then edge vectors b-a, c-b, a-c (FP64,
    // computed on the host with the same subtractions the reference's
    // point-in-triangle test performs, utils.pyx:332-385)
    const double2* __restrict__ geo;
    // [2*nt] FP32 P1 gradients {gx0,gx1,gx2,gy0}, {gy1,gy2,-,-} (mixed form)
    const float4* __restrict__ g32;
    // [4*nt] packed 64-byte record per triangle for the mixed form:
    // {v0, v1, v2, e0} | {xa, ya} (FP64) | {gx0, gx1, gx2, gy0} | {gy1, gy2, e1, e2}
    const int4* __restrict__ t64;
    // [4*nt] the same with {xa_hi, ya_hi, xa_lo, ya_lo} (FP32 pairs) as the
    // second quarter and the three neighbours in place of the edge ids
    // (split working positions, Tri32S)
    const int4* __restrict__ t64s;
    const int4* __restrict__ tv;        // [2*nt]: {v0,v1,v2,e0}, {e1,e2,-,-}
    const double2* __restrict__ basis;  // [5*nt]: det0..2, gx0..2, gy0..2, pad
    const int4* __restrict__ edge;      // [ne]: {n0, n1, t0, t1}
    // [nt]: the triangle across the edge opposite each vertex {n0, n1, n2, -}
    // (-1: boundary edge)
    const int4* __restrict__ nbr;
    const int* __restrict__ elabel;     // [ne]
    // [8*nt] walk record per element (WalkRec): what one hop of the mixed
    // form's path walk reads, in one 128-byte line instead of the element
    // row, three edge records and six vertices
    const int4* __restrict__ wrec;
    double gx0, gy0, ginv;
    int gnx, gny;
    const int* __restrict__ gstart;     // [gnx*gny+1]
    const int* __restrict__ gtris;
    // bounds-checked builds (CG_DEBUG_BOUNDS): error word for out-of-range
    // gather indices (ERR_BOUNDS); unused otherwise
    uint32_t* dbg;
};

// Every index read from the mesh tables or the particle state goes through
// CG_IDX(m, i, n) before it addresses an array of n entries.  Normal builds:
// the index as it is.  Bounds-checked builds (-DCG_DEBUG_BOUNDS, selected by
// CYLAG_DEBUG_BOUNDS=1 at load time): an index outside [0, n) sets
// ERR_BOUNDS in m.dbg and is replaced by 0, so the access stays in bounds
// and the run reports the error instead of faulting.
#ifdef CG_DEBUG_BOUNDS
__device__ __forceinline__ long long cg_checked_index(uint32_t* dbg, long long i, long long n) {
    if ((unsigned long long)i < (unsigned long long)n) return i;
    if (dbg) atomicOr(dbg, ERR_BOUNDS);
    return 0;
}
#define CG_IDX(m, i, n) cg_checked_index((m).dbg, (long long)(i), (long long)(n))
#else
#define CG_IDX(m, i, n) (i)
#endif

// Time-interpolated node fields for one step, packed per node.
// 2D: 4 values {ux, uy, K, zs};  3D: 8 values {zs, ux, uy, uz, K, -, -, -}
// where K = (Cmu/sigc) k^2 / max(eps, EPSILON) is the nodal k-epsilon
// diffusivity (eulerian_field_set.pyx:1995-1997), exactly what the
// reference evaluates per node inside _interpolate_diffusivity_gradient_c.
// prev: the record of the previous time interpolation (the Eulerian time
// derivative of the LSM2/LSM3 acceleration, valid when prev_valid).
// turb: {k, eps} per node, time-interpolated, for the LSM2/LSM3 k-epsilon
// diffusion (nullptr when the run does not need them).
template <typename FT>
struct DevFields {
    const FT* __restrict__ cur;
    const FT* __restrict__ prev;
    int npoints, nlayers, dim;
    int prev_valid;
    const FT* __restrict__ turb;   // [nnodes][2]
};

// one stranded particle (compute_bc.pyx:109-121): its position when it
// stranded, with the step and the particle's index, which order the records
// as the reference's particle loop appends them
struct StrandRec {
    int step, index;
    double x, y, z;
};

// a control section's segment {x0, y0, x1, y1}
struct SectionSeg {
    double x0, y0, x1, y1;
};

struct DevParams {
    int model, time_scheme, rng_method, diffmod;
    int bc_on, bc_type, max_rebounds, bnd_statistics, nopen;
    int pdim;
    double dt, sqrtdt, nux, nuz;
    double diffx_const, diffz_const;     // sqrt(2 nu) * sqrt(dt)
    double damp, strand, roughness;
    double buoy_wb;                      // constant buoyancy velocity (model 0)
    int buoy_model;
    double density, rho0, drag_coef;
    // LSM2 / LSM3: particle coefficients (lagrangian_particle_set.pyx:355-375)
    // and model options (parameters.pyx)
    // FP32 copies for the mixed form (no per-particle conversions)
    float dt32, sqrtdt32, diffx32;
    int added_mass, drag_model, nuopt, edge_opt;
    double a0c, a1c, a2c, a3c;
    double tl_h, tl_v;               // diffusion_lsm3_tl_horizontal / _vertical
    // control sections: one segment {x0, y0, x1, y1} each; their per-step
    // counts follow the nopen exit counts in a step's statistics row
    int ncsec;
    const SectionSeg* csec;
    // stranding output: records of this call's stranded particles
    int strand_cap;
    int* strand_count;
    StrandRec* strand_rec;
    // the field set's friction law (pseudo-3D log-law correction,
    // eulerian_field_set.pyx:1957-1993)
    int friction_model;
    double friction_coef;
    // FP32 copies of the LSM2/LSM3 coefficients for the mixed form
    float a0c32, a1c32, a2c32, nux32, nuz32, tl_h32, tl_v32, drag_coef32;
};

// a parameter in the arithmetic R: its FP64 value, or (R = float) its FP32
// copy, which equals R(v) without a conversion per particle
template <typename R>
__device__ __forceinline__ R par(double v, float v32) {
    if constexpr (sizeof(R) == sizeof(float)) return v32;
    else return v;
}

// x**y (x > 0) as the compiled reference evaluates it: Cython gives
// double ** double a complex result, computed by the C library's complex
// power exp(y * log x) through the complex logarithm, whose real part is
// log1p((x-1)(x+1))/2 for 0.5 <= x < 2 and log(x) elsewhere.
template <typename R>
__device__ __forceinline__ R cpow_re(R x, R y) {
    R L = (x >= R(0.5) && x < R(2.)) ? log1p((x - R(1.)) * (x + R(1.))) / R(2.) : log(x);
    return exp(y * L);
}

__device__ __forceinline__ void record_strand(const DevParams& p, int step, int index, double x,
                                              double y, double z) {
    if (p.strand_rec == nullptr) return;
    const int k = atomicAdd(p.strand_count, 1);
    if (k < p.strand_cap) p.strand_rec[k] = StrandRec{step, index, x, y, z};
}

struct DevState {
    int n;
    double* __restrict__ pos;
    double* __restrict__ vel;
    double* __restrict__ fvs;
    double* __restrict__ last_pos;
    double* __restrict__ last_vel;
    int* __restrict__ tri;
    int* __restrict__ last_tri;
    int* __restrict__ lowerlayer;
    int* __restrict__ tag;
    double* __restrict__ diameter;
    uint64_t* __restrict__ rng;
    double* __restrict__ depth;   // depth below the free surface (compute_depth) or nullptr
    // sorted runs: pos/tri/tag/rng are working copies in sorted order and
    // slot[i] is the caller's index of working particle i, where the
    // remaining arrays live, except those flagged in `work` (W_*), which are
    // working copies too (indexed by i)
    const int* __restrict__ slot;
    int work;
    int base;   // index of entry 0 in the whole pool (a chunk of it: its offset)
};

constexpr int W_VEL = 1, W_FVS = 2, W_LAYER = 4, W_DIAM = 8;
// working positions held as float4 {x_hi, y_hi, x_lo, y_lo}, the unevaluated
// sums x_hi + x_lo (mixed LSM1 2D step over sorted working copies)
constexpr int W_SPLIT = 16;
// the step's outputs that no later step reads -- last_position,
// last_velocity, last_tri and (unless W_FVS carries it) the fluid velocity
// seen -- are written to working arrays in element order instead of the
// caller's slots.  A re-sort does not move them: each working last_tri is
// reset to LAST_UNSET there (or kept at -1, a deletion, whose outputs are
// zero), and only entries set since are written back.  Every call ends with
// a step that sets them for each active particle.
constexpr int W_AUXW = 32;
constexpr int LAST_UNSET = INT_MIN;
// mixed LSM2/LSM3: the working velocities (W_VEL) and, with W_FVS, the
// working fluid velocities seen are FP32 -- the values the mixed step
// computes in FP32 and rounds every velocity it stores to
constexpr int W_V32 = 64;
// mixed LSM2/LSM3 3D direct integrators: working positions as an FP32 pair
// hi + lo per coordinate, {x_hi, x_lo, y_hi, y_lo, z_hi, z_lo} in the
// 24-byte row of the FP64 position
constexpr int W_SPLIT3 = 128;
// LSM1 runs (the velocity is an output, U(x0), equal to the fluid velocity
// seen): two working velocity arrays that the steps writing the velocity
// alternate between, so that the other one holds the last velocity.  A
// step writes its velocity into DevState::vel only; the write-back gives
// velocity and fluid velocity seen from the newest array, last_velocity
// from the other (no per-particle copies of the last velocity, no second
// write of the same velocity).
constexpr int W_VEL2 = 256;

// component k of the particle velocity / fluid velocity seen of a state
// whose working copies may be FP32 (W_V32); the caller's arrays are FP64
__device__ __forceinline__ double vel_ld(const DevState& s, size_t k) {
    return (s.work & W_V32) ? (double)reinterpret_cast<const float*>(s.vel)[k] : s.vel[k];
}
__device__ __forceinline__ void vel_st(const DevState& s, size_t k, double v) {
    if (s.work & W_V32) reinterpret_cast<float*>(s.vel)[k] = (float)v;
    else s.vel[k] = v;
}
__device__ __forceinline__ bool fvs_is32(const DevState& s) {
    return (s.work & (W_V32 | W_FVS)) == (W_V32 | W_FVS);
}
__device__ __forceinline__ double fvs_ld(const DevState& s, size_t k) {
    return fvs_is32(s) ? (double)reinterpret_cast<const float*>(s.fvs)[k] : s.fvs[k];
}
__device__ __forceinline__ void fvs_st(const DevState& s, size_t k, double v) {
    if (fvs_is32(s)) reinterpret_cast<float*>(s.fvs)[k] = (float)v;
    else s.fvs[k] = v;
}

// An FP64 position as a pair of FP32 values hi + lo (|lo| <= ulp(hi)/2):
// 48 significant bits, so the step's arithmetic on it stays in FP32.
__device__ __forceinline__ float4 split_pos(double x, double y) {
    const float hx = (float)x, hy = (float)y;
    return make_float4(hx, hy, (float)(x - (double)hx), (float)(y - (double)hy));
}

// one coordinate as an FP32 pair hi + lo (|lo| <= ulp(hi)/2), and back
__device__ __forceinline__ float2 split1(double v) {
    const float h = (float)v;
    return make_float2(h, (float)(v - (double)h));
}
__device__ __forceinline__ double join1(float2 p) { return (double)p.x + (double)p.y; }

// the FP64 value of a split position (rounded to nearest double)
__device__ __forceinline__ double2 join_pos(float4 p) {
    return make_double2((double)p.x + (double)p.z, (double)p.y + (double)p.w);
}

// hi + lo + d as a new normalized pair: TwoSum(hi, d) (Knuth), the low
// parts added, then Fast2Sum; the result is within about ulp(lo) of the
// exact sum.  No multiplications, so no contraction can change it.
__device__ __forceinline__ void split_add1(float& hi, float& lo, float d) {
    const float s = hi + d;
    const float bb = s - hi;
    const float e = (hi - (s - bb)) + (d - bb);
    const float t = e + lo;
    hi = s + t;
    lo = t - (hi - s);
}

__device__ __forceinline__ float4 split_add(float4 p, float dx, float dy) {
    split_add1(p.x, p.z, dx);
    split_add1(p.y, p.w, dy);
    return p;
}

// index of particle i in an array that is a working copy when `flag` is set
__device__ __forceinline__ int widx(const DevState& s, int i, int a, int flag) {
    return (s.work & flag) ? i : a;
}

__device__ __forceinline__ int aux_index(const DevState& s, int i) {
    return s.slot ? __ldg(&s.slot[i]) : i;
}

// Particles that leave their start triangle are finished by a second kernel
// (path walk + boundary conditions) from a compacted queue, so that the
// walk's FP64 work runs with full warps instead of inside divergent ones.
struct WalkEntry {
    double xn, yn;       // end-of-step position (before localization)
    uint64_t rng;        // PCG32 state after the step's draws
    int i;               // particle index
    int tri0;            // element at the step's start
};

struct WalkQueue {
    int* count;          // entries this step (zero when the step starts)
    WalkEntry* e;        // capacity: one entry per particle
    // a run's steps alternate between two counters: the step kernel zeroes
    // the other one here for the next step (nullptr: nothing to zero)
    int* reset;
};

// block 0 of a step kernel that fills the walk queue: the next step's
// counter (the previous step's, whose walk has finished) back to zero
__device__ __forceinline__ void reset_next_queue(const WalkQueue& wq) {
    if (wq.reset != nullptr && blockIdx.x == 0 && threadIdx.x == 0) *wq.reset = 0;
}

// warp-aggregated slot reservation
__device__ __forceinline__ int queue_slot(const WalkQueue& q) {
    unsigned mask = __activemask();
    int lane = threadIdx.x & 31;
    int leader = __ffs(mask) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(q.count, __popc(mask));
    base = __shfl_sync(mask, base, leader);
    return base + __popc(mask & ((1u << lane) - 1u));
}

// ---------------------------------------------------------------------------
// PCG32 + normal variates (cylag/lsm/random_utils.pyx)
// ---------------------------------------------------------------------------
struct Rng {
    uint64_t state, inc;
    uint32_t err;
};

struct ZigTables {
    uint32_t kn[128];
    double wn[128];
    double fn[128];
};

// random_utils.pyx:22-28
__device__ __forceinline__ uint32_t pcg_next(Rng& r) {
    uint64_t old = r.state;
    r.state = old * 6364136223846793005ULL + r.inc;
    uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
    uint32_t rot = (uint32_t)(old >> 59);
    return (xs >> rot) | (xs << ((32u - rot) & 31u));
}

// random_utils.pyx:30-37
__host__ __device__ inline void pcg_seed(uint64_t seed, uint64_t stream, uint64_t& state,
                                         uint64_t& inc) {
    uint64_t m = 6364136223846793005ULL;
    inc = (stream << 1) | 1ULL;
    state = 0ULL * m + inc;
    state += seed;
    state = state * m + inc;
}

// random_utils.pyx:55-67
__device__ __forceinline__ double rng_uniform(Rng& r) {
    uint32_t u = pcg_next(r);
    return u * (1.0 / 4294967296.0);
}

// random_utils.pyx:154-194
__device__ inline double rng_ziggurat(Rng& r, const ZigTables& z) {
    for (int tries = 0; tries < RNG_MAX_TRIES; ++tries) {
        int32_t hz = (int32_t)pcg_next(r);
        uint32_t iz = (uint32_t)hz & 127u;
        uint32_t ahz = hz < 0 ? 0u - (uint32_t)hz : (uint32_t)hz;  // c_abs(INT_MIN) == INT_MIN
        if (ahz < z.kn[iz]) return hz * z.wn[iz];
        if (iz == 0) {
            for (int t2 = 0; t2 < RNG_MAX_TRIES; ++t2) {
                double x = -log(rng_uniform(r)) * 0.2904764;
                double y = -log(rng_uniform(r));
                if (y + y >= x * x) return hz > 0 ? 3.442619855899 + x : -3.442619855899 - x;
            }
            r.err |= ERR_RNG_LIMIT;
            return 0.0;
        }
        double x = hz * z.wn[iz];
        if (z.fn[iz] + rng_uniform(r) * (z.fn[iz - 1] - z.fn[iz]) < exp(-0.5 * x * x)) return x;
    }
    r.err |= ERR_RNG_LIMIT;
    return 0.0;
}

// random_utils.pyx:72-108 (pair == true returns both coordinates)
__device__ inline void rng_polar(Rng& r, double& a, double& b) {
    double x1 = 0., x2 = 0., w = 2.0;
    int tries = 0;
    while ((w >= 1.0 || w == 0.0) && tries < RNG_MAX_TRIES) {
        x1 = 2.0 * rng_uniform(r) - 1.0;
        x2 = 2.0 * rng_uniform(r) - 1.0;
        w = x1 * x1 + x2 * x2;
        ++tries;
    }
    if (tries == RNG_MAX_TRIES) { r.err |= ERR_RNG_LIMIT; a = b = 0.; return; }
    w = sqrt((-2.0 * log(w)) / w);
    a = x1 * w;
    b = x2 * w;
}

// random_utils.pyx:202-233
__device__ inline void rng_pair(Rng& r, int method, const ZigTables& z, double& a, double& b) {
    if (method == 1) {
        a = (rng_uniform(r) - 0.5) * TWO_SQRT3;
        b = (rng_uniform(r) - 0.5) * TWO_SQRT3;
    } else if (method == 2) {
        a = rng_ziggurat(r, z);
        b = rng_ziggurat(r, z);
    } else {
        rng_polar(r, a, b);
    }
}

// random_utils.pyx:235-263
__device__ inline double rng_single(Rng& r, int method, const ZigTables& z) {
    if (method == 1) return (rng_uniform(r) - 0.5) * TWO_SQRT3;
    if (method == 2) return rng_ziggurat(r, z);
    double a, b;
    rng_polar(r, a, b);
    return a;
}

// FP32 samplers of the mixed form (tables in shared memory)
struct Zig32 {
    uint32_t kn[128];
    float wn[128];
    float fn[128];
};

// random_utils.pyx:55-67 in FP32
// (explicitly rounded operations here and below: every compiled form of a
// step draws the same values)
__device__ __forceinline__ float uniform32(Rng& r) {
    return __fmul_rn((float)pcg_next(r), 2.3283064365386963e-10f);
}

// random_utils.pyx:154-194 in FP32 (same stream consumption as the FP64
// version except where an FP32 wedge/tail test rounds the other way)
__device__ inline float zig32(Rng& r, const Zig32& z) {
    for (int tries = 0; tries < RNG_MAX_TRIES; ++tries) {
        int32_t hz = (int32_t)pcg_next(r);
        uint32_t iz = (uint32_t)hz & 127u;
        uint32_t ahz = hz < 0 ? 0u - (uint32_t)hz : (uint32_t)hz;
        if (ahz < z.kn[iz]) return __fmul_rn((float)hz, z.wn[iz]);
        if (iz == 0) {
            for (int t2 = 0; t2 < RNG_MAX_TRIES; ++t2) {
                float x = __fmul_rn(-__logf(uniform32(r)), 0.2904764f);
                float y = -__logf(uniform32(r));
                if (__fadd_rn(y, y) >= __fmul_rn(x, x))
                    return hz > 0 ? __fadd_rn(3.442619855899f, x) : __fsub_rn(-3.442619855899f, x);
            }
            r.err |= ERR_RNG_LIMIT;
            return 0.f;
        }
        float x = __fmul_rn((float)hz, z.wn[iz]);
        if (__fmaf_rn(uniform32(r), __fsub_rn(z.fn[iz - 1], z.fn[iz]), z.fn[iz]) <
            __expf(__fmul_rn(__fmul_rn(-0.5f, x), x)))
            return x;
    }
    r.err |= ERR_RNG_LIMIT;
    return 0.f;
}

__device__ inline void polar32(Rng& r, float& a, float& b) {
    float x1 = 0.f, x2 = 0.f, w = 2.f;
    int tries = 0;
    while ((w >= 1.f || w == 0.f) && tries < RNG_MAX_TRIES) {
        x1 = __fmaf_rn(2.f, uniform32(r), -1.f);
        x2 = __fmaf_rn(2.f, uniform32(r), -1.f);
        w = __fmaf_rn(x2, x2, __fmul_rn(x1, x1));
        ++tries;
    }
    if (tries == RNG_MAX_TRIES) { r.err |= ERR_RNG_LIMIT; a = b = 0.f; return; }
    w = sqrtf(__fdiv_rn(__fmul_rn(-2.f, __logf(w)), w));
    a = __fmul_rn(x1, w);
    b = __fmul_rn(x2, w);
}

__device__ inline void pair32(Rng& r, int method, const Zig32& z, float& a, float& b) {
    if (method == 1) {
        a = __fmul_rn(__fsub_rn(uniform32(r), 0.5f), (float)TWO_SQRT3);
        b = __fmul_rn(__fsub_rn(uniform32(r), 0.5f), (float)TWO_SQRT3);
    } else if (method == 2) {
        a = zig32(r, z);
        b = zig32(r, z);
    } else {
        polar32(r, a, b);
    }
}

// Outlined draws for the large LSM2/LSM3 integrators: one copy of the
// sampler per kernel instead of one per call site (their per-dimension
// loops are unrolled), which keeps their instruction footprint down.  The
// stream state goes in and out by value, so no particle state needs an
// address (it stays in registers).
template <typename T>
struct DrawOut {
    uint64_t state;
    uint32_t err;
    T a, b;
};

static __device__ __noinline__ DrawOut<double> rng_draws_ol(uint64_t st, uint64_t inc, int method,
                                                           const ZigTables& z, int two) {
    Rng r{st, inc, 0};
    DrawOut<double> o;
    o.b = 0.;
    if (two) rng_pair(r, method, z, o.a, o.b);
    else o.a = rng_single(r, method, z);
    o.state = r.state;
    o.err = r.err;
    return o;
}

static __device__ __noinline__ DrawOut<float> draws32_ol(uint64_t st, uint64_t inc, int method,
                                                        const Zig32& z, int two) {
    Rng r{st, inc, 0};
    DrawOut<float> o;
    o.b = 0.f;
    if (two) {
        pair32(r, method, z, o.a, o.b);
    } else if (method == 1) {
        o.a = __fmul_rn(__fsub_rn(uniform32(r), 0.5f), (float)TWO_SQRT3);
    } else if (method == 2) {
        o.a = zig32(r, z);
    } else {
        float b;
        polar32(r, o.a, b);
    }
    o.state = r.state;
    o.err = r.err;
    return o;
}

__device__ __forceinline__ void rng_pair_ol(Rng& r, int method, const ZigTables& z, double& a,
                                            double& b) {
    const DrawOut<double> o = rng_draws_ol(r.state, r.inc, method, z, 1);
    r.state = o.state;
    r.err |= o.err;
    a = o.a;
    b = o.b;
}
__device__ __forceinline__ double rng_single_ol(Rng& r, int method, const ZigTables& z) {
    const DrawOut<double> o = rng_draws_ol(r.state, r.inc, method, z, 0);
    r.state = o.state;
    r.err |= o.err;
    return o.a;
}
__device__ __forceinline__ void pair32_ol(Rng& r, int method, const Zig32& z, float& a, float& b) {
    const DrawOut<float> o = draws32_ol(r.state, r.inc, method, z, 1);
    r.state = o.state;
    r.err |= o.err;
    a = o.a;
    b = o.b;
}
__device__ __forceinline__ float single32_ol(Rng& r, int method, const Zig32& z) {
    const DrawOut<float> o = draws32_ol(r.state, r.inc, method, z, 0);
    r.state = o.state;
    r.err |= o.err;
    return o.a;
}

// ---------------------------------------------------------------------------
// geometry (cylag/geom/utils.pyx, intersections.pyx, xylocalizer.pyx)
// ---------------------------------------------------------------------------

// utils.pyx:332-361
__device__ __forceinline__ double pintri(double x, double y, double xa, double ya, double xb,
                                         double yb, double xc, double yc) {
    return ((xb - xa) * (y - ya) - (x - xa) * (yb - ya)) *
           ((x - xa) * (yc - ya) - (xc - xa) * (y - ya));
}

// Decision of (t1 * t2 >= 0) taken on the sign bits (integer pipe) instead
// of an FP64 multiply and compare.  Identical for every finite t1, t2 whose
// product is not subnormal; a subnormal product needs cross products below
// ~1e-154, i.e. coordinates below ~1e-77 m.
__device__ __forceinline__ bool prod_nonneg(double t1, double t2) {
    long long b1 = __double_as_longlong(t1), b2 = __double_as_longlong(t2);
    const long long EXP = 0x7ff0000000000000LL, ABS = 0x7fffffffffffffffLL;
    bool nan = ((b1 & ABS) > EXP) || ((b2 & ABS) > EXP);
    bool zero = ((b1 << 1) == 0) || ((b2 << 1) == 0);
    return !nan && (zero || (b1 ^ b2) >= 0);
}

// One rotation of point_in_triangle_dotp (utils.pyx:363-385): with w = p - v,
// t1 = eo x w, t2 = ei x w for the edge leaving v (eo) and entering v (ei).
// Exactly the reference's pintri(x, y, v, next, prev): (next - v) is eo and
// (prev - v) == -ei bit for bit, and negated operands give negated products.
// Written with _rn intrinsics so that no build flag can contract it to FMA.
__device__ __forceinline__ bool rot_ok(double x, double y, double2 v, double2 eo, double2 ei) {
    double wx = __dsub_rn(x, v.x), wy = __dsub_rn(y, v.y);
    double t1 = __dsub_rn(__dmul_rn(eo.x, wy), __dmul_rn(wx, eo.y));
    double t2 = __dsub_rn(__dmul_rn(ei.x, wy), __dmul_rn(wx, ei.y));
    return prod_nonneg(t1, t2);
}

// utils.pyx:363-385 with xylocalizer.pyx:126-167
__device__ __forceinline__ bool in_tri(const DevMesh& m, int k, double x, double y) {
    const double2* g = m.geo + 6 * (size_t)CG_IDX(m, k, m.nt);
    double2 a = __ldg(&g[0]), b = __ldg(&g[1]), c = __ldg(&g[2]);
    double2 dab = __ldg(&g[3]), dbc = __ldg(&g[4]), dca = __ldg(&g[5]);
    return rot_ok(x, y, a, dab, dca) && rot_ok(x, y, b, dbc, dab) && rot_ok(x, y, c, dca, dbc);
}

// utils.pyx:228-252
__device__ __forceinline__ int orientation(double v0x, double v0y, double v1x, double v1y,
                                           double v2x, double v2y) {
    double delta = __dsub_rn(__dmul_rn(__dsub_rn(v0y, v1y), __dsub_rn(v2x, v0x)),
                             __dmul_rn(__dsub_rn(v0x, v1x), __dsub_rn(v2y, v0y)));
    if (delta == 0.) return 0;
    if (delta > 0.) return 1;
    return 2;
}

// utils.pyx:282-303
__device__ __forceinline__ bool on_segment(double v0x, double v0y, double v1x, double v1y,
                                           double v2x, double v2y) {
    return v2x <= fmax(v1x, v0x) && v2x >= fmin(v1x, v0x) && v2y <= fmax(v1y, v0y) &&
           v2y >= fmin(v1y, v0y);
}

// intersections.pyx:106-148
__device__ inline bool intersec2d(double p0x, double p0y, double p1x, double p1y, double s0x,
                                  double s0y, double s1x, double s1y) {
    int o1 = orientation(p0x, p0y, p1x, p1y, s0x, s0y);
    int o2 = orientation(p0x, p0y, p1x, p1y, s1x, s1y);
    int o3 = orientation(s0x, s0y, s1x, s1y, p0x, p0y);
    int o4 = orientation(s0x, s0y, s1x, s1y, p1x, p1y);
    if (o1 != o2 && o3 != o4) return true;
    if (o1 == 0 && on_segment(p0x, p0y, p1x, p1y, s0x, s0y)) return true;
    if (o2 == 0 && on_segment(p0x, p0y, p1x, p1y, s1x, s1y)) return true;
    if (o3 == 0 && on_segment(s0x, s0y, s1x, s1y, p0x, p0y)) return true;
    if (o4 == 0 && on_segment(s0x, s0y, s1x, s1y, p1x, p1y)) return true;
    return false;
}

// Control sections (solver.pyx:542-549, control_shapes.pyx:74-101,
// intersections.pyx:150-192): once a particle's step is over, each section
// whose segment meets the step's segment (step-start position -> final
// position; both (0, 0) when the step deleted the particle, as the reference
// tests the zeroed arrays) counts it once.  The reference's ControlSection
// tests only its first segment (nseg = poly.shape[1] - 1 = 1), so a section
// is that one segment here.  stats: the step's row, max(1, nopen) exit
// counts then the sections'.
__device__ __forceinline__ void count_sections(const DevParams& p, int* stats, double x0,
                                               double y0, double x1, double y1) {
    if (p.ncsec == 0 || stats == nullptr) return;
    int* row = stats + (p.nopen > 0 ? p.nopen : 1);
    for (int c = 0; c < p.ncsec; ++c) {
        const SectionSeg g = p.csec[c];
        if (intersec2d(x0, y0, x1, y1, g.x0, g.y0, g.x1, g.y1)) atomicAdd(&row[c], 1);
    }
}

// Global point location: first triangle (lowest id) in the point's grid
// bucket that contains it.  Stands in for the KD-tree fallback of
// xylocalizer.pyx:200-286; same result unless the point lies exactly on an
// edge shared by two triangles.
__device__ inline int grid_locate(const DevMesh& m, double x, double y) {
    double fx = floor(__dmul_rn(__dsub_rn(x, m.gx0), m.ginv));
    double fy = floor(__dmul_rn(__dsub_rn(y, m.gy0), m.ginv));
    if (!(fx >= 0.)) fx = 0.;
    if (!(fy >= 0.)) fy = 0.;
    int cx = fx > (double)(m.gnx - 1) ? m.gnx - 1 : (int)fx;
    int cy = fy > (double)(m.gny - 1) ? m.gny - 1 : (int)fy;
    int c = cy * m.gnx + cx;
    c = (int)CG_IDX(m, c, (long long)m.gnx * m.gny);
    int b = __ldg(&m.gstart[c]), e = __ldg(&m.gstart[c + 1]);
    for (int j = b; j < e; ++j) {
        int k = __ldg(&m.gtris[j]);
        if (in_tri(m, k, x, y)) return k;
    }
    return -1;
}

// The walk record of element k (DevMesh::wrec, 8 x 16 bytes): vertices a,
// b, c (FP64, the element's vertex order), its FP32 P1 gradients as in
// Tri32, the ids of its three edges in the element's edge order, the two
// elements of each edge as the edge table holds them, and each edge's end
// points as local vertex indices (2 bits each: first end, second end).
struct WalkRec {
    double2 a, b, c;
    float4 g0, g1;    // {gx0, gx1, gx2, gy0}, {gy1, gy2, -, -}
    int e0, e1, e2;
    int z0, w0, z1, w1, z2, w2;
    int order;
};

__device__ __forceinline__ double2 bits_double2(int4 w) {
    return make_double2(__hiloint2double(w.y, w.x), __hiloint2double(w.w, w.z));
}

__device__ __forceinline__ WalkRec load_walkrec(const DevMesh& m, int k) {
    const int4* r = m.wrec + 8 * (size_t)CG_IDX(m, k, m.nt);
    const int4 w0 = __ldg(&r[0]), w1 = __ldg(&r[1]), w2 = __ldg(&r[2]), w3 = __ldg(&r[3]);
    const int4 w4 = __ldg(&r[4]), w5 = __ldg(&r[5]), w6 = __ldg(&r[6]);
    WalkRec t;
    t.a = bits_double2(w0);
    t.b = bits_double2(w1);
    t.c = bits_double2(w2);
    t.g0 = make_float4(__int_as_float(w3.x), __int_as_float(w3.y), __int_as_float(w3.z),
                       __int_as_float(w3.w));
    t.g1 = make_float4(__int_as_float(w4.x), __int_as_float(w4.y), 0.f, 0.f);
    t.e0 = w4.z; t.e1 = w4.w; t.e2 = w5.x;
    t.z0 = w5.y; t.w0 = w5.z; t.z1 = w5.w;
    t.w1 = w6.x; t.z2 = w6.y; t.w2 = w6.z;
    t.order = w6.w;
    return t;
}

__device__ __forceinline__ double2 rec_vertex(const WalkRec& t, int l) {
    return l == 0 ? t.a : (l == 1 ? t.b : t.c);
}

// edge slot i of the record: id, end points (the edge table's order) and
// the element across it from k (the edge table's test, so that k == -1
// behaves as in the reference)
__device__ __forceinline__ void rec_edge(const WalkRec& t, int i, int k, int& j, double2& ea,
                                         double2& eb, int& kn) {
    const int ez = i == 0 ? t.z0 : (i == 1 ? t.z1 : t.z2);
    const int ew = i == 0 ? t.w0 : (i == 1 ? t.w1 : t.w2);
    j = i == 0 ? t.e0 : (i == 1 ? t.e1 : t.e2);
    ea = rec_vertex(t, (t.order >> (4 * i)) & 3);
    eb = rec_vertex(t, (t.order >> (4 * i + 2)) & 3);
    kn = ez == k ? ew : ez;
}

// in_tri from the record: the same vertices and edge vectors (b - a, c - b,
// a - c, formed with the host's FP64 subtractions) as DevMesh::geo
__device__ __forceinline__ bool in_tri_rec(const WalkRec& t, double x, double y) {
    const double2 dab = make_double2(__dsub_rn(t.b.x, t.a.x), __dsub_rn(t.b.y, t.a.y));
    const double2 dbc = make_double2(__dsub_rn(t.c.x, t.b.x), __dsub_rn(t.c.y, t.b.y));
    const double2 dca = make_double2(__dsub_rn(t.a.x, t.c.x), __dsub_rn(t.a.y, t.c.y));
    return rot_ok(x, y, t.a, dab, dca) && rot_ok(x, y, t.b, dbc, dab) &&
           rot_ok(x, y, t.c, dca, dbc);
}

// The three edge records of a triangle and their end points, issued
// together: a hop of the walk then waits for two dependent loads instead of
// two per edge tested.  Every id is a valid edge of the mesh (the intersected
// edge too, loaded and not tested).
__device__ __forceinline__ void walk_gather(const DevMesh& m, const int* ed, int4* er,
                                            double2* va, double2* vb) {
#pragma unroll
    for (int i = 0; i < 3; ++i) er[i] = __ldg(&m.edge[CG_IDX(m, ed[i], m.ne)]);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        va[i] = __ldg(&m.xy[CG_IDX(m, er[i].x, m.nv)]);
        vb[i] = __ldg(&m.xy[CG_IDX(m, er[i].y, m.nv)]);
    }
}

// xylocalizer.pyx:338-435
__device__ inline void path_walk(const DevMesh& m, int k, double p0x, double p0y, double x,
                                 double y, int& new_k, int& bnd) {
    int intersected_edge = -1;
    for (int niter = 0; niter <= NITER_MAX; ++niter) {
        // k == -1 (an element index set to "outside" by a Runge-Kutta stage
        // that left the mesh): the reference reads the last triangle's row
        // (numpy wraparound) but compares with -1
        int row = k < 0 ? k + m.nt : k;
        if (row < 0) break;
        row = (int)CG_IDX(m, row, m.nt);
        int4 ta = __ldg(&m.tv[2 * row]);
        int4 tb = __ldg(&m.tv[2 * row + 1]);
        int ed[3] = {ta.w, tb.x, tb.y};
        // the three edges and their end points are loaded together (two
        // dependent levels per hop), then tested in the reference's order
        int4 er[3];
        double2 va[3], vb[3];
        walk_gather(m, ed, er, va, vb);
        bool intersects = false;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            int j = ed[i];
            if (j == intersected_edge) continue;
            const int4 e = er[i];
            const double2 a = va[i], b = vb[i];
            if (intersec2d(p0x, p0y, x, y, a.x, a.y, b.x, b.y)) {
                intersects = true;
                int kn = (e.z == k) ? e.w : e.z;
                if (kn == -1) { new_k = -1; bnd = j; return; }
                if (in_tri(m, kn, x, y)) { new_k = kn; bnd = -1; return; }
                k = kn;
                intersected_edge = j;
                break;
            }
        }
        if (!intersects) {
            new_k = (k >= 0 && in_tri(m, k, x, y)) ? k : -1;
            bnd = -1;
            return;
        }
    }
    new_k = -1;
    bnd = -1;
}

// ---- FP32-filtered walk (mixed form) --------------------------------------
// Orientation of (a, b, c) from FP32 offsets to a common origin, with a
// bound on its rounding error; `certain` is false inside the bound.  Offsets
// are rounded FP64 differences (relative error <= 2^-24 each), so the
// computed value differs from the exact one by at most ~48 eps32 M^2, M the
// largest offset magnitude; the bound takes 4e-6 M^2 (~67 eps32 M^2).  Beyond
// it the exact value is nonzero with the FP32 sign, which is also the sign
// the FP64 evaluation gives.
__device__ __forceinline__ int orient32(float2 a, float2 b, float2 c, bool& certain) {
    float d = (a.y - b.y) * (c.x - a.x) - (a.x - b.x) * (c.y - a.y);
    float M = fmaxf(fmaxf(fmaxf(fabsf(a.x), fabsf(a.y)), fmaxf(fabsf(b.x), fabsf(b.y))),
                    fmaxf(fabsf(c.x), fabsf(c.y)));
    float bound = 4.0e-6f * M * M + 1.0e-30f;
    certain = fabsf(d) > bound;
    return d > 0.f ? 1 : 2;
}

// intersections.pyx:106-148 with the orientations decided in FP32 when all
// four are certain (then none is zero and the result is o1 != o2 && o3 != o4,
// exactly what the FP64 test gives); otherwise the FP64 test.
__device__ __forceinline__ bool intersec2d_filtered(float2 p1, float2 e0, float2 e1, double p0x,
                                                    double p0y, double p1x, double p1y,
                                                    double2 E0, double2 E1) {
    const float2 p0 = make_float2(0.f, 0.f);
    bool c1, c2, c3, c4;
    int o1 = orient32(p0, p1, e0, c1);
    int o2 = orient32(p0, p1, e1, c2);
    int o3 = orient32(e0, e1, p0, c3);
    int o4 = orient32(e0, e1, p1, c4);
    if (c1 && c2 && c3 && c4) return o1 != o2 && o3 != o4;
    return intersec2d(p0x, p0y, p1x, p1y, E0.x, E0.y, E1.x, E1.y);
}

// xylocalizer.pyx:27-124, method 3
__device__ inline void xy_localize(const DevMesh& m, int k, double p0x, double p0y, double x,
                                   double y, int& new_k, int& bnd) {
    bnd = -1;
    // point_in_tri with k == -1 returns -1 whether or not the point is in the
    // last triangle (xylocalizer.pyx:126-167): "not found"
    if (k >= 0 && in_tri(m, k, x, y)) { new_k = k; return; }
    path_walk(m, k, p0x, p0y, x, y, new_k, bnd);
    if (new_k == -1 && bnd == -1) new_k = grid_locate(m, x, y);
}

// zlocalizer.pyx:51-71
__device__ __forceinline__ int lower_layer_index(int nl, double zs, double zb, double z) {
    if (nl == 1) return 0;
    double hl = (zs - zb) / (nl - 1);
    if (!(hl > 0.)) return 0;
    double findex = floor((z - zb) / hl);
    if (!(findex >= 0.)) return 0;
    if (!(findex <= (double)(nl - 2))) return nl - 2;
    return (int)findex;
}

// ---------------------------------------------------------------------------
// P1 interpolation (cylag/core/eulerian_field_set.pyx)
// ---------------------------------------------------------------------------
struct P1 {
    int i0, i1, i2;
    double f0, f1, f2;
    double gx0, gx1, gx2, gy0, gy1, gy2;
};

// eulerian_field_set.pyx:1043-1052 (factors) + the vertex ids
__device__ __forceinline__ P1 p1_at(const DevMesh& m, int k, double x, double y) {
    P1 p;
    k = (int)CG_IDX(m, k, m.nt);
    int4 t = __ldg(&m.tv[2 * k]);
    p.i0 = t.x; p.i1 = t.y; p.i2 = t.z;
    double2 b0 = __ldg(&m.basis[5 * k]), b1 = __ldg(&m.basis[5 * k + 1]),
            b2 = __ldg(&m.basis[5 * k + 2]), b3 = __ldg(&m.basis[5 * k + 3]),
            b4 = __ldg(&m.basis[5 * k + 4]);
    // basis layout: det0 det1 | det2 gx0 | gx1 gx2 | gy0 gy1 | gy2 pad
    p.gx0 = b1.y; p.gx1 = b2.x; p.gx2 = b2.y;
    p.gy0 = b3.x; p.gy1 = b3.y; p.gy2 = b4.x;
    p.f0 = b0.x + x * p.gx0 + y * p.gy0;
    p.f1 = b0.y + x * p.gx1 + y * p.gy1;
    p.f2 = b1.x + x * p.gx2 + y * p.gy2;
    return p;
}

// node record accessors --------------------------------------------------------
template <int DIM> struct Slots;
template <> struct Slots<2> { static constexpr int NF = 4, UX = 0, UY = 1, K = 2, ZS = 3, UZ = -1; };
// 3D records also carry the bed elevation (BOTTOM) for 3D particles on 2D
// fields (pseudo-3D), whose records use this layout with one layer
template <> struct Slots<3> { static constexpr int NF = 8, ZS = 0, UX = 1, UY = 2, UZ = 3, K = 4, ZB = 5; };

template <int DIM, typename FT>
__device__ __forceinline__ double nodev(const FT* __restrict__ f, int node, int slot) {
    return (double)__ldg(&f[(size_t)node * Slots<DIM>::NF + slot]);
}

template <int DIM, typename FT>
__device__ __forceinline__ double p1_eval(const FT* __restrict__ f, int off, const P1& p, int slot) {
    return nodev<DIM>(f, off + p.i0, slot) * p.f0 + nodev<DIM>(f, off + p.i1, slot) * p.f1 +
           nodev<DIM>(f, off + p.i2, slot) * p.f2;
}

template <int DIM, typename FT>
__device__ __forceinline__ double p1_gx(const FT* __restrict__ f, int off, const P1& p, int slot) {
    return nodev<DIM>(f, off + p.i0, slot) * p.gx0 + nodev<DIM>(f, off + p.i1, slot) * p.gx1 +
           nodev<DIM>(f, off + p.i2, slot) * p.gx2;
}

template <int DIM, typename FT>
__device__ __forceinline__ double p1_gy(const FT* __restrict__ f, int off, const P1& p, int slot) {
    return nodev<DIM>(f, off + p.i0, slot) * p.gy0 + nodev<DIM>(f, off + p.i1, slot) * p.gy1 +
           nodev<DIM>(f, off + p.i2, slot) * p.gy2;
}

// per-triangle data of the FP32 barycentric evaluation
struct Tri32 {
    int4 tv;      // v0, v1, v2, e0
    double2 a;    // vertex a (FP64)
    float4 g0;    // gx0 gx1 gx2 gy0
    float4 g1;    // gy1 gy2 - -
};

// the same record with vertex a as a split pair {xa_hi, ya_hi, xa_lo, ya_lo}
// (DevMesh::t64s), for split working positions; in place of the edge ids it
// holds the triangles across the edges opposite vertices 0, 1, 2 (DevMesh::nbr):
// tv.w, g1.z, g1.w (as int bits)
struct Tri32S {
    int4 tv;
    float4 as;
    float4 g0;
    float4 g1;
};

__device__ __forceinline__ int tri32s_nbr(const Tri32S& t, int j) {
    return j == 0 ? t.tv.w : (j == 1 ? __float_as_int(t.g1.z) : __float_as_int(t.g1.w));
}

__device__ __forceinline__ Tri32S load_tri32s(const DevMesh& m, int k) {
    Tri32S t;
    k = (int)CG_IDX(m, k, m.nt);
    const float4* r = reinterpret_cast<const float4*>(m.t64s + 4 * (size_t)k);
    t.tv = __ldg(&m.t64s[4 * (size_t)k]);
    t.as = __ldg(&r[1]);
    t.g0 = __ldg(&r[2]);
    t.g1 = __ldg(&r[3]);
    return t;
}

// offset of a split position to the record's vertex a, in FP32:
// (x_hi - xa_hi) + (x_lo - xa_lo); within 2^-23 relative of the exact
// offset (the hi difference is exact when both are within a factor 2, as
// they are near the triangle; else one rounding), inside bary32_off's bounds
__device__ __forceinline__ float2 split_offset(const Tri32S& t, float4 p) {
    return make_float2((p.x - t.as.x) + (p.z - t.as.z), (p.y - t.as.y) + (p.w - t.as.w));
}

__device__ __forceinline__ Tri32 load_tri32(const DevMesh& m, int k) {
    Tri32 t;
    k = (int)CG_IDX(m, k, m.nt);
    const int4* r = m.t64 + 4 * (size_t)k;
    t.tv = __ldg(&r[0]);
    int4 a = __ldg(&r[1]);
    t.a = make_double2(__hiloint2double(a.y, a.x), __hiloint2double(a.w, a.z));
    int4 g0 = __ldg(&r[2]);
    t.g0 = make_float4(__int_as_float(g0.x), __int_as_float(g0.y), __int_as_float(g0.z),
                       __int_as_float(g0.w));
    int4 g1 = __ldg(&r[3]);
    t.g1 = make_float4(__int_as_float(g1.x), __int_as_float(g1.y), __int_as_float(g1.z),
                       __int_as_float(g1.w));   // z, w: edge ids e1, e2 as bits
    return t;
}

template <typename T>
__device__ __forceinline__ int tri32_edge(const T& t, int i) {
    return i == 0 ? t.tv.w : (i == 1 ? __float_as_int(t.g1.z) : __float_as_int(t.g1.w));
}

struct Bary {
    float l0, l1, l2;
    float e0, e1, e2;   // rounding bounds of l0, l1, l2
};

// barycentric coordinates from the FP32 offset (rx, ry) to vertex a:
// l_j = gx_j rx + gy_j ry.  The bounds cover the offset rounding (relative
// 2^-24), the FP32 gradients and products: <= ~4 ulp of the terms.
template <typename T>
__device__ __forceinline__ Bary bary32_off(const T& t, float rx, float ry) {
    Bary b;
    float p1 = t.g0.y * rx, q1 = t.g1.x * ry;
    float p2 = t.g0.z * rx, q2 = t.g1.y * ry;
    b.l1 = p1 + q1;
    b.l2 = p2 + q2;
    b.l0 = 1.f - b.l1 - b.l2;
    b.e1 = 6.0e-7f * (fabsf(p1) + fabsf(q1)) + 1.0e-6f;
    b.e2 = 6.0e-7f * (fabsf(p2) + fabsf(q2)) + 1.0e-6f;
    b.e0 = b.e1 + b.e2 + 1.0e-6f;
    return b;
}

// barycentric coordinates of (x, y): l_j = gx_j (x - xa) + gy_j (y - ya)
__device__ __forceinline__ Bary bary32(const Tri32& t, double x, double y) {
    return bary32_off(t, (float)(x - t.a.x), (float)(y - t.a.y));
}

// Offset of an FP64 position advanced by an FP32 increment, (x0 + d) - a,
// formed in FP32 as (x0 - a) + d: one more rounding of the start offset
// (relative 2^-24 of |x0 - a|), so the bounds get that term added.
template <typename T>
__device__ __forceinline__ Bary bary32_moved(const T& t, float rx0, float ry0, float dx,
                                             float dy) {
    Bary b = bary32_off(t, rx0 + dx, ry0 + dy);
    float s1 = 1.2e-7f * (fabsf(t.g0.y * rx0) + fabsf(t.g1.x * ry0));
    float s2 = 1.2e-7f * (fabsf(t.g0.z * rx0) + fabsf(t.g1.y * ry0));
    b.e1 += s1;
    b.e2 += s2;
    b.e0 += s1 + s2;
    return b;
}

// the in-element decision from FP32 barycentrics, exact FP64 test in the band
__device__ __forceinline__ bool in_tri_decide(const DevMesh& m, const Bary& b, int k, double x,
                                              double y);

__device__ __forceinline__ bool in_tri_decide(const DevMesh& m, const Bary& b, int k, double x,
                                              double y) {
    if (b.l0 > b.e0 && b.l1 > b.e1 && b.l2 > b.e2) return true;
    if (b.l0 < -b.e0 || b.l1 < -b.e1 || b.l2 < -b.e2) return false;
    return in_tri(m, k, x, y);
}

// same decision as in_tri (the FP64 predicate), FP32 outside the band
__device__ __forceinline__ bool in_tri_mixed(const DevMesh& m, const Tri32& t, int k, double x,
                                             double y) {
    return in_tri_decide(m, bary32(t, x, y), k, x, y);
}

// the same from a walk record (its vertex a and gradients are Tri32's)
__device__ __forceinline__ bool in_tri_mixed_rec(const WalkRec& t, double x, double y) {
    const Bary b = bary32_off(t, (float)(x - t.a.x), (float)(y - t.a.y));
    if (b.l0 > b.e0 && b.l1 > b.e1 && b.l2 > b.e2) return true;
    if (b.l0 < -b.e0 || b.l1 < -b.e1 || b.l2 < -b.e2) return false;
    return in_tri_rec(t, x, y);
}

// xylocalizer.pyx:338-435 with FP32-filtered predicates: the in-element
// tests through in_tri_mixed, the segment/edge tests through
// intersec2d_filtered, both falling back to FP64 where the FP32 value is
// within its rounding bound.  Same decisions, hence the same triangle or
// boundary edge, as path_walk.
__device__ inline void path_walk_mixed(const DevMesh& m, int k, double p0x, double p0y, double x,
                                       double y, int& new_k, int& bnd) {
    new_k = -1;
    bnd = -1;
    int intersected_edge = -1;
    const float2 p1 = make_float2((float)(x - p0x), (float)(y - p0y));
    WalkRec t = load_walkrec(m, k);
    for (int niter = 0; niter <= NITER_MAX; ++niter) {
        bool intersects = false;
        // the element's three vertices relative to the segment's start, once
        // per element (each edge takes two of them; the FP64 subtraction and
        // the conversion are the walk's FP64-pipe work)
        const float2 va = make_float2((float)(t.a.x - p0x), (float)(t.a.y - p0y));
        const float2 vb = make_float2((float)(t.b.x - p0x), (float)(t.b.y - p0y));
        const float2 vc = make_float2((float)(t.c.x - p0x), (float)(t.c.y - p0y));
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            int j, kn;
            double2 a, b;
            rec_edge(t, i, k, j, a, b, kn);
            if (j == intersected_edge) continue;
            const int la = (t.order >> (4 * i)) & 3, lb = (t.order >> (4 * i + 2)) & 3;
            const float2 fa = la == 0 ? va : (la == 1 ? vb : vc);
            const float2 fb = lb == 0 ? va : (lb == 1 ? vb : vc);
            if (intersec2d_filtered(p1, fa, fb, p0x, p0y, x, y, a, b)) {
                intersects = true;
                if (kn == -1) { bnd = j; return; }
                const WalkRec tn = load_walkrec(m, kn);
                if (in_tri_mixed_rec(tn, x, y)) { new_k = kn; return; }
                k = kn;
                t = tn;
                intersected_edge = j;
                break;
            }
        }
        if (!intersects) {
            if (in_tri_mixed_rec(t, x, y)) new_k = k;
            return;
        }
    }
}

// in-element decision from FP32 barycentrics: 1 certainly inside, 0
// certainly outside, -1 within the rounding band (exact test needed)
__device__ __forceinline__ int decide32(const Bary& b) {
    if (b.l0 > b.e0 && b.l1 > b.e1 && b.l2 > b.e2) return 1;
    if (b.l0 < -b.e0 || b.l1 < -b.e1 || b.l2 < -b.e2) return 0;
    return -1;
}

// index of the one edge (opposite vertex j) that the point is certainly
// beyond while certainly inside the other two; -1 otherwise
__device__ __forceinline__ int single_exit(const Bary& b) {
    const bool n0 = b.l0 < -b.e0, n1 = b.l1 < -b.e1, n2 = b.l2 < -b.e2;
    const bool p0 = b.l0 > b.e0, p1 = b.l1 > b.e1, p2 = b.l2 > b.e2;
    if (n0 && p1 && p2) return 0;
    if (n1 && p0 && p2) return 1;
    if (n2 && p0 && p1) return 2;
    return -1;
}

// One-hop exit.  When the start point is certainly inside the start
// triangle and the end point certainly beyond exactly one of its edges (the
// other two barycentric coordinates certainly positive at both points), the
// segment crosses that edge alone, in its interior: the first edge the
// reference's path walk finds (xylocalizer.pyx:375-415).  The walk's next
// test, the point in the neighbour across it, is made here, and so are up
// to two further crossings of the same kind (see hop_walk_split).  Returns
// the triangle holding the end point, else -1 (the full walk decides).
__device__ __forceinline__ int one_hop(const DevMesh& m, int tri0, const Bary& bs, const Bary& be,
                                       double xn, double yn) {
    if (!(bs.l0 > bs.e0 && bs.l1 > bs.e1 && bs.l2 > bs.e2)) return -1;
    int k = tri0;
    Bary b = be;
    // further crossings as hop_walk_split argues (up to three in all)
#pragma unroll 1
    for (int h = 0; h < 3; ++h) {
        const bool n0 = b.l0 < -b.e0, n1 = b.l1 < -b.e1, n2 = b.l2 < -b.e2;
        const bool p0 = b.l0 > b.e0, p1 = b.l1 > b.e1, p2 = b.l2 > b.e2;
        int j;
        if (n0 && p1 && p2) j = 0;
        else if (n1 && p0 && p2) j = 1;
        else if (n2 && p0 && p1) j = 2;
        else return -1;
        int4 nb = __ldg(&m.nbr[CG_IDX(m, k, m.nt)]);
        int kn = j == 0 ? nb.x : (j == 1 ? nb.y : nb.z);
        if (kn < 0) return -1;   // boundary edge: the full walk finds it
        Tri32 tn = load_tri32(m, kn);
        b = bary32(tn, xn, yn);
        if (b.l0 > b.e0 && b.l1 > b.e1 && b.l2 > b.e2) return kn;
        if (!(b.l0 < -b.e0 || b.l1 < -b.e1 || b.l2 < -b.e2))   // rounding band
            return in_tri(m, kn, xn, yn) ? kn : -1;
        k = kn;
    }
    return -1;
}

// xy_localize (xylocalizer.pyx:27-124, method 3) with the FP32-filtered
// in-element and walk tests of the mixed form: the same decisions, with the
// FP64 arithmetic only inside the rounding bands.  A start index below 0 (a
// Runge-Kutta stage that left the mesh) takes the plain path.
__device__ inline void xy_localize_filtered(const DevMesh& m, int k, double p0x, double p0y,
                                            double x, double y, int& new_k, int& bnd) {
    if (k < 0) {
        xy_localize(m, k, p0x, p0y, x, y, new_k, bnd);
        return;
    }
    bnd = -1;
    const Tri32 t = load_tri32(m, k);
    const Bary be = bary32(t, x, y);
    if (in_tri_decide(m, be, k, x, y)) { new_k = k; return; }
    // certain single-edge crossings in FP32 (one_hop), the full walk else
    new_k = one_hop(m, k, bary32(t, p0x, p0y), be, x, y);
    if (new_k >= 0) return;
    path_walk_mixed(m, k, p0x, p0y, x, y, new_k, bnd);
    if (new_k == -1 && bnd == -1) new_k = grid_locate(m, x, y);
}

}  // namespace cg
