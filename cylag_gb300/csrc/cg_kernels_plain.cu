// cg_kernels_plain.cu -- the plain (FP64 end-to-end) form.
//
// Compiled with -fmad=false: every multiply and add rounds on its own, as in
// the reference's C, so element indices and PCG32 streams match it bit for
// bit and positions agree to rounding of libm transcendentals.
#include <cstdio>

#include "cg_internal.h"
#include "cg_step.cuh"

namespace cg {

// ---------------------------------------------------------------------------
// time interpolation of the node fields (eulerian_field_set.pyx:866-938)
// ---------------------------------------------------------------------------
template <int DIM, typename FT>
__global__ void blend_kernel(DevFrames fr, int rec, double tf, int frozen, double fac,
                             FT* __restrict__ cur, FT* __restrict__ turb) {
    using S = Slots<DIM>;
    int64_t n = fr.nnodes;
    int64_t node = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= n) return;
    const double* f0 = fr.frames + (int64_t)rec * fr.nraw * n;
    const double* f1 = f0 + (int64_t)fr.nraw * n;
    auto val = [&](int rf) -> double {
        int sl = fr.raw_slot[rf];
        if (sl < 0) return 0.0;
        double a = f0[(int64_t)sl * n + node];
        if (frozen) return a;
        double b = f1[(int64_t)sl * n + node];
        return tf * a + (1. - tf) * b;
    };
    FT* r = cur + node * S::NF;
    double zs = val(RF_ZS), ux = val(RF_UX), uy = val(RF_UY);
    double kt = val(RF_KT), ep = val(RF_EP);
    // eulerian_field_set.pyx:1995-1997
    double K = fac * kt * kt / fmax(ep, EPSILON);
    r[S::ZS] = (FT)zs;
    r[S::UX] = (FT)ux;
    r[S::UY] = (FT)uy;
    r[S::K] = (FT)K;
    if (DIM == 3) {
        r[Slots<3>::UZ] = (FT)val(RF_UZ);
        r[Slots<3>::ZB] = (FT)val(RF_ZB);   // BOTTOM (2D fields: pseudo-3D runs)
        r[6] = (FT)0;
        r[7] = (FT)0;
    }
    if (turb) {
        turb[2 * node] = (FT)kt;
        turb[2 * node + 1] = (FT)ep;
    }
}

// the mixed form's blend: FP32 frames and FP32 arithmetic (the record is
// FP32 either way; interpolation and K add a few FP32 roundings)
template <int DIM>
__global__ void blend32_kernel(DevFrames fr, int rec, float tf, int frozen, float fac,
                               float* __restrict__ cur, float* __restrict__ turb) {
    using S = Slots<DIM>;
    const int64_t n = fr.nnodes;
    const int64_t node = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= n) return;
    const float* f0 = fr.frames32 + (int64_t)rec * fr.nraw * n;
    const float* f1 = f0 + (int64_t)fr.nraw * n;
    auto val = [&](int rf) -> float {
        const int sl = fr.raw_slot[rf];
        if (sl < 0) return 0.f;
        const float a = __ldg(&f0[(int64_t)sl * n + node]);
        if (frozen) return a;
        const float b = __ldg(&f1[(int64_t)sl * n + node]);
        return tf * a + (1.f - tf) * b;
    };
    float* r = cur + node * S::NF;
    const float kt = val(RF_KT), ep = val(RF_EP);
    r[S::ZS] = val(RF_ZS);
    r[S::UX] = val(RF_UX);
    r[S::UY] = val(RF_UY);
    r[S::K] = fac * kt * kt / fmaxf(ep, 1e-16f);   // eulerian_field_set.pyx:1995-1997
    if (DIM == 3) {
        r[Slots<3>::UZ] = val(RF_UZ);
        r[Slots<3>::ZB] = val(RF_ZB);
        r[6] = 0.f;
        r[7] = 0.f;
    }
    if (turb) {
        turb[2 * node] = kt;
        turb[2 * node + 1] = ep;
    }
}

void launch_blend(const DevFrames& fr, int rec, double tf, bool frozen, double fac, void* cur,
                  void* turb, int precision, int rdim, cudaStream_t st) {
    int bs = 256;
    int64_t nb = (fr.nnodes + bs - 1) / bs;
    if (precision == 0) {
        double *c = (double*)cur, *t = (double*)turb;
        if (rdim == 2) blend_kernel<2, double><<<nb, bs, 0, st>>>(fr, rec, tf, frozen, fac, c, t);
        else blend_kernel<3, double><<<nb, bs, 0, st>>>(fr, rec, tf, frozen, fac, c, t);
    } else if (fr.frames32) {
        float *c = (float*)cur, *t = (float*)turb;
        if (rdim == 2)
            blend32_kernel<2><<<nb, bs, 0, st>>>(fr, rec, (float)tf, frozen, (float)fac, c, t);
        else
            blend32_kernel<3><<<nb, bs, 0, st>>>(fr, rec, (float)tf, frozen, (float)fac, c, t);
    } else {
        // FP64 interpolation, rounded once to the FP32 record
        float *c = (float*)cur, *t = (float*)turb;
        if (rdim == 2) blend_kernel<2, float><<<nb, bs, 0, st>>>(fr, rec, tf, frozen, fac, c, t);
        else blend_kernel<3, float><<<nb, bs, 0, st>>>(fr, rec, tf, frozen, fac, c, t);
    }
}

// ---------------------------------------------------------------------------
// the fused step
// ---------------------------------------------------------------------------
void launch_step_plain(const DevMesh& m, const FieldView& fv, const DevParams& p,
                       const DevState& s, const WalkQueue& wq, int aux, int step_index,
                       int* stats, uint32_t* err, cudaStream_t st) {
    if (p.model != 1) {
        launch_lsm23_plain(m, fv, p, s, aux, step_index, stats, err, st);
        return;
    }
    DevFields<double> f = fv.as<double>();
    if (p.pdim == 2) {
        launch_lsm1_kernel<2, double>(m, f, p, s, wq, aux, step_index, stats, err, st);
    } else {
        WalkQueue none{nullptr, nullptr};
        launch_lsm1_kernel<3, double>(m, f, p, s, none, aux, step_index, stats, err, st);
    }
}

void launch_walk_plain(const DevMesh& m, const FieldView& fv, const DevParams& p,
                       const DevState& s, const WalkQueue& wq, int aux, int step_index,
                       int* stats, uint32_t* err, cudaStream_t st) {
    // grid-stride over the (device-side) entry count: a fixed grid of
    // 32 blocks of 64 per SM covers any count without a host round trip;
    // small blocks spread a short queue (a few thousand boundary and
    // multi-hop entries) over every SM instead of a few dozen
    int dev = 0, nsm = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    DevFields<double> f = fv.as<double>();
    walk_kernel<double, false><<<nsm * WALK_BLOCKS_PER_SM, WALK_BLOCK, 0, st>>>(
        m, f, p, s, wq, aux, step_index, stats, err);
}

// ---------------------------------------------------------------------------
// Solver.initialize_particle_state (solver.pyx:238-379)
// ---------------------------------------------------------------------------
template <int DIM, typename FT>
__global__ void init_kernel(DevMesh m, DevFields<FT> f, DevParams p, DevState s, int vinit,
                            int del_mark, uint32_t* err) {
    __shared__ ZigTables zt;
    for (int t = threadIdx.x; t < 128; t += blockDim.x) {
        zt.kn[t] = g_zig.kn[t];
        zt.wn[t] = g_zig.wn[t];
        zt.fn[t] = g_zig.fn[t];
    }
    __syncthreads();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.n || s.tri[i] != -2) return;
    const int D = DIM;
    Particle<DIM, FT> q(m, f, p, zt);
#pragma unroll
    for (int d = 0; d < D; ++d) q.x[d] = s.pos[(size_t)i * D + d];
    int k = grid_locate(m, q.x[0], q.x[1]);
    if (k == -1) {
#pragma unroll
        for (int d = 0; d < D; ++d) {
            s.pos[(size_t)i * D + d] = 0.;
            s.vel[(size_t)i * D + d] = 0.;
            s.fvs[(size_t)i * D + d] = 0.;
            s.last_pos[(size_t)i * D + d] = 0.;
            s.last_vel[(size_t)i * D + d] = 0.;
        }
        s.diameter[i] = 0.;
        if (s.depth) s.depth[i] = 0.;
        s.tri[i] = -1;
        s.last_tri[i] = -1;
        s.lowerlayer[i] = 0;
        s.tag[i] = del_mark;  // deleted during initialization (new tag given on the host)
        return;
    }
    int ll = 0;
    if (DIM == 3) {
        double zs = q.zs_at(k, f.nlayers - 1, q.x[0], q.x[1]);
        double zb = q.zb_at(k, q.x[0], q.x[1]);
        ll = lower_layer_index(f.nlayers, zs, zb, q.x[2]);
        if (q.x[2] < zb) q.x[2] = zb + EPSILON;
        if (q.x[2] > zs) q.x[2] = zs - EPSILON;
        s.pos[(size_t)i * D + 2] = q.x[2];
        s.lowerlayer[i] = ll;
        if (s.depth) s.depth[i] = zs - q.x[2];   // solver.pyx:325-332
    }
    s.tri[i] = k;
    if (vinit == 1) {
        double ux, uy, uz;
        if (DIM == 3 && f.dim == 2) {
            // 2D fields: the depth-averaged velocity, no pseudo-3D
            // correction; the vertical components keep their values
            // (solver.pyx:334-340, 366-372)
            P1 q1 = p1_at(m, k, q.x[0], q.x[1]);
            ux = p1_eval<DIM>(f.cur, 0, q1, Slots<3>::UX);
            uy = p1_eval<DIM>(f.cur, 0, q1, Slots<3>::UY);
            uz = s.vel[(size_t)i * D + 2];
        } else {
            q.velocity(k, ll, q.x[0], q.x[1], DIM == 3 ? q.x[2] : 0., ux, uy, uz);
        }
        double u[3] = {ux, uy, uz}, w[3] = {ux, uy, uz};
        if (p.model >= 2) {
            // stationary fluctuations from the particle's own stream
            // (solver.pyx:342-379)
            q.tri = k;
            q.ll = ll;
            q.rng.state = s.rng[i];
            q.rng.inc = ((uint64_t)(uint32_t)s.tag[i] << 1) | 1ULL;
            q.rng.err = 0;
            double fl[3];
            if (p.model == 2 && p.nuopt >= 2 && p.diffmod != 0) {
                lsm2_fluctuations(q, s.diameter[i], fl);
#pragma unroll
                for (int d = 0; d < D; ++d) u[d] += fl[d];
            }
#pragma unroll
            for (int d = 0; d < D; ++d) w[d] = u[d];
            if (p.model == 3) {
                lsm3_fluctuations(q, fl);
#pragma unroll
                for (int d = 0; d < D; ++d) w[d] += fl[d];
            }
            s.rng[i] = q.rng.state;
            q.err |= q.rng.err;
        }
#pragma unroll
        for (int d = 0; d < D; ++d) {
            s.vel[(size_t)i * D + d] = u[d];
            s.fvs[(size_t)i * D + d] = w[d];
        }
    }
    if (q.err) atomicOr(err, q.err);
}

void launch_init(int precision, const DevMesh& m, const FieldView& fv, const DevParams& p,
                 const DevState& s, int vinit, int del_mark, uint32_t* err, cudaStream_t st) {
    int bs = 256;
    int nb = (s.n + bs - 1) / bs;
    if (nb == 0) return;
    if (precision != 0) {
        DevFields<float> f = fv.as<float>();
        if (p.pdim == 2) init_kernel<2, float><<<nb, bs, 0, st>>>(m, f, p, s, vinit, del_mark, err);
        else init_kernel<3, float><<<nb, bs, 0, st>>>(m, f, p, s, vinit, del_mark, err);
        return;
    }
    DevFields<double> f = fv.as<double>();
    if (p.pdim == 2) init_kernel<2, double><<<nb, bs, 0, st>>>(m, f, p, s, vinit, del_mark, err);
    else init_kernel<3, double><<<nb, bs, 0, st>>>(m, f, p, s, vinit, del_mark, err);
}

// solver.pyx:526-538: depth below the free surface of every active 3D
// particle, from its end-of-step position and element and the step's
// fields (a sorted run's working copies, written to the caller's slots)
template <typename FT>
__global__ void depth_kernel(DevMesh m, DevFields<FT> f, DevState s) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.n) return;
    const int k = s.tri[i];
    if (k < 0) return;
    const double px = s.pos[(size_t)i * 3], py = s.pos[(size_t)i * 3 + 1];
    const P1 q = p1_at(m, k, px, py);
    const double zs = p1_eval<3>(f.cur, (f.nlayers - 1) * f.npoints, q, Slots<3>::ZS);
    s.depth[aux_index(s, i)] = zs - s.pos[(size_t)i * 3 + 2];
}

void launch_depth(int precision, const DevMesh& m, const FieldView& fv, const DevState& s,
                  cudaStream_t st) {
    const int bs = 256, nb = (s.n + bs - 1) / bs;
    if (nb == 0 || s.depth == nullptr) return;
    if (precision != 0) depth_kernel<float><<<nb, bs, 0, st>>>(m, fv.as<float>(), s);
    else depth_kernel<double><<<nb, bs, 0, st>>>(m, fv.as<double>(), s);
}

// ---------------------------------------------------------------------------
// stream seeding (random_utils.pyx:30-37)
// ---------------------------------------------------------------------------
__global__ void seed_kernel(const int* __restrict__ tag, uint64_t* __restrict__ rng, int n,
                            uint64_t seed) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint64_t st, inc;
    pcg_seed(seed, (uint64_t)(uint32_t)tag[i], st, inc);
    rng[i] = st;
}

// random_utils.pyx's public draws from pcg32_seed(seed, stream), in stream
// order (one thread): 0 uniform, 1 ziggurat normal, 2 polar normal (the
// first of a pair), 3 pairs of generate_random_pair(method) (2n values),
// 4 generate_random_single(method).  Plain form (FP64 samplers).
__global__ void rng_draws_kernel(uint64_t seed, uint64_t stream, int kind, int method, int64_t n,
                                 double* __restrict__ out, uint32_t* __restrict__ err) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    Rng r;
    pcg_seed(seed, stream, r.state, r.inc);
    r.err = 0;
    for (int64_t i = 0; i < n; ++i) {
        if (kind == 0) {
            out[i] = rng_uniform(r);
        } else if (kind == 1) {
            out[i] = rng_ziggurat(r, g_zig);
        } else if (kind == 2) {
            double a, b;
            rng_polar(r, a, b);
            out[i] = a;
        } else if (kind == 3) {
            rng_pair(r, method, g_zig, out[2 * i], out[2 * i + 1]);
        } else {
            out[i] = rng_single(r, method, g_zig);
        }
    }
    if (r.err) atomicOr(err, r.err);
}

void launch_rng_draws(uint64_t seed, uint64_t stream, int kind, int method, int64_t n,
                      double* out, uint32_t* err, cudaStream_t st) {
    rng_draws_kernel<<<1, 32, 0, st>>>(seed, stream, kind, method, n, out, err);
}

void launch_seed(const int* tag, uint64_t* rng, int n, uint64_t seed, cudaStream_t st) {
    int bs = 256;
    int nb = (n + bs - 1) / bs;
    if (nb) seed_kernel<<<nb, bs, 0, st>>>(tag, rng, n, seed);
}

__global__ void seed_added_kernel(const int* __restrict__ tri, const int* __restrict__ tag,
                                  uint64_t* __restrict__ rng, int n, uint64_t seed) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || tri[i] != -2) return;
    uint64_t st, inc;
    pcg_seed(seed, (uint64_t)(uint32_t)tag[i], st, inc);
    rng[i] = st;
}

void launch_seed_added(const int* tri, const int* tag, uint64_t* rng, int n, uint64_t seed,
                       cudaStream_t st) {
    int bs = 256;
    int nb = (n + bs - 1) / bs;
    if (nb) seed_added_kernel<<<nb, bs, 0, st>>>(tri, tag, rng, n, seed);
}

}  // namespace cg
