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
                             FT* __restrict__ cur) {
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
        r[5] = (FT)0;
        r[6] = (FT)0;
        r[7] = (FT)0;
    }
}

void launch_blend(const DevFrames& fr, int rec, double tf, bool frozen, double fac, void* cur,
                  int precision, cudaStream_t st) {
    int bs = 256;
    int64_t nb = (fr.nnodes + bs - 1) / bs;
    if (precision == 0) {
        if (fr.dim == 2)
            blend_kernel<2, double><<<nb, bs, 0, st>>>(fr, rec, tf, frozen, fac, (double*)cur);
        else
            blend_kernel<3, double><<<nb, bs, 0, st>>>(fr, rec, tf, frozen, fac, (double*)cur);
    } else {
        // FP64 interpolation, rounded once to the FP32 record
        if (fr.dim == 2)
            blend_kernel<2, float><<<nb, bs, 0, st>>>(fr, rec, tf, frozen, fac, (float*)cur);
        else
            blend_kernel<3, float><<<nb, bs, 0, st>>>(fr, rec, tf, frozen, fac, (float*)cur);
    }
}

// ---------------------------------------------------------------------------
// the fused step
// ---------------------------------------------------------------------------
// one wave of resident blocks (persistent grid), capped by the work
template <typename K>
static int resident_grid(K kernel, int n, int bs) {
    int dev = 0, nsm = 152, per = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, bs, 0);
    if (per < 1) per = 1;
    int need = (n + bs - 1) / bs;
    int wave = nsm * per;
    return need < wave ? need : wave;
}

void launch_step_plain(int dim, const DevMesh& m, const void* cur, const void* prev, int npoints,
                       int nlayers, int prev_valid, const DevParams& p, const DevState& s,
                       const WalkQueue& wq, int aux, int step_index, int* stats, uint32_t* err,
                       cudaStream_t st) {
    int bs = 256;
    if (s.n == 0) return;
    static int nb2 = 0, nb3 = 0;
    if (!nb2) nb2 = resident_grid(step_kernel<2, double>, 1 << 30, bs);
    if (!nb3) nb3 = resident_grid(step_kernel<3, double>, 1 << 30, bs);
    int need = (s.n + bs - 1) / bs;
    int nb = dim == 2 ? nb2 : nb3;
    nb = need < nb ? need : nb;
    if (dim == 2) {
        DevFields<double> f{(const double*)cur, (const double*)prev, npoints, nlayers, 2, prev_valid};
        step_kernel<2, double><<<nb, bs, 0, st>>>(m, f, p, s, wq, aux, step_index, stats, err);
    } else {
        DevFields<double> f{(const double*)cur, (const double*)prev, npoints, nlayers, 3, prev_valid};
        WalkQueue none{nullptr, nullptr};
        step_kernel<3, double><<<nb, bs, 0, st>>>(m, f, p, s, none, aux, step_index, stats, err);
    }
}

void launch_walk_plain(int precision, const DevMesh& m, const void* cur, int npoints, int nlayers,
                 const DevParams& p, const DevState& s, const WalkQueue& wq, int aux,
                 int step_index, int* stats, uint32_t* err, cudaStream_t st) {
    // grid-stride over the (device-side) entry count: a fixed grid of
    // 8 blocks per SM covers any count without a host round trip
    int dev = 0, nsm = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    int nb = nsm * 8;
    (void)precision;
    DevFields<double> f{(const double*)cur, (const double*)cur, npoints, nlayers, 2, 0};
    walk_kernel<double, false><<<nb, 256, 0, st>>>(m, f, p, s, wq, aux, step_index, stats, err);
}

// ---------------------------------------------------------------------------
// Solver.initialize_particle_state (solver.pyx:238-379)
// ---------------------------------------------------------------------------
template <int DIM, typename FT>
__global__ void init_kernel(DevMesh m, DevFields<FT> f, DevParams p, DevState s, int vinit,
                            uint32_t* err) {
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
        s.tri[i] = -1;
        s.last_tri[i] = -1;
        s.lowerlayer[i] = 0;
        s.tag[i] = -1;  // deleted during initialization
        return;
    }
    int ll = 0;
    if (DIM == 3) {
        double zs = q.zs_at(k, f.nlayers - 1, q.x[0], q.x[1]);
        double zb = q.zs_at(k, 0, q.x[0], q.x[1]);
        ll = lower_layer_index(f.nlayers, zs, zb, q.x[2]);
        if (q.x[2] < zb) q.x[2] = zb + EPSILON;
        if (q.x[2] > zs) q.x[2] = zs - EPSILON;
        s.pos[(size_t)i * D + 2] = q.x[2];
        s.lowerlayer[i] = ll;
    }
    s.tri[i] = k;
    if (vinit == 1) {
        double ux, uy, uz;
        q.velocity(k, ll, q.x[0], q.x[1], DIM == 3 ? q.x[2] : 0., ux, uy, uz);
        double u[3] = {ux, uy, uz};
#pragma unroll
        for (int d = 0; d < D; ++d) {
            s.vel[(size_t)i * D + d] = u[d];
            s.fvs[(size_t)i * D + d] = u[d];
        }
    }
    if (q.err) atomicOr(err, q.err);
}

void launch_init(int dim, int precision, const DevMesh& m, const void* cur, int npoints,
                 int nlayers, const DevParams& p, const DevState& s, int vinit, uint32_t* err,
                 cudaStream_t st) {
    int bs = 256;
    int nb = (s.n + bs - 1) / bs;
    if (nb == 0) return;
    if (precision != 0) {
        if (dim == 2) {
            DevFields<float> f{(const float*)cur, (const float*)cur, npoints, nlayers, 2, 0};
            init_kernel<2, float><<<nb, bs, 0, st>>>(m, f, p, s, vinit, err);
        } else {
            DevFields<float> f{(const float*)cur, (const float*)cur, npoints, nlayers, 3, 0};
            init_kernel<3, float><<<nb, bs, 0, st>>>(m, f, p, s, vinit, err);
        }
        return;
    }
    if (dim == 2) {
        DevFields<double> f{(const double*)cur, (const double*)cur, npoints, nlayers, 2, 0};
        init_kernel<2, double><<<nb, bs, 0, st>>>(m, f, p, s, vinit, err);
    } else {
        DevFields<double> f{(const double*)cur, (const double*)cur, npoints, nlayers, 3, 0};
        init_kernel<3, double><<<nb, bs, 0, st>>>(m, f, p, s, vinit, err);
    }
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

void launch_seed(const int* tag, uint64_t* rng, int n, uint64_t seed, cudaStream_t st) {
    int bs = 256;
    int nb = (n + bs - 1) / bs;
    if (nb) seed_kernel<<<nb, bs, 0, st>>>(tag, rng, n, seed);
}

}  // namespace cg
