// cg_kernels_mixed.cu -- the mixed-precision form (FP32 fields and
// increments, FP64 positions and localization decisions).  Compiled with
// the default FMA contraction; the exact FP64 predicates it shares with the
// plain form are written with _rn intrinsics and are not contracted.
#include <cstdlib>

#include "cg_internal.h"
#include "cg_step_mixed.cuh"

namespace cg {

void launch_step_mixed(const DevMesh& m, const FieldView& fv, const DevParams& p,
                       const DevState& s, const WalkQueue& wq, int aux, int step_index,
                       int* stats, uint32_t* err, cudaStream_t st) {
    int bs = 256;
    int nb = (s.n + bs - 1) / bs;
    if (nb == 0) return;
    auto wave = [](auto kernel, int bs_) {
        int dev = 0, nsm = 152, per = 1;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, bs_, 0);
        return nsm * (per < 1 ? 1 : per);
    };
    if (p.model != 1) {
        // LSM2 / LSM3: FP32 node records and Langevin coefficients, inline walk
        launch_lsm23_mixed(m, fv, p, s, aux, step_index, stats, err, st);
        return;
    }
    DevFields<float> f = fv.as<float>();
    WalkQueue none{nullptr, nullptr};
    if (fv.dim == 2) {
        // occupancy variant (resident blocks of 256 per SM): by default 4 (64
        // registers) for the Euler-with-queue form, which has no out-of-line
        // calls, and 3 (80) for the others; 2, 3 or 4 on request
        static int minb_env = [] {
            const char* e = getenv("CYLAG_MIXED_MINB");
            int v = e ? atoi(e) : 0;
            return (v >= 2 && v <= 4) ? v : 0;
        }();
        // persistent grid: one wave of resident blocks
        static int w2 = wave(step_mixed2d_kernel<2>, bs), w3 = wave(step_mixed2d_kernel<3>, bs),
                   w4 = wave(step_mixed2d_kernel<4>, bs),
                   w3s = wave(step_mixed2d_kernel<3, true>, bs),
                   w2s = wave(step_mixed2d_kernel<2, true>, bs),
                   w4s = wave(step_mixed2d_kernel<4, true>, bs),
                   w2st = wave(step_mixed2d_kernel<2, true, true>, bs),
                   w3sa = wave(step_mixed2d_kernel<3, true, true, true>, bs),
                   w3st = wave(step_mixed2d_kernel<3, true, true>, bs),
                   w3t = wave(step_mixed2d_kernel<3, false, true>, bs);
        // bulk-copy staging of the state tiles: 16-byte aligned arrays
        // (0: off, the default; 2 or 3: bulk copies per warp tile at 2 or 3
        // resident blocks per SM; 4: per-thread cp.async one particle ahead).
        // Measured on the default 1e7-particle LSM1 case (kernels per step,
        // before the call-free Euler-with-queue form, which the staged
        // variants do not have): 0.478-0.495 ms off, 0.567 ms bulk at 2
        // blocks/SM (no spills),
        // 0.640 ms bulk at 3 (spills), 0.521 ms per-thread cp.async: the
        // state's HBM latency is not what bounds the step, and staging costs
        // registers and instructions
        static const int stage_minb = [] {
            const char* e = getenv("CYLAG_MIXED_STAGE");
            int v = e ? atoi(e) : 0;
            return (v >= 2 && v <= 4) ? v : 0;
        }();
        const bool stage_on = stage_minb != 0;
        auto a16 = [](const void* q) { return ((uintptr_t)q & 15u) == 0; };
        const bool staged = stage_on && s.n >= 32 && a16(s.pos) && a16(s.rng) && a16(s.tri) &&
                            a16(s.tag);
        // EQ: the Euler scheme with a walk queue, no out-of-line calls
        const bool eq = p.time_scheme == 1 && wq.e != nullptr;
        const int minb = minb_env ? minb_env : (eq ? 4 : 3);
        static int w2e = wave(step_mixed2d_kernel<2, false, false, false, true>, bs),
                   w3e = wave(step_mixed2d_kernel<3, false, false, false, true>, bs),
                   w4e = wave(step_mixed2d_kernel<4, false, false, false, true>, bs),
                   w2se = wave(step_mixed2d_kernel<2, true, false, false, true>, bs),
                   w3se = wave(step_mixed2d_kernel<3, true, false, false, true>, bs),
                   w4se = wave(step_mixed2d_kernel<4, true, false, false, true>, bs);
        auto grid = [nb](int w) { return nb < w ? nb : w; };
        if ((s.work & W_SPLIT) && staged && stage_minb == 4)   // per-thread cp.async prefetch
            step_mixed2d_kernel<3, true, true, true><<<grid(w3sa), bs, 0, st>>>(
                m, f, p, s, wq, aux, step_index, stats, err);
        else if ((s.work & W_SPLIT) && staged && stage_minb == 2)
            step_mixed2d_kernel<2, true, true><<<grid(w2st), bs, 0, st>>>(
                m, f, p, s, wq, aux, step_index, stats, err);
        else if ((s.work & W_SPLIT) && staged)
            step_mixed2d_kernel<3, true, true><<<grid(w3st), bs, 0, st>>>(
                m, f, p, s, wq, aux, step_index, stats, err);
        else if ((s.work & W_SPLIT) && eq && minb == 2)
            step_mixed2d_kernel<2, true, false, false, true><<<grid(w2se), bs, 0, st>>>(
                m, f, p, s, wq, aux, step_index, stats, err);
        else if ((s.work & W_SPLIT) && eq && minb == 4)
            step_mixed2d_kernel<4, true, false, false, true><<<grid(w4se), bs, 0, st>>>(
                m, f, p, s, wq, aux, step_index, stats, err);
        else if ((s.work & W_SPLIT) && eq)
            step_mixed2d_kernel<3, true, false, false, true><<<grid(w3se), bs, 0, st>>>(
                m, f, p, s, wq, aux, step_index, stats, err);
        else if ((s.work & W_SPLIT) && minb == 2)
            step_mixed2d_kernel<2, true><<<grid(w2s), bs, 0, st>>>(m, f, p, s, wq, aux,
                                                                  step_index, stats, err);
        else if ((s.work & W_SPLIT) && minb == 4)
            step_mixed2d_kernel<4, true><<<grid(w4s), bs, 0, st>>>(m, f, p, s, wq, aux,
                                                                  step_index, stats, err);
        else if (s.work & W_SPLIT)   // sorted working copies with split positions
            step_mixed2d_kernel<3, true><<<grid(w3s), bs, 0, st>>>(m, f, p, s, wq, aux,
                                                                  step_index, stats, err);
        else if (staged && minb == 3)
            step_mixed2d_kernel<3, false, true><<<grid(w3t), bs, 0, st>>>(
                m, f, p, s, wq, aux, step_index, stats, err);
        else if (eq && minb == 2)
            step_mixed2d_kernel<2, false, false, false, true><<<grid(w2e), bs, 0, st>>>(
                m, f, p, s, wq, aux, step_index, stats, err);
        else if (eq && minb == 3)
            step_mixed2d_kernel<3, false, false, false, true><<<grid(w3e), bs, 0, st>>>(
                m, f, p, s, wq, aux, step_index, stats, err);
        else if (eq)
            step_mixed2d_kernel<4, false, false, false, true><<<grid(w4e), bs, 0, st>>>(
                m, f, p, s, wq, aux, step_index, stats, err);
        else if (minb == 3)
            step_mixed2d_kernel<3><<<grid(w3), bs, 0, st>>>(m, f, p, s, wq, aux, step_index,
                                                           stats, err);
        else if (minb == 2)
            step_mixed2d_kernel<2><<<grid(w2), bs, 0, st>>>(m, f, p, s, wq, aux, step_index,
                                                           stats, err);
        else
            step_mixed2d_kernel<4><<<grid(w4), bs, 0, st>>>(m, f, p, s, wq, aux, step_index,
                                                           stats, err);
    } else {
        // 3D: FP32 node records, FP64 arithmetic
        launch_lsm1_kernel<3, float>(m, f, p, s, none, aux, step_index, stats, err, st);
    }
}

void launch_walk_mixed(const DevMesh& m, const FieldView& fv, const DevParams& p,
                       const DevState& s, const WalkQueue& wq, int aux, int step_index,
                       int* stats, uint32_t* err, cudaStream_t st) {
    int dev = 0, nsm = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    DevFields<float> f = fv.as<float>();
    walk_kernel<float, true><<<nsm * WALK_BLOCKS_PER_SM, WALK_BLOCK, 0, st>>>(
        m, f, p, s, wq, aux, step_index, stats, err);
}

}  // namespace cg
