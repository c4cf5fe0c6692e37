// cg_kernels_mixed.cu -- the mixed-precision form (FP32 fields and
// increments, FP64 positions and localization decisions).  Compiled with
// the default FMA contraction; the exact FP64 predicates it shares with the
// plain form are written with _rn intrinsics and are not contracted.
#include "cg_internal.h"
#include "cg_step_mixed.cuh"

namespace cg {

// blocks of one wave of resident blocks of `kernel` (persistent grid)
template <typename K>
static int wave_of(K kernel, int bs) {
    int dev = 0, nsm = 152, per = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, bs, 0);
    return nsm * (per < 1 ? 1 : per);
}

// the split Euler step compiled for one configuration (diffusion class DC,
// random number method RM): the steps without per-call outputs (aux 0), five
// blocks of 256 per SM (48 registers), or (TWO) those with them, on two
// working velocity arrays, four blocks (64 registers)
template <int DC, int RM, bool TWO>
static void launch_split_conf(const DevMesh& m, const DevFields<float>& f, const DevParams& p,
                              const DevState& s, const WalkQueue& wq, int aux, int step_index,
                              int* stats, uint32_t* err, int nb, int bs, cudaStream_t st) {
    constexpr int MINB = TWO ? 4 : 5;
    static const int w = wave_of(step_mixed2d_kernel<MINB, true, true, TWO, DC, RM>, bs);
    step_mixed2d_kernel<MINB, true, true, TWO, DC, RM><<<nb < w ? nb : w, bs, 0, st>>>(
        m, f, p, s, wq, aux, step_index, stats, err);
}

using SplitConfLaunch = void (*)(const DevMesh&, const DevFields<float>&, const DevParams&,
                                 const DevState&, const WalkQueue&, int, int, int*, uint32_t*,
                                 int, int, cudaStream_t);
#define CG_CONF_ROW(DC, TWO) \
    { launch_split_conf<DC, 1, TWO>, launch_split_conf<DC, 2, TWO>, launch_split_conf<DC, 3, TWO> }

void launch_step_mixed(const DevMesh& m, const FieldView& fv, const DevParams& p,
                       const DevState& s, const WalkQueue& wq, int aux, int step_index,
                       int* stats, uint32_t* err, cudaStream_t st) {
    int bs = 256;
    int nb = (s.n + bs - 1) / bs;
    if (nb == 0) return;
    auto wave = [](auto kernel, int bs_) { return wave_of(kernel, bs_); };
    if (p.model != 1) {
        // LSM2 / LSM3: FP32 node records and Langevin coefficients, inline walk
        launch_lsm23_mixed(m, fv, p, s, aux, step_index, stats, err, st);
        return;
    }
    DevFields<float> f = fv.as<float>();
    WalkQueue none{nullptr, nullptr};
    if (p.pdim == 2) {
        // persistent grid: one wave of resident blocks.  The Euler scheme with
        // a walk queue (EQ) has no out-of-line calls and runs 4 blocks of 256
        // per SM (64 registers); the other forms 3 (80).  Split positions on
        // the element-sorted working copies (W_SPLIT), which always come with
        // two velocity arrays (W_VEL2: TWO); the steps without per-call
        // outputs (aux 0) write no velocity, so they run the one-array form.
        static const int w3 = wave(step_mixed2d_kernel<3>, bs),
                         w3s = wave(step_mixed2d_kernel<3, true, false, true>, bs),
                         w4e = wave(step_mixed2d_kernel<4, false, true>, bs),
                         w4se = wave(step_mixed2d_kernel<4, true, true>, bs),
                         w4s2 = wave(step_mixed2d_kernel<4, true, true, true>, bs);
        auto grid = [nb](int w) { return nb < w ? nb : w; };
        const bool eq = p.time_scheme == 1 && wq.e != nullptr;
        const bool split = (s.work & W_SPLIT) != 0;
        // the configuration forms: diffusion off / constant / k-epsilon x
        // random number methods 1-3, without and with per-call outputs, for
        // runs without control sections
        static const SplitConfLaunch conf[2][3][3] = {
            {CG_CONF_ROW(0, false), CG_CONF_ROW(1, false), CG_CONF_ROW(2, false)},
            {CG_CONF_ROW(0, true), CG_CONF_ROW(1, true), CG_CONF_ROW(2, true)}};
#undef CG_CONF_ROW
        const int dc = p.diffmod == 0 ? 0 : (p.diffmod == 1 ? 1 : 2);
        if (split && eq && p.ncsec == 0 && p.rng_method >= 1 && p.rng_method <= 3 &&
            p.diffmod >= 0 && p.diffmod <= 3)
            conf[aux > 0][dc][p.rng_method - 1](m, f, p, s, wq, aux, step_index, stats, err, nb,
                                                bs, st);
        else if (split && eq && aux == 0)
            step_mixed2d_kernel<4, true, true><<<grid(w4se), bs, 0, st>>>(m, f, p, s, wq, aux,
                                                                        step_index, stats, err);
        else if (split && eq)
            step_mixed2d_kernel<4, true, true, true><<<grid(w4s2), bs, 0, st>>>(
                m, f, p, s, wq, aux, step_index, stats, err);
        else if (eq)
            step_mixed2d_kernel<4, false, true><<<grid(w4e), bs, 0, st>>>(m, f, p, s, wq, aux,
                                                                         step_index, stats, err);
        else if (split)
            step_mixed2d_kernel<3, true, false, true><<<grid(w3s), bs, 0, st>>>(
                m, f, p, s, wq, aux, step_index, stats, err);
        else
            step_mixed2d_kernel<3><<<grid(w3), bs, 0, st>>>(m, f, p, s, wq, aux, step_index,
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
    // programmatic dependent launch: the walk grid is set up while the step
    // kernel's last blocks run (they signal it at their start); its blocks
    // wait for the step grid to finish before reading the queue
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nsm * WALK_BLOCKS_PER_SM);
    cfg.blockDim = dim3(WALK_BLOCK);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, walk_kernel<float, true>, m, f, p, s, wq, aux, step_index, stats, err);
}

}  // namespace cg
