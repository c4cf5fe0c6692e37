// cg_kernels_mixed.cu -- the mixed-precision form (FP32 fields and
// increments, FP64 positions and localization decisions).  Compiled with
// the default FMA contraction; the exact FP64 predicates it shares with the
// plain form are written with _rn intrinsics and are not contracted.
#include "cg_internal.h"
#include "cg_step_mixed.cuh"

namespace cg {

void launch_step_mixed(int dim, const DevMesh& m, const void* cur, const void* prev, int npoints,
                       int nlayers, int prev_valid, const DevParams& p, const DevState& s,
                       const WalkQueue& wq, int aux, int step_index, int* stats, uint32_t* err,
                       cudaStream_t st) {
    int bs = 256;
    int nb = (s.n + bs - 1) / bs;
    if (nb == 0) return;
    if (dim == 2) {
        DevFields<float> f{(const float*)cur, (const float*)prev, npoints, nlayers, 2, prev_valid};
        step_mixed2d_kernel<<<nb, bs, 0, st>>>(m, f, p, s, wq, aux, step_index, stats, err);
    } else {
        // 3D: FP32 node records, FP64 arithmetic
        DevFields<float> f{(const float*)cur, (const float*)prev, npoints, nlayers, 3, prev_valid};
        WalkQueue none{nullptr, nullptr};
        step_kernel<3, float><<<nb, bs, 0, st>>>(m, f, p, s, none, aux, step_index, stats, err);
    }
}

}  // namespace cg
