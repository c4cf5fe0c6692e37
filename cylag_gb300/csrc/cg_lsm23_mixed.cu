// cg_lsm23_mixed.cu -- the LSM2/LSM3 step kernels, mixed form (FP32 node records and Langevin coefficients).
//
// One kernel per (dimension, model, time scheme) with the integrator
// inlined, and the 3D direct-integrator kernels over FP32-pair working
// positions; kept out of the LSM1 units so that they compile in parallel.
// Compiled with FMA contraction like cg_kernels_mixed.cu.
#include "cg_internal.h"
#include "cg_step.cuh"
#include "cg_step_split3.cuh"

namespace cg {

void launch_lsm23_mixed(const DevMesh& m, const FieldView& fv, const DevParams& p,
                        const DevState& s, int aux, int step_index, int* stats, uint32_t* err,
                        cudaStream_t st) {
    DevFields<float> f = fv.as<float>();
    // 3D direct integrators over FP32-pair working positions
    if (s.work & W_SPLIT3) return launch_split3_kernel(m, f, p, s, aux, step_index, stats, err, st);
    if (fv.dim == 2) launch_lsm23_kernel<2, float>(m, f, p, s, aux, step_index, stats, err, st);
    else launch_lsm23_kernel<3, float>(m, f, p, s, aux, step_index, stats, err, st);
}

}  // namespace cg
