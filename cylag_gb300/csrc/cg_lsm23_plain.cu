// cg_lsm23_plain.cu -- the LSM2/LSM3 step kernels, plain form (FP64 end to end).
//
// One kernel per (dimension, model, time scheme) with the integrator
// inlined; kept out of the LSM1 units so that they compile in parallel.
// Compiled with -fmad=false like cg_kernels_plain.cu.
#include "cg_internal.h"
#include "cg_step.cuh"

namespace cg {

void launch_lsm23_plain(const DevMesh& m, const FieldView& fv, const DevParams& p,
                        const DevState& s, int aux, int step_index, int* stats, uint32_t* err,
                        cudaStream_t st) {
    DevFields<double> f = fv.as<double>();
    if (fv.dim == 2) launch_lsm23_kernel<2, double>(m, f, p, s, aux, step_index, stats, err, st);
    else launch_lsm23_kernel<3, double>(m, f, p, s, aux, step_index, stats, err, st);
}

}  // namespace cg
