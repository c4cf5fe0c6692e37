// cg_serve_mixed.cu -- the serving pool's step kernel, mixed form.
// Compiled with FMA contraction like cg_kernels_mixed.cu, so that a served
// run rounds as the standalone mixed step does.
#include "cg_internal.h"
#include "cg_serve.cuh"

namespace cg {

int serve_grid_mixed() { return resident_blocks(serve_step_kernel<float, true>, 256); }

void launch_serve_mixed(int grid, const DevMesh& m, const FieldView& fv, const DevState& pool,
                        const ServeRun* runs, const int2* active, const int* nactive,
                        ServeClock* clk, uint32_t* run_err, cudaStream_t st) {
    serve_step_kernel<float, true><<<grid, 256, 0, st>>>(m, fv.as<float>(), pool, runs, active,
                                                            nactive, clk, run_err);
}

}  // namespace cg
