// cg_serve_plain.cu -- the serving pool's step kernel, plain form.
// Compiled with -fmad=false like cg_kernels_plain.cu, so that a served run
// rounds as the standalone plain step does.
#include "cg_internal.h"
#include "cg_serve.cuh"

namespace cg {

int serve_grid_plain() { return resident_blocks(serve_step_kernel<double, false>, 256); }

void launch_serve_plain(int grid, const DevMesh& m, const FieldView& fv, const DevState& pool,
                        const ServeRun* runs, const int2* active, const int* nactive,
                        ServeClock* clk, uint32_t* run_err, cudaStream_t st) {
    serve_step_kernel<double, false><<<grid, 256, 0, st>>>(m, fv.as<double>(), pool, runs, active,
                                                            nactive, clk, run_err);
}

}  // namespace cg
