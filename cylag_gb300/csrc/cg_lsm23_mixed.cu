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

// The split 3D step (W_SPLIT3): the form compiled for the run's
// configuration when there is one (launch_split3_form), else the general
// kernels (persistent grid).
static void launch_split3_kernel(const DevMesh& m, const DevFields<float>& f,
                                 const DevParams& p, const DevState& s, int aux, int step_index,
                                 int* stats, uint32_t* err, cudaStream_t st) {
    using Form = void (*)(const DevMesh&, const DevFields<float>&, const DevParams&,
                          const DevState&, int, int, int*, uint32_t*, cudaStream_t);
#define CG_FORMS8(B)                                                                   \
    launch_split3_form<B>, launch_split3_form<B + 1>, launch_split3_form<B + 2>,           \
        launch_split3_form<B + 3>, launch_split3_form<B + 4>, launch_split3_form<B + 5>,   \
        launch_split3_form<B + 6>, launch_split3_form<B + 7>
    static const Form forms[32] = {CG_FORMS8(0), CG_FORMS8(8), CG_FORMS8(16), CG_FORMS8(24)};
#undef CG_FORMS8
    if (p.ncsec == 0 && (p.drag_model == 0 || p.drag_model == 1)) {
        const int am = p.added_mass ? 1 : 0;
        if (p.model == 3) {
            const int keps = (p.diffmod == 2 || p.diffmod == 3) ? 1 : 0;
            forms[8 * p.drag_model + 4 * keps + 2 * (p.edge_opt == 2 ? 1 : 0) + am](
                m, f, p, s, aux, step_index, stats, err, st);
            return;
        }
        if (p.model == 2 && p.diffmod >= 0 && p.diffmod <= 3) {
            forms[16 + 8 * p.drag_model + 2 * p.diffmod + am](m, f, p, s, aux, step_index, stats,
                                                              err, st);
            return;
        }
    }
    const int bs = 256;
    const int need = (s.n + bs - 1) / bs;
    if (need == 0) return;
    static int wave2 = 0, wave3 = 0;
    if (p.model == 2) {
        if (!wave2) wave2 = resident_blocks(step_split3_kernel<2>, bs);
        step_split3_kernel<2><<<need < wave2 ? need : wave2, bs, 0, st>>>(m, f, p, s, aux,
                                                                         step_index, stats, err);
    } else {
        if (!wave3) wave3 = resident_blocks(step_split3_kernel<3>, bs);
        step_split3_kernel<3><<<need < wave3 ? need : wave3, bs, 0, st>>>(m, f, p, s, aux,
                                                                         step_index, stats, err);
    }
}

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
