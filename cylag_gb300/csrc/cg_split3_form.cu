// cg_split3_form.cu -- one form of the split 3D LSM3 or LSM2 step, compiled
// for one run configuration (launch_split3_form, cg_step_split3.cuh).  The
// build compiles this file once per form, with CG_FORM = 8 DRAG + 4 KEPS + 2
// EDGE2 + AM (LSM3, 0..15) or 16 + 8 DRAG + 2 DM + AM (LSM2, 16..31), so
// that each form's kernel is the only kernel of its unit.  The arithmetic
// is that of the general kernel; a form drops the tests of these parameters
// and the code of the other branches (the Almedeij drag law in FP64, the
// k-epsilon time scale, the added-mass acceleration, the other Cholesky
// factorization), which keeps the kernel's instruction footprint and
// register use down.  A run steps every step with the same form.  (The LSM2
// forms of diffusion model 0 complete the index range; such runs do not
// take the split kernels, whose LSM2 runs have velocity diffusion.)
#include "cg_internal.h"
#include "cg_step_split3.cuh"

#ifndef CG_FORM
#error "cg_split3_form.cu is compiled once per form with -DCG_FORM=0..31"
#endif

namespace cg {

template <>
void launch_split3_form<CG_FORM>(const DevMesh& m, const DevFields<float>& f,
                                 const DevParams& p, const DevState& s, int aux, int step_index,
                                 int* stats, uint32_t* err, cudaStream_t st) {
    constexpr int LSM2 = CG_FORM >= 16, K = CG_FORM - 16 * LSM2;
    constexpr int MODEL = LSM2 ? 2 : 3, DRAG = (K >> 3) & 1, AM = K & 1;
    constexpr int DIFF = LSM2 ? (K >> 1) & 3 : (K >> 2) & 1, EDGE2 = LSM2 ? -1 : (K >> 1) & 1;
    const int bs = 256;
    const int need = (s.n + bs - 1) / bs;
    if (need == 0) return;
    static const int wave =
        resident_blocks(step_split3_kernel<MODEL, DRAG, DIFF, EDGE2, AM>, bs);
    step_split3_kernel<MODEL, DRAG, DIFF, EDGE2, AM><<<need < wave ? need : wave, bs, 0, st>>>(
        m, f, p, s, aux, step_index, stats, err);
}

}  // namespace cg
