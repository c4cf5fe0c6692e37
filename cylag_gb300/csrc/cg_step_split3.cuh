// cg_step_split3.cuh -- the mixed LSM2/LSM3 direct-integrator step over 3D
// element-sorted working copies whose positions are FP32 pairs hi + lo per
// coordinate (W_SPLIT3), velocities FP32 (W_V32).
//
// The generic step keeps FP64 positions: every step then forms the FP32
// offset to the element's anchor vertex with an FP64 subtraction and a
// conversion, adds the FP32 displacement back in FP64, converts again for
// the in-element test and the layer, and converts the velocities to and from
// FP64 -- about 40 float/double conversions and 17 FP64 adds per warp per
// step, each occupying the FP64 pipe (2 lanes per clock) 16 cycles whatever
// its active lanes.  Here the offsets are (x_hi - a_hi) + (x_lo - a_lo)
// against the element record's FP32-pair anchor (DevMesh::t64s, within
// 2^-23 of the exact offset, inside the barycentric bounds), the
// displacement is added by TwoSum in FP32 (48 significant bits), the
// in-element test and the first crossings are decided in FP32 (exact FP64
// only in the rounding band), and the integrator runs on FP32 state
// (di_lsm2_32 / di_lsm3_32, the same code as the generic mixed step).  The
// FP64 position is formed only for the full walk, the boundary conditions,
// control sections and the last step's last_position.
#pragma once

#include "cg_step_mixed.cuh"

namespace cg {

// DRAG >= 0: the form compiled for one run configuration, without control
// sections: DRAG the drag law, AM added mass or not; DIFF: for LSM3
// k-epsilon diffusion or not (KEPS of di_lsm3_32, with EDGE2), for LSM2 the
// diffusion model (0-3).
template <int MODEL, int DRAG = -1, int DIFF = -1, int EDGE2 = -1, int AM = -1>
__device__ __forceinline__ void split3_particle(const DevMesh& m, const DevFields<float>& f,
                                                const DevParams& p, DevState& s, int aux,
                                                int step_index, int* __restrict__ stats,
                                                uint32_t* __restrict__ err_word,
                                                const ZigTables& zt, const Zig32& z32, int i) {
    const int ncsec = DRAG >= 0 ? 0 : p.ncsec;
    const int tri0 = s.tri[i];
    if (tri0 < 0) return;   // inactive (-1) or awaiting initialization (-2)
    // every per-particle array is a working copy (W_VEL, W_FVS for LSM3,
    // W_LAYER, W_DIAM, W_AUXW): indexed by i
    Particle<3, float> q(m, f, p, zt);
    q.z32 = &z32;
    q.tri = q.tri0 = q.ltri = tri0;
    q.ll = q.ll0 = s.lowerlayer[i];
    q.rng.state = s.rng[i];
    q.rng.inc = ((uint64_t)(uint32_t)s.tag[i] << 1) | 1ULL;
    q.rng.err = 0;
    float2* P = reinterpret_cast<float2*>(s.pos) + 3 * (size_t)i;
    const float2 sx = P[0], sy = P[1], sz = P[2];
    float* V = reinterpret_cast<float*>(s.vel) + 3 * (size_t)i;
    float up[3] = {V[0], V[1], V[2]}, us[3] = {0.f, 0.f, 0.f};
    if constexpr (MODEL == 3) {
        const float* U = reinterpret_cast<const float*>(s.fvs) + 3 * (size_t)i;
        us[0] = U[0];
        us[1] = U[1];
        us[2] = U[2];
    }
    const float dp = (float)s.diameter[i];
    // start element: offset to its anchor vertex, barycentrics, P1 factors
    const Tri32S t0 = load_tri32s(m, tri0);
    const float4 xs = make_float4(sx.x, sy.x, sx.y, sy.y);
    const float2 r0 = split_offset(t0, xs);
    const Bary b0 = bary32_off(t0, r0.x, r0.y);
    float dx[3] = {0.f, 0.f, 0.f};
    if constexpr (MODEL == 2)
        di_lsm2_32<3, float, DRAG, AM>(q, q.p1f_of(t0, b0), sz.x + sz.y, dp,
                                       DIFF >= 0 ? DIFF : p.diffmod, p.nuopt, up, us, dx);
    else if (p.dt != 0.)   // update_state_lsm3.pyx: no update for a zero step
        di_lsm3_32<3, float, DRAG, DIFF, EDGE2, AM>(q, q.p1f_of(t0, b0), sz.x + sz.y, dp, up,
                                                    us, dx);
    // end position as FP32 pairs
    float2 ex = sx, ey = sy, ez = sz;
    split_add1(ex.x, ex.y, dx[0]);
    split_add1(ey.x, ey.y, dx[1]);
    split_add1(ez.x, ez.y, dx[2]);
    const float4 xe = make_float4(ex.x, ey.x, ex.y, ey.y);
    // xylocalizer.pyx:27-124: the start element, else the certain crossings
    // (hop_walk_split), else the FP32-filtered FP64 walk
    const float2 re = split_offset(t0, xe);
    Bary be = bary32_off(t0, re.x, re.y);
    int in0 = decide32(be);
    if (in0 < 0) in0 = in_tri(m, tri0, join1(ex), join1(ey)) ? 1 : 0;
    int kn = tri0, bnd = -1;
    if (!in0) {
        kn = hop_walk_split<MIXED_HOPS>(m, t0, b0, be, xe);
        if (kn < 0) xy_localize_filtered(m, tri0, join1(sx), join1(sy), join1(ex), join1(ey), kn, bnd);
    }
    q.tri = kn;
    // zlocalizer (the layer of the end point) from FP32 elevations
    const float ze = ez.x + ez.y;
    if (kn == tri0) {
        q.ll = q.z_localize32_q(q.p1f_of(t0, be), ze);
    } else if (kn >= 0) {
        const Tri32S tk = load_tri32s(m, kn);
        const float2 rk = split_offset(tk, xe);
        q.ll = q.z_localize32_q(q.p1f_of(tk, bary32_off(tk, rk.x, rk.y)), ze);
    } else {
        q.ll = PART_LOC_O;
    }
    const int a = aux_index(s, i);   // the caller's index (stranding records)
    // compute_bc.pyx:35-395 on the FP64 state, only where it acts: a wall or
    // open boundary crossed, the element left, or the bed or surface crossed
    if (bnd != -1 || q.tri == PART_LOC_O || q.ll == PART_LOC_B || q.ll == PART_LOC_A) {
        if (p.bc_on) {
            q.x0[0] = join1(sx);
            q.x0[1] = join1(sy);
            q.x0[2] = join1(sz);
            q.x[0] = join1(ex);
            q.x[1] = join1(ey);
            q.x[2] = join1(ez);
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                q.up[d] = up[d];
                q.us[d] = us[d];
            }
            q.pidx = a + s.base;
            q.pstep = step_index;
            q.compute_bc(bnd, stats);
            ex = split1(q.x[0]);
            ey = split1(q.x[1]);
            ez = split1(q.x[2]);
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                up[d] = (float)q.up[d];
                us[d] = (float)q.us[d];
            }
        } else if (q.tri == PART_LOC_O || q.ll == PART_LOC_B || q.ll == PART_LOC_A) {
            q.deleted = true;
        }
    }
    const uint32_t e = q.err | q.rng.err;
    if (e) atomicOr(err_word, e);
    // end of the step (solver.pyx:505-524), as Particle::store for these
    // working copies; deletion per lagrangian_particle_set.pyx:766-788
    if (q.deleted) {
        const float2 z2 = make_float2(0.f, 0.f);
        P[0] = z2;
        P[1] = z2;
        P[2] = z2;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            V[d] = 0.f;
            fvs_st(s, 3 * (size_t)i + d, 0.);
            s.last_pos[3 * (size_t)i + d] = 0.;
            s.last_vel[3 * (size_t)i + d] = 0.;
        }
        s.diameter[i] = 0.;
        s.tri[i] = -1;
        s.last_tri[i] = -1;
        s.lowerlayer[i] = 0;
        s.tag[i] = -2 - step_index;
        s.rng[i] = q.rng.state;
        if (ncsec) count_sections(p, stats, 0., 0., 0., 0.);
        return;
    }
    P[0] = ex;
    P[1] = ey;
    P[2] = ez;
    s.tri[i] = q.tri;
    s.lowerlayer[i] = q.ll;
    s.rng[i] = q.rng.state;
    if (aux >= 2) {
        // the velocity this step started from (still in the working copy)
#pragma unroll
        for (int d = 0; d < 3; ++d) s.last_vel[3 * (size_t)i + d] = (double)V[d];
        s.last_pos[3 * (size_t)i] = join1(sx);
        s.last_pos[3 * (size_t)i + 1] = join1(sy);
        s.last_pos[3 * (size_t)i + 2] = join1(sz);
        s.last_tri[i] = tri0;
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) V[d] = up[d];
    if (MODEL == 3 || aux >= 1) {
#pragma unroll
        for (int d = 0; d < 3; ++d) fvs_st(s, 3 * (size_t)i + d, (double)us[d]);
    }
    if (ncsec) count_sections(p, stats, join1(sx), join1(sy), join1(ex), join1(ey));
}

// One step of every particle of a W_SPLIT3 run (persistent grid), MODEL 2 or
// 3: two resident blocks of 256 per SM for LSM2, as the generic mixed
// LSM2/LSM3 kernels; three for LSM3 (85 registers, spilling; 2% faster
// than two on the LSM3 workload, where LSM2 is 8% slower with three), four
// for the LSM3 configuration forms (64 registers, spilling; 3% faster than
// three).
template <int MODEL, int DRAG = -1, int DIFF = -1, int EDGE2 = -1, int AM = -1>
__global__ void __launch_bounds__(256, MODEL == 3 ? (DRAG >= 0 ? 4 : 3) : 2) step_split3_kernel(DevMesh m, DevFields<float> f,
                                                             DevParams p, DevState s, int aux,
                                                             int step_index,
                                                             int* __restrict__ stats,
                                                             uint32_t* __restrict__ err_word) {
    __shared__ ZigTables zt;
    __shared__ Zig32 z32;
    for (int t = threadIdx.x; t < 128; t += blockDim.x) {
        z32.kn[t] = g_zig.kn[t];
        z32.wn[t] = (float)g_zig.wn[t];
        z32.fn[t] = (float)g_zig.fn[t];
    }
    load_zig(zt);   // ends with __syncthreads
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < s.n; i += gridDim.x * blockDim.x)
        split3_particle<MODEL, DRAG, DIFF, EDGE2, AM>(m, f, p, s, aux, step_index, stats,
                                                      err_word, zt, z32, i);
}

// The forms compiled for one run configuration, for runs without control
// sections: the drag law (drag_coefficient_model 0 or 1) and added mass or
// not, and for LSM3 k-epsilon diffusion (diffusion model 2 or 3) or not and
// lsm3_edge_opt 2 (clipped coefficients) or not: form K = 8 DRAG + 4 KEPS +
// 2 EDGE2 + AM (0-15); for LSM2 the diffusion model DM: form K = 16 + 8 DRAG
// + 2 DM + AM (16-31).  launch_split3_form<K> is defined in
// cg_split3_form.cu, which the build compiles once per form: alone in its
// unit, the form's kernel gets the inlining decisions of a single call site.
template <int K>
void launch_split3_form(const DevMesh& m, const DevFields<float>& f, const DevParams& p,
                      const DevState& s, int aux, int step_index, int* stats, uint32_t* err,
                      cudaStream_t st);

}  // namespace cg
