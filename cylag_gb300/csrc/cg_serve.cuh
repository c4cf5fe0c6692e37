// cg_serve.cuh -- one step of every admitted dispersion run in one launch.
//
// The serving pool holds the particles of many runs in one set of device
// arrays; each run owns a range of whole warps (32 particles), so a warp
// never mixes runs and every lane of a warp follows the same run's model
// and parameters.  The kernel strides over the list of active warps
// {warp, run}; a run's step index is the global step minus the step at which
// it was admitted, so finished runs (and runs admitted later) are skipped
// without host involvement, and the kernel itself advances the global step
// (the last block to finish).  The launch arguments never change, which is
// what lets the step be captured once in a CUDA graph and replayed.
//
// Per particle the work is exactly that of a standalone run's step kernel
// (step_particle / step_mixed_particle with the walk inline), so a run's
// result does not depend on which other runs share the launch.
#pragma once

#include "cg_internal.h"
#include "cg_step_mixed.cuh"

namespace cg {

// ServeRun and ServeClock: cg_internal.h

// one LSM2/LSM3 particle of a served run, out of line: each variant keeps
// its own register allocation and the kernel's LSM1 path stays lean
template <typename FT, int MODEL, int SCHEME>
__device__ __noinline__ void serve_particle(const DevMesh& m, const DevFields<FT>& f,
                                            const DevParams& p, DevState& pool, int aux, int k,
                                            uint32_t* err, const ZigTables& zt, int i,
                                            const Zig32* z32) {
    const WalkQueue none{nullptr, nullptr};
    step_particle<2, FT, MODEL, SCHEME>(m, f, p, pool, none, aux, k, nullptr, err, zt, i, z32);
}

// the mixed form is bounded to two resident blocks of 256 per SM (128
// registers), as the step kernels of the mixed LSM2/LSM3 runs it steps
template <typename FT, bool MIXED>
__global__ void __launch_bounds__(256, MIXED ? 2 : 1) serve_step_kernel(DevMesh m, DevFields<FT> f, DevState pool,
                                                         const ServeRun* __restrict__ runs,
                                                         const int2* __restrict__ active,
                                                         const int* __restrict__ nactive,
                                                         ServeClock* clk,
                                                         uint32_t* __restrict__ run_err) {
    __shared__ ZigTables zt;
    __shared__ Zig32 z32;
    if constexpr (MIXED) {
        for (int t = threadIdx.x; t < 128; t += blockDim.x) {
            z32.kn[t] = g_zig.kn[t];
            z32.wn[t] = (float)g_zig.wn[t];
            z32.fn[t] = (float)g_zig.fn[t];
        }
    }
    load_zig(zt);   // ends with __syncthreads
    const Zig32* z32p = MIXED ? &z32 : nullptr;
    const unsigned long long g = *(volatile unsigned long long*)&clk->gstep;
    const int na = *nactive;
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const WalkQueue none{nullptr, nullptr};
    for (int a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; a < na; a += nw) {
        const int2 e = active[a];   // {warp, run}
        const ServeRun& R = runs[e.y];
        const long long k = (long long)g - R.start;
        const int i = e.x * 32 + lane;
        if (k < 0 || k >= R.horizon || i >= R.first + R.count) continue;
        const int aux = (k == R.horizon - 1) ? 2 : (k == R.horizon - 2 ? 1 : 0);
        uint32_t* err = run_err + e.y;
        const int model = R.p.model;
        if constexpr (MIXED) {
            if (model == 1) {
                step_mixed_particle<false>(m, f, R.p, pool, none, aux, (int)k, nullptr, err, z32,
                                           load_mixed_in(pool, i), i);
                continue;
            }
        }
        const int ts = R.p.time_scheme, kk = (int)k;
        if (model == 1)
            step_particle<2, FT, 1>(m, f, R.p, pool, none, aux, kk, nullptr, err, zt, i);
        else if (model == 2 && ts == 5) serve_particle<FT, 2, 5>(m, f, R.p, pool, aux, kk, err, zt, i, z32p);
        else if (model == 2 && ts == 1) serve_particle<FT, 2, 1>(m, f, R.p, pool, aux, kk, err, zt, i, z32p);
        else if (model == 2 && ts == 2) serve_particle<FT, 2, 2>(m, f, R.p, pool, aux, kk, err, zt, i, z32p);
        else if (model == 2 && ts == 3) serve_particle<FT, 2, 3>(m, f, R.p, pool, aux, kk, err, zt, i, z32p);
        else if (model == 2) serve_particle<FT, 2, 4>(m, f, R.p, pool, aux, kk, err, zt, i, z32p);
        else if (ts == 5) serve_particle<FT, 3, 5>(m, f, R.p, pool, aux, kk, err, zt, i, z32p);
        else serve_particle<FT, 3, 1>(m, f, R.p, pool, aux, kk, err, zt, i, z32p);
    }
    // the last block to finish advances the global step
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned int t = atomicAdd(&clk->done, 1u);
        if (t == gridDim.x - 1) {
            clk->done = 0;
            clk->gstep = g + 1;
            __threadfence();
        }
    }
}


}  // namespace cg
