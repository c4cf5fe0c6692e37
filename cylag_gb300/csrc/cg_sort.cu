// cg_sort.cu -- periodic re-sort of the particles by element id.
//
// Particles that share an element then sit in the same warps, so the
// element's mesh record and node values are fetched once per warp instead
// of once per particle, and the neighbour walks touch few distinct lines.
// The reference never reorders particles; the sort is invisible to callers:
// the step runs on working copies in sorted order and the results are
// scattered back to the caller's slots at the end of each chunk of steps
// (every per-particle computation is independent of the order).
//
// Counting sort on the key tri (inactive and uninitialized particles, tri <
// 0, get the key nt and go last):
//   1. histogram of the keys (global atomics),
//   2. exclusive scan of the nt+1 counts (warp-shuffle block scans, then a
//      scan of the block sums, then the carry-in),
//   3. scatter of the particle indices (one atomic per particle),
//   4. gather of the working state in sorted order.
#include "cg_internal.h"

namespace cg {

constexpr int SCAN_BLOCK = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_BLOCK * SCAN_ITEMS;

__device__ __forceinline__ int sort_key(int tri, int nt) { return tri >= 0 ? tri : nt; }

__global__ void hist_kernel(const int* __restrict__ tri, int n, int nt, int* __restrict__ count) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) atomicAdd(&count[sort_key(__ldg(&tri[i]), nt)], 1);
}

// inclusive warp scan
__device__ __forceinline__ int warp_scan(int v) {
    int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// exclusive scan of one tile of SCAN_TILE values in place; block total to sums[blockIdx.x]
__global__ void __launch_bounds__(SCAN_BLOCK) scan_tiles_kernel(int* __restrict__ v, int n,
                                                                int* __restrict__ sums) {
    __shared__ int warp_tot[SCAN_BLOCK / 32];
    int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    int x[SCAN_ITEMS];
    int run = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        x[k] = (base + k < n) ? v[base + k] : 0;
        run += x[k];
    }
    int inc = warp_scan(run);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 31) warp_tot[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        int w = warp_tot[lane];
        int wi = warp_scan(w);
        warp_tot[lane] = wi - w;   // exclusive warp offsets
    }
    __syncthreads();
    int off = warp_tot[wid] + inc - run;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        if (base + k < n) v[base + k] = off;
        off += x[k];
    }
    if (threadIdx.x == SCAN_BLOCK - 1) sums[blockIdx.x] = off;
}

// exclusive scan of the block sums (one block; nblocks <= SCAN_TILE)
__global__ void __launch_bounds__(SCAN_BLOCK) scan_sums_kernel(int* __restrict__ sums, int nb) {
    __shared__ int warp_tot[SCAN_BLOCK / 32];
    int base = threadIdx.x * SCAN_ITEMS;
    int x[SCAN_ITEMS];
    int run = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        x[k] = (base + k < nb) ? sums[base + k] : 0;
        run += x[k];
    }
    int inc = warp_scan(run);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 31) warp_tot[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        int w = warp_tot[lane];
        int wi = warp_scan(w);
        warp_tot[lane] = wi - w;
    }
    __syncthreads();
    int off = warp_tot[wid] + inc - run;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        if (base + k < nb) sums[base + k] = off;
        off += x[k];
    }
}

__global__ void add_carry_kernel(int* __restrict__ v, int n, const int* __restrict__ sums) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] += sums[i / SCAN_TILE];
}

__global__ void scatter_index_kernel(const int* __restrict__ tri, int n, int nt,
                                     int* __restrict__ offset, int* __restrict__ perm) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) perm[atomicAdd(&offset[sort_key(__ldg(&tri[i]), nt)], 1)] = i;
}

__global__ void gather_state_kernel(SortBuffers b, DevState user, int n) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    int i = __ldg(&b.perm[j]);
    b.pos[j] = __ldcs(reinterpret_cast<const double2*>(user.pos) + i);
    b.tri[j] = __ldcs(&user.tri[i]);
    b.tag[j] = __ldcs(&user.tag[i]);
    b.rng[j] = __ldcs(reinterpret_cast<const unsigned long long*>(user.rng) + i);
}

__global__ void scatter_state_kernel(SortBuffers b, DevState user, int n) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    int i = __ldg(&b.perm[j]);
    __stcs(reinterpret_cast<double2*>(user.pos) + i, b.pos[j]);
    __stcs(&user.tri[i], b.tri[j]);
    __stcs(&user.tag[i], b.tag[j]);
    __stcs(reinterpret_cast<unsigned long long*>(user.rng) + i, b.rng[j]);
}

int scan_scratch_ints(int nkeys) { return (nkeys + SCAN_TILE - 1) / SCAN_TILE; }

void launch_sort_gather(const DevState& user, int nt, const SortBuffers& b, cudaStream_t st) {
    int n = user.n;
    if (n == 0) return;
    int nkeys = nt + 1;
    int bs = 256;
    cudaMemsetAsync(b.count, 0, (size_t)nkeys * sizeof(int), st);
    hist_kernel<<<(n + bs - 1) / bs, bs, 0, st>>>(user.tri, n, nt, b.count);
    int ntiles = scan_scratch_ints(nkeys);
    scan_tiles_kernel<<<ntiles, SCAN_BLOCK, 0, st>>>(b.count, nkeys, b.block_sums);
    scan_sums_kernel<<<1, SCAN_BLOCK, 0, st>>>(b.block_sums, ntiles);
    add_carry_kernel<<<(nkeys + bs - 1) / bs, bs, 0, st>>>(b.count, nkeys, b.block_sums);
    scatter_index_kernel<<<(n + bs - 1) / bs, bs, 0, st>>>(user.tri, n, nt, b.count, b.perm);
    gather_state_kernel<<<(n + bs - 1) / bs, bs, 0, st>>>(b, user, n);
}

void launch_sort_scatter(const DevState& user, const SortBuffers& b, cudaStream_t st) {
    int n = user.n;
    if (n == 0) return;
    int bs = 256;
    scatter_state_kernel<<<(n + bs - 1) / bs, bs, 0, st>>>(b, user, n);
}

}  // namespace cg
