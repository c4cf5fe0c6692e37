// cg_sort.cu -- periodic re-sort of the particles by element id.
//
// Particles that share an element then sit in the same warps, so the
// element's mesh record and node values are fetched once per warp instead
// of once per particle, and the neighbour walks touch few distinct lines.
// The reference never reorders particles; the sort is invisible to callers:
// a call of several steps gathers the state into working copies in element
// order, re-sorts them every few steps (a nearly coherent gather, since
// particles move little between sorts) and scatters the results back to the
// caller's slots when it returns.  Every per-particle computation is
// independent of the order, so results do not depend on the sort.
//
// Counting sort on the key tri (in 3D tri * layers + layer; inactive and
// uninitialized particles, tri < 0, get the last key):
//   1. histogram of the keys (global atomics),
//   2. exclusive scan of the nt+1 counts (warp-shuffle block scans, then a
//      scan of the block sums, then the carry-in),
//   3. scatter of the particle indices (one atomic per particle),
//   4. gather of the working state in the new order.
#include "cg_internal.h"

namespace cg {

constexpr int SCAN_BLOCK = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_BLOCK * SCAN_ITEMS;

// key of a particle: its element (and, in 3D, its layer within the
// column); inactive and uninitialized particles (tri < 0) go last
__device__ __forceinline__ int sort_key(int tri, int layer, int nt, int nl) {
    if (tri < 0) return nt * nl;
    int l = layer < 0 ? 0 : (layer >= nl ? nl - 1 : layer);
    return tri * nl + l;
}

// Keys of neighbouring particles mostly agree (the particles are sorted but
// for the last period's moves): the lanes of a warp with the same key add
// their count with one atomic.
__global__ void hist_kernel(const int* __restrict__ tri, const int* __restrict__ layer, int n,
                            int nt, int nl, int* __restrict__ count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int key = i < n ? sort_key(__ldg(&tri[i]), layer ? __ldg(&layer[i]) : 0, nt, nl) : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    if (key >= 0 && (threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&count[key], __popc(peers));
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

__global__ void scatter_index_kernel(const int* __restrict__ tri, const int* __restrict__ layer,
                                     int n, int nt, int nl, int* __restrict__ offset,
                                     int* __restrict__ perm) {
    // one atomic per key and warp; the lanes of a key keep their order
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const int key = i < n ? sort_key(__ldg(&tri[i]), layer ? __ldg(&layer[i]) : 0, nt, nl) : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const int leader = __ffs(peers) - 1;
    int base = 0;
    if (key >= 0 && lane == leader) base = atomicAdd(&offset[key], __popc(peers));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (key >= 0) perm[base + __popc(peers & ((1u << lane) - 1u))] = i;
}

template <typename T>
__device__ __forceinline__ void move_rows(const T* __restrict__ src, T* __restrict__ dst, int from,
                                          int to, int dim) {
    for (int d = 0; d < dim; ++d) dst[(size_t)to * dim + d] = __ldcs(src + (size_t)from * dim + d);
}

// velocity rows: FP64 in the caller's arrays, FP32 in working copies under
// W_V32 (converted on the way in from the caller's arrays)
__device__ __forceinline__ void move_vel_rows(const double* __restrict__ src,
                                              double* __restrict__ dst, int from, int to,
                                              int dim, bool v32, bool from_caller) {
    if (!v32) {
        move_rows(src, dst, from, to, dim);
        return;
    }
    float* d32 = reinterpret_cast<float*>(dst);
    if (from_caller) {
        for (int d = 0; d < dim; ++d)
            d32[(size_t)to * dim + d] = (float)__ldcs(src + (size_t)from * dim + d);
    } else {
        move_rows(reinterpret_cast<const float*>(src), d32, from, to, dim);
    }
}

// working velocity row j -> the caller's FP64 row i
__device__ __forceinline__ void put_vel_rows(const double* __restrict__ w, double* __restrict__ user,
                                             int j, int i, int dim, bool v32) {
    for (int d = 0; d < dim; ++d) {
        const size_t k = (size_t)j * dim + d;
        __stcs(user + (size_t)i * dim + d, v32 ? (double)reinterpret_cast<const float*>(w)[k] : w[k]);
    }
}

// dst[j] = src[perm[j]]; src.slot == nullptr: the source is the caller's arrays.
// split: working positions are split FP32 pairs (W_SPLIT), made from the
// caller's FP64 positions here and moved as they are between working copies.
// The outputs kept with W_AUXW are not moved: dst's last element becomes
// LAST_UNSET, or stays -1 for a particle deleted since the last write-back
// (its outputs are zero).
// W_VEL2 re-sorts move the newest velocity array alone (vpar): the other one
// is the next velocity-writing step's target, and every call ends with such
// a step (the last one, after any re-sort of the call), before any read.
__global__ void gather_state_kernel(const int* __restrict__ perm, WorkState src, WorkState dst,
                                    int n, int dim, int work, int vpar) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    int i = __ldg(&perm[j]);
    const bool split = (work & W_SPLIT) != 0;
    if (split && src.slot == nullptr) {
        const double2 x = __ldcs(reinterpret_cast<const double2*>(src.pos) + i);
        reinterpret_cast<float4*>(dst.pos)[j] = split_pos(x.x, x.y);
    } else if ((work & W_SPLIT3) && src.slot == nullptr) {
        for (int d = 0; d < dim; ++d)
            reinterpret_cast<float2*>(dst.pos)[(size_t)j * dim + d] =
                split1(__ldcs(src.pos + (size_t)i * dim + d));
    } else {
        move_rows(src.pos, dst.pos, i, j, dim);
    }
    dst.tri[j] = __ldcs(src.tri + i);
    dst.tag[j] = __ldcs(src.tag + i);
    dst.rng[j] = __ldcs(src.rng + i);
    dst.slot[j] = src.slot ? __ldcs(src.slot + i) : i;
    const bool v32 = (work & W_V32) != 0, from_caller = src.slot == nullptr;
    if ((work & W_VEL2) && !from_caller) {
        if (vpar) move_rows(src.vel2, dst.vel2, i, j, dim);
        else move_rows(src.vel, dst.vel, i, j, dim);
    } else if (work & W_VEL) {
        move_vel_rows(src.vel, dst.vel, i, j, dim, v32, from_caller);
    }
    if (work & W_FVS) move_vel_rows(src.fvs, dst.fvs, i, j, dim, v32, from_caller);
    if (work & W_LAYER) dst.layer[j] = __ldcs(src.layer + i);
    if (work & W_DIAM) dst.diam[j] = __ldcs(src.diam + i);
    if (work & W_AUXW)
        dst.ltri[j] = (src.slot != nullptr && __ldcs(src.ltri + i) == -1) ? -1 : LAST_UNSET;
}

// caller[slot[j]] = work[j]; the W_AUXW outputs only where a step set them
__global__ void scatter_state_kernel(WorkState w, WorkState user, int n, int dim, int work,
                                     int vpar) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    int i = __ldg(&w.slot[j]);
    if (work & W_SPLIT)
        __stcs(reinterpret_cast<double2*>(user.pos) + i,
               join_pos(reinterpret_cast<const float4*>(w.pos)[j]));
    else if (work & W_SPLIT3)
        for (int d = 0; d < dim; ++d)
            __stcs(user.pos + (size_t)i * dim + d,
                   join1(reinterpret_cast<const float2*>(w.pos)[(size_t)j * dim + d]));
    else
        for (int d = 0; d < dim; ++d)
            __stcs(user.pos + (size_t)i * dim + d, w.pos[(size_t)j * dim + d]);
    __stcs(user.tri + i, w.tri[j]);
    __stcs(user.tag + i, w.tag[j]);
    __stcs(user.rng + i, w.rng[j]);
    const bool v32 = (work & W_V32) != 0;
    // W_VEL2: the newest velocity and the one before it
    const double* vnew = ((work & W_VEL2) && vpar) ? w.vel2 : w.vel;
    const double* vold = ((work & W_VEL2) && vpar) ? w.vel : w.vel2;
    if ((work & W_VEL2) && w.tri[j] == -1) {
        // inactive: zero velocity (the arrays are written only by the steps
        // that output the velocity)
        for (int d = 0; d < dim; ++d) __stcs(user.vel + (size_t)i * dim + d, 0.);
    } else if (work & W_VEL) {
        put_vel_rows(vnew, user.vel, j, i, dim, v32);
    }
    if (work & W_FVS) put_vel_rows(w.fvs, user.fvs, j, i, dim, v32);
    if (work & W_LAYER) __stcs(user.layer + i, w.layer[j]);
    if (work & W_DIAM) __stcs(user.diam + i, w.diam[j]);
    if (work & W_AUXW) {
        const int lt = w.ltri[j];
        if (lt == LAST_UNSET) return;
        const bool del = lt == -1;
        const bool two = (work & W_VEL2) != 0;
        for (int d = 0; d < dim; ++d) {
            const size_t u = (size_t)i * dim + d, k = (size_t)j * dim + d;
            __stcs(user.lpos + u, del ? 0. : w.lpos[k]);
            __stcs(user.lvel + u, del ? 0. : (two ? vold[k] : w.lvel[k]));
            if (!(work & W_FVS)) __stcs(user.fvs + u, del ? 0. : (two ? vnew[k] : w.fvs[k]));
        }
        __stcs(user.ltri + i, lt);
    }
}

int scan_scratch_ints(int nkeys) { return (nkeys + SCAN_TILE - 1) / SCAN_TILE; }

static void sort_perm(const int* tri, const int* layer, int n, int nt, SortBuffers& b,
                      cudaStream_t st) {
    int nkeys = nt * b.nl + 1;
    int bs = 256;
    cudaMemsetAsync(b.count, 0, (size_t)nkeys * sizeof(int), st);
    hist_kernel<<<(n + bs - 1) / bs, bs, 0, st>>>(tri, layer, n, nt, b.nl, b.count);
    int ntiles = scan_scratch_ints(nkeys);
    scan_tiles_kernel<<<ntiles, SCAN_BLOCK, 0, st>>>(b.count, nkeys, b.block_sums);
    scan_sums_kernel<<<1, SCAN_BLOCK, 0, st>>>(b.block_sums, ntiles);
    add_carry_kernel<<<(nkeys + bs - 1) / bs, bs, 0, st>>>(b.count, nkeys, b.block_sums);
    scatter_index_kernel<<<(n + bs - 1) / bs, bs, 0, st>>>(tri, layer, n, nt, b.nl, b.count, b.perm);
}

// the caller's arrays seen as a working state
static WorkState user_view(const DevState& u) {
    WorkState w;
    w.pos = u.pos;
    w.tri = u.tri;
    w.tag = u.tag;
    w.rng = reinterpret_cast<unsigned long long*>(u.rng);
    w.slot = nullptr;
    w.vel = u.vel;
    w.vel2 = nullptr;
    w.fvs = u.fvs;
    w.layer = u.lowerlayer;
    w.diam = u.diameter;
    w.lpos = u.last_pos;
    w.lvel = u.last_vel;
    w.ltri = u.last_tri;
    return w;
}

void launch_sort_gather(const DevState& user, int nt, SortBuffers& b, cudaStream_t st) {
    b.vpar = 0;   // the caller's velocity lands in vel
    int n = user.n;
    if (n == 0) return;
    sort_perm(user.tri, (b.work & W_LAYER) ? user.lowerlayer : nullptr, n, nt, b, st);
    gather_state_kernel<<<(n + 255) / 256, 256, 0, st>>>(b.perm, user_view(user), b.a, n, b.dim,
                                                         b.work, 0);
}

void launch_sort_resort(int n, int nt, SortBuffers& b, cudaStream_t st) {
    if (n == 0) return;
    sort_perm(b.a.tri, b.a.layer, n, nt, b, st);
    gather_state_kernel<<<(n + 255) / 256, 256, 0, st>>>(b.perm, b.a, b.b, n, b.dim, b.work,
                                                         b.vpar);
    WorkState t = b.a;
    b.a = b.b;
    b.b = t;
}

void launch_sort_scatter(const DevState& user, const SortBuffers& b, cudaStream_t st) {
    int n = user.n;
    if (n == 0) return;
    scatter_state_kernel<<<(n + 255) / 256, 256, 0, st>>>(b.a, user_view(user), n, b.dim,
                                                          b.work, b.vpar);
}

DevState sorted_view(const DevState& user, const SortBuffers& b) {
    DevState w = user;
    w.pos = b.a.pos;
    w.tri = b.a.tri;
    w.tag = b.a.tag;
    w.rng = reinterpret_cast<uint64_t*>(b.a.rng);
    w.slot = b.a.slot;
    // W_VEL2: a step that writes the velocity writes the older array (the
    // run then flips vpar); no kernel reads it
    if (b.work & W_VEL) w.vel = ((b.work & W_VEL2) && !b.vpar) ? b.a.vel2 : b.a.vel;
    if (b.work & (W_FVS | W_AUXW)) w.fvs = b.a.fvs;
    if (b.work & W_LAYER) w.lowerlayer = b.a.layer;
    if (b.work & W_DIAM) w.diameter = b.a.diam;
    if (b.work & W_AUXW) {
        w.last_pos = b.a.lpos;
        w.last_vel = b.a.lvel;
        w.last_tri = b.a.ltri;
    }
    w.work = b.work;
    return w;
}

}  // namespace cg
