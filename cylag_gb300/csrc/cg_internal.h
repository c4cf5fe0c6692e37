// cg_internal.h -- launchers shared between the C-ABI layer (cg_api.cu) and
// the kernel translation units.  Not part of the public ABI.
#pragma once

#include <cstdint>

#include <nvtx3/nvToolsExt.h>
#include <cuda_runtime.h>

#include "cg_device.cuh"

namespace cg {

// An NVTX range for the scope (shown by Nsight tools, free otherwise):
// the library's host phases -- a step call, the element sort, admissions
// and steps of the serving pool -- appear on the timeline by name.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// Raw node fields on the device, planar: frames[t][f][node] for the raw
// field ids below (absent fields are not stored; raw_slot[f] == -1).
enum RawField { RF_ZS = 0, RF_UX, RF_UY, RF_UZ, RF_KT, RF_EP, RF_ZB, RF_COUNT };

struct DevFrames {
    const double* frames;   // [ntimes][nraw][nnodes]
    const float* frames32;  // the same rounded to FP32 (mixed form), or nullptr
    int nraw;
    int raw_slot[RF_COUNT]; // position of each raw field in a frame, -1 if absent
    int64_t nnodes;         // npoints * nlayers
    int dim;
};

// The node records a step reads, type-erased for the launchers: cur/prev
// are FP64 (plain form) or FP32 (mixed form) records.
struct FieldView {
    const void* cur;
    const void* prev;
    const void* turb;   // {k, eps} per node or nullptr
    int npoints, nlayers, dim, prev_valid;
    template <typename FT>
    DevFields<FT> as() const {
        return DevFields<FT>{(const FT*)cur, (const FT*)prev, npoints, nlayers, dim, prev_valid,
                             (const FT*)turb};
    }
};

// Time interpolation + nodal diffusivity into the packed per-node record
// (eulerian_field_set.pyx:866-938 and 1995-1997); turb != nullptr also
// receives {k, eps} per node.  frozen: copy record 0.  rdim: the record
// layout (the particles' dimension: 3 for 3D particles on 2D fields)
void launch_blend(const DevFrames& fr, int rec, double tf, bool frozen, double fac_keps,
                  void* cur, void* turb, int precision, int rdim, cudaStream_t st);

// depth below the free surface of every active particle of a 3D run with a
// depth array (solver.pyx:526-538)
void launch_depth(int precision, const DevMesh& m, const FieldView& fv, const DevState& s,
                  cudaStream_t st);

// One fused step over every particle of a run (plain FP64 form).
// wq.e == nullptr: walk inline; else queue leavers and run launch_walk after.
void launch_step_plain(const DevMesh& m, const FieldView& fv, const DevParams& p,
                       const DevState& s, const WalkQueue& wq, int aux, int step_index,
                       int* stats, uint32_t* err, cudaStream_t st);

// second half of a 2D LSM1 step: path walk + boundary conditions of queued
// particles (exact FP64 predicates / FP32-filtered predicates)
void launch_walk_plain(const DevMesh& m, const FieldView& fv, const DevParams& p,
                       const DevState& s, const WalkQueue& wq, int aux, int step_index,
                       int* stats, uint32_t* err, cudaStream_t st);
void launch_walk_mixed(const DevMesh& m, const FieldView& fv, const DevParams& p,
                       const DevState& s, const WalkQueue& wq, int aux, int step_index,
                       int* stats, uint32_t* err, cudaStream_t st);

// The LSM2/LSM3 step kernels (cg_lsm23_plain.cu, cg_lsm23_mixed.cu)
void launch_lsm23_plain(const DevMesh& m, const FieldView& fv, const DevParams& p,
                        const DevState& s, int aux, int step_index, int* stats, uint32_t* err,
                        cudaStream_t st);
void launch_lsm23_mixed(const DevMesh& m, const FieldView& fv, const DevParams& p,
                        const DevState& s, int aux, int step_index, int* stats, uint32_t* err,
                        cudaStream_t st);

// The same step, mixed-precision form (FP32 node records).
void launch_step_mixed(const DevMesh& m, const FieldView& fv, const DevParams& p,
                       const DevState& s, const WalkQueue& wq, int aux, int step_index,
                       int* stats, uint32_t* err, cudaStream_t st);

// Solver.initialize_particle_state for particles with tri == -2 (FP64
// arithmetic; node records FP64 or FP32 by precision).  A particle outside
// the mesh is deleted with tag = del_mark (-1 at the run's creation, -2 - it
// when added particles are initialized in iteration it).
void launch_init(int precision, const DevMesh& m, const FieldView& fv, const DevParams& p,
                 const DevState& s, int velocity_init, int del_mark, uint32_t* err,
                 cudaStream_t st);

// Serving pool (cg_serve.cuh): one launch steps every admitted run.
// Device run table entry:
struct ServeRun {
    DevParams p;
    int first;        // first particle of the run's range in the pool
    int count;        // particles
    int horizon;      // steps
    int pad;
    long long start;  // global step at which the run's step 0 executes
};
struct ServeClock {
    unsigned long long gstep;  // steps executed so far
    unsigned int done;         // blocks finished in the current launch
    unsigned int pad;
};
// blocks of one wave of resident serve_step_kernel blocks
int serve_grid_plain();
int serve_grid_mixed();
void launch_serve_plain(int grid, const DevMesh& m, const FieldView& fv, const DevState& pool,
                        const ServeRun* runs, const int2* active, const int* nactive,
                        ServeClock* clk, uint32_t* run_err, cudaStream_t st);
void launch_serve_mixed(int grid, const DevMesh& m, const FieldView& fv, const DevState& pool,
                        const ServeRun* runs, const int2* active, const int* nactive,
                        ServeClock* clk, uint32_t* run_err, cudaStream_t st);

// Working copies of the per-step state in element order (cg_sort.cu):
// always position, tri, tag, PCG32 state and the caller slot; velocity,
// fluid velocity seen, layer and diameter as well when the model reads them
// (nullptr otherwise: reached through slot).  With W_AUXW the outputs no
// step reads (last position, last velocity, last element and, unless W_FVS
// carries it, the fluid velocity seen) have working arrays too; the re-sort
// does not move them (see W_AUXW).
struct WorkState {
    double* pos;              // [n][dim]
    int* tri;                 // [n]
    int* tag;                 // [n]
    unsigned long long* rng;  // [n]
    int* slot;                // [n] caller index of each working particle
    double* vel;              // [n][dim] or nullptr (float rows under W_V32)
    double* vel2;             // [n][dim] the second velocity array (W_VEL2) or nullptr
    double* fvs;              // [n][dim] or nullptr (float rows under W_V32 with W_FVS)
    int* layer;               // [n] or nullptr
    double* diam;             // [n] or nullptr
    double* lpos;             // [n][dim] last position (W_AUXW) or nullptr
    double* lvel;             // [n][dim] last velocity (W_AUXW) or nullptr
    int* ltri;                // [n] last element, LAST_UNSET or -1 (W_AUXW) or nullptr
};
struct SortBuffers {
    int* count;          // [nkeys] histogram, then scan offsets
    int* block_sums;     // [scan_scratch_ints(nkeys)]
    int* perm;           // [n] new order -> old order
    WorkState a, b;      // current and spare working copies
    int dim;             // 2 or 3
    int nl;              // layers per column (1 in 2D): key = tri * nl + layer
    int work;            // W_* flags of the optional arrays
    int vpar;            // W_VEL2: the array holding the newest velocity (0: vel, 1: vel2)
};
int scan_scratch_ints(int nkeys);
// caller arrays -> b.a in element order
void launch_sort_gather(const DevState& user, int nt, SortBuffers& b, cudaStream_t st);
// b.a -> re-sorted by element (through b.b; swaps a and b)
void launch_sort_resort(int n, int nt, SortBuffers& b, cudaStream_t st);
// b.a -> caller arrays
void launch_sort_scatter(const DevState& user, const SortBuffers& b, cudaStream_t st);
// the run's state with the working copies of b.a in place of the caller's
DevState sorted_view(const DevState& user, const SortBuffers& b);

// random_utils.pyx draws on the device (see rng_draws_kernel); out holds n
// values (2n for kind 3)
void launch_rng_draws(uint64_t seed, uint64_t stream, int kind, int method, int64_t n,
                      double* out, uint32_t* err, cudaStream_t st);

// rng[i] = pcg32_seed(seed, tag[i])
void launch_seed(const int* tag, uint64_t* rng, int n, uint64_t seed, cudaStream_t st);
// the same for the particles awaiting initialization (tri == -2)
void launch_seed_added(const int* tri, const int* tag, uint64_t* rng, int n, uint64_t seed,
                       cudaStream_t st);

// values in one packed node record, and its bytes by precision
inline int record_values(int dim) { return dim == 2 ? Slots<2>::NF : Slots<3>::NF; }
inline size_t record_bytes(int dim, int precision) {
    return (size_t)record_values(dim) * (precision ? sizeof(float) : sizeof(double));
}

}  // namespace cg
