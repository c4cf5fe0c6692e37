// cg_api.cu -- the C ABI of libcylag_gpu.so (declared in include/cylag_gpu.h).
//
// Host side of the GB300 particle step: context and stream, one-time mesh
// and field uploads into packed device layouts, per-run time stepping
// (SimuTime and the field time-interpolation record, cylag/core/simutime.pyx
// and cylag/core/eulerian_field_set.pyx:845-938), kernel launches and error
// reporting.  No exception leaves this file.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include <cuda.h>

#include "../../include/cylag_gpu.h"
#include "cg_host.h"

using namespace cg;

struct cg_run {
    cg_ctx* ctx = nullptr;
    cg_params prm{};
    DevParams dp{};
    DevState st{};
    double time = 0.;
    int64_t iteration = 0;
    int64_t nt = 0;
    bool frozen = false;
    int record = 0;
    double fields_time = NAN;   // the time the current field record was blended at
    bool interp_done = false;
    bool prev_valid = false;
    bool fields_ready = false;
    DevBuf cur, prev;
    DevBuf turb;          // {k, eps} per node (LSM2/LSM3 k-epsilon runs)
    DevBuf stats;
    int stats_rows = 0;
    int qpar = 0;   // which of the walk queue's two counters the next step uses
    int stats_cols = 0;
    DevBuf csec;                     // control-section segments {x0, y0, x1, y1}
    std::vector<int32_t> csec_counts;  // [nsteps, ncsec] of the last cg_run_step
    int csec_steps = 0;
    cudaStream_t h2d = nullptr, d2h = nullptr;   // cg_run_step_host copy streams
    // cg_run_step of a run with a walk queue: the next step's field blend on
    // its own stream, during this step (step_started -> blend -> blended)
    cudaStream_t bstream = nullptr;
    cudaEvent_t step_started = nullptr, blended = nullptr;
    std::vector<cudaEvent_t> hev;                // ... and its per-chunk events
    DevBuf strand;                   // stranding output: count (first 256 B) + n records
    bool strand_on = false;
    std::vector<StrandRec> strand_host;  // the last cg_run_step's, in the reference's order
    DevBuf errw;
    DevBuf queue;          // walk queue: count (first 256 B) + one entry per particle
    bool use_queue = false;
    DevBuf sortbuf;        // element-order working copies (cg_sort.cu)
    SortBuffers sb{};
    int sort_period = 0;
    // the working copies hold the newest position, element, tag and PCG32
    // state (and the model's working arrays): the caller's copies of those
    // are stale until cg_run_writeback
    bool resident = false;
    int since_sort = 0;    // steps taken on the working copies since their last sort
    uint64_t bytes = 0;
    uint64_t scratch_bytes = 0;   // walk queue + sort buffers (follow the particle count)
    bool pending_init = false;    // particles added (tri == -2): initialize at the next step
    int32_t init_n = 0;           // ... those with an index below init_n
    std::vector<cudaEvent_t> ev;
    int last_launches = 0;
    double last_ms = 0.;
    double last_step_ms = 0., last_walk_ms = 0.;   // the step kernel alone, the walk alone
};

template <typename T>
static int upload(cg_ctx* c, const std::vector<T>& h, const T*& out) {
    c->mesh_bufs.emplace_back();
    DevBuf& b = c->mesh_bufs.back();
    int rc = dalloc(c, b, h.size() * sizeof(T));
    if (rc) return rc;
    if (!h.empty()) CUDA_TRY(c, cudaMemcpy(b.p, h.data(), b.bytes, cudaMemcpyHostToDevice));
    out = (const T*)b.p;
    c->used += b.bytes;
    return CG_OK;
}


// ---------------------------------------------------------------------------
// Scratch of cg_run_step_noalloc: the walk queue of one step, in a
// file-scope device array instead of memory from cudaMalloc.  Every GPU that
// loads the library holds it (8 MiB + 256 B) until the process exits.
// ---------------------------------------------------------------------------
#define CG_NOALLOC_QUEUE_COUNT_INTS 64
struct NoallocScratch {
    int count[CG_NOALLOC_QUEUE_COUNT_INTS];        // entry counter (256 B)
    WalkEntry entries[CG_NOALLOC_MAX_PARTICLES];   // one entry per particle at most
};
static __device__ __align__(256) NoallocScratch g_noalloc_scratch;

// Device address of g_noalloc_scratch per device ordinal, looked up with that
// device current (in host code the symbol's name is only a stand-in for the
// device array, never an address a kernel may use).  The address belongs to
// the context the module was loaded into: it is cached with that context's
// id and looked up again when the device's current context is a new one
// (after cudaDeviceReset or a reset of the primary context).
static std::mutex g_noalloc_mutex;
static NoallocScratch* g_noalloc_ptr[64] = {nullptr};
static unsigned long long g_noalloc_ctx[64] = {0};

static int noalloc_scratch(cg_ctx* c, NoallocScratch** out) {
    if (c->device < 0 || c->device >= 64)
        return set_err(c, CG_EINVAL, "cg_run_step_noalloc: device ordinal %d out of range",
                       c->device);
    // driver entry points through the runtime (the library does not link
    // libcuda, so that it loads on machines without a driver)
    static CUresult (*get_current)(CUcontext*) = nullptr;
    static CUresult (*get_id)(CUcontext, unsigned long long*) = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        if (!get_current || !get_id) {
            void *f0 = nullptr, *f1 = nullptr;
            cudaDriverEntryPointQueryResult q0, q1;
            if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000, cudaEnableDefault,
                                                 &q0) != cudaSuccess ||
                cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault,
                                                 &q1) != cudaSuccess ||
                q0 != cudaDriverEntryPointSuccess || q1 != cudaDriverEntryPointSuccess)
                return set_err(c, CG_ECUDA, "cg_run_step_noalloc: driver context queries unavailable");
            get_current = (CUresult(*)(CUcontext*))f0;
            get_id = (CUresult(*)(CUcontext, unsigned long long*))f1;
        }
    }
    CUcontext cu = nullptr;
    unsigned long long id = 0;
    if (get_current(&cu) != CUDA_SUCCESS || cu == nullptr || get_id(cu, &id) != CUDA_SUCCESS)
        return set_err(c, CG_ECUDA, "cg_run_step_noalloc: no current CUDA context on device %d",
                       c->device);
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[c->device] || g_noalloc_ctx[c->device] != id) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr)
            return set_err(c, CG_ECUDA, "cudaGetSymbolAddress(g_noalloc_scratch) failed: %s",
                           cudaGetErrorString(e));
        g_noalloc_ptr[c->device] = (NoallocScratch*)ptr;
        g_noalloc_ctx[c->device] = id;
    }
    *out = g_noalloc_ptr[c->device];
    return CG_OK;
}

// ---------------------------------------------------------------------------
// run parameters
// ---------------------------------------------------------------------------
int check_params(cg_ctx* c, const cg_params* p) {
    if (p->precision != CG_PRECISION_FP64 && p->precision != CG_PRECISION_MIXED)
        return set_err(c, CG_EINVAL, "unknown precision %d", p->precision);
    if (p->model < 1 || p->model > 3)
        return set_err(c, CG_EINVAL, "model %d is not built in this library (1, 2, 3)", p->model);
    // solver.pyx:122-132; 3D particles on 2D fields (pseudo-3D) for LSM1
    if (p->dim != c->fdim) {
        if (!(c->fdim == 2 && p->dim == 3))
            return set_err(c, CG_EINVAL,
                           "EulerianFieldSet dimension (%d) does not match LagrangianParticleSet "
                           "set dimension (%d)", c->fdim, p->dim);
        if (!c->has_bottom)
            return set_err(c, CG_EINVAL,
                           "2D EulerianFieldSet with 3D LagrangianParticleSet : EulerianFieldSet "
                           "should contain free surface and bottom fields");
        if (p->model != 1)
            return set_err(c, CG_EINVAL,
                           "pseudo-3D (2D fields, 3D particles) is built for LSM1 only");
    }
    // parameters.pyx:208-279
    if (p->model == 1 && (p->time_scheme < 1 || p->time_scheme > 4))
        return set_err(c, CG_EINVAL, "LSM1 time_scheme must be 1..4");
    if (p->model == 2 && p->diffusion_model == 0 && (p->time_scheme < 1 || p->time_scheme > 5))
        return set_err(c, CG_EINVAL, "LSM2 time_scheme must be 1..5");
    if (p->model >= 2 && p->diffusion_model != 0 && p->time_scheme != 1 && p->time_scheme != 5)
        return set_err(c, CG_EINVAL, "LSM%d with diffusion needs time_scheme 1 or 5", p->model);
    if (p->model == 3 && p->diffusion_model == 0)
        return set_err(c, CG_EINVAL, "LSM3 needs a diffusion model");
    if (p->diffusion_lsm2_option < 1 || p->diffusion_lsm2_option > 3)
        return set_err(c, CG_EINVAL, "diffusion_lsm2_option must be 1..3");
    if (p->lsm3_edge_opt < 1 || p->lsm3_edge_opt > 2)
        return set_err(c, CG_EINVAL, "lsm3_edge_opt must be 1 or 2");
    if (!(p->tl_horizontal > 0.) || !(p->tl_vertical > 0.))
        return set_err(c, CG_EINVAL, "diffusion_lsm3_tl_* must be > 0");
    if (p->diffusion_model < 0 || p->diffusion_model > 3)
        return set_err(c, CG_EINVAL, "diffusion_model must be 0..3");
    if (p->rng_method < 1 || p->rng_method > 3) return set_err(c, CG_EINVAL, "bad rng_method");
    if ((p->diffusion_model == 2 || p->diffusion_model == 3) && !c->has_keps)
        return set_err(c, CG_EINVAL,
                       "diffusion_model=%d requires 'TURBULENT ENERG.' and 'DISSIPATION' fields",
                       p->diffusion_model);
    return CG_OK;
}

void make_dev_params(const cg_ctx* c, const cg_params* p, DevParams& d) {
    d = DevParams{};
    d.model = p->model;
    d.time_scheme = p->time_scheme;
    d.rng_method = p->rng_method;
    d.diffmod = p->diffusion_model;
    d.bc_on = p->boundary_conditions != 0;
    d.bc_type = p->boundary_conditions_type;
    d.max_rebounds = p->max_wall_rebounds;
    d.bnd_statistics = p->bnd_statistics != 0;
    d.nopen = c->nopen;
    d.pdim = p->dim;
    d.dt = p->time_step;
    d.sqrtdt = std::sqrt(p->time_step);
    d.nux = p->horizontal_diffusivity;
    d.nuz = p->vertical_diffusivity;
    // update_state_lsm1.pyx:708-713
    d.diffx_const = std::sqrt(2. * d.nux) * d.sqrtdt;
    d.diffz_const = std::sqrt(2. * d.nuz) * d.sqrtdt;
    d.dt32 = (float)d.dt;
    d.sqrtdt32 = (float)d.sqrtdt;
    d.diffx32 = (float)d.diffx_const;
    d.damp = std::fmin(p->rebound_damping_coef, 1.0 - EPSILON_REBOUND);  // compute_bc.pyx:76
    d.strand = p->stranding_probability;
    d.roughness = p->wall_roughness_angle * DEG_TO_RAD;
    d.buoy_model = p->buoyancy_velocity_model;
    d.buoy_wb = p->buoyancy_velocity;
    d.density = p->particle_density;
    d.rho0 = p->water_density;
    d.drag_coef = p->drag_coefficient;
    d.added_mass = p->added_mass_force != 0;
    d.drag_model = p->drag_coefficient_model;
    d.nuopt = p->diffusion_lsm2_option;
    d.edge_opt = p->lsm3_edge_opt;
    d.tl_h = p->tl_horizontal;
    d.tl_v = p->tl_vertical;
    d.friction_model = c->friction_model;
    d.friction_coef = c->friction_coef;
    // lagrangian_particle_set.pyx:361-375
    {
        double rhop = p->particle_density, rho0 = p->water_density;
        if (!d.added_mass) {
            d.a0c = (rhop - rho0) / rhop;
            d.a1c = 0.5 * (rho0 / rhop);
            d.a2c = 0.;
            d.a3c = 1. / rhop;
        } else {
            double aux = 1. / (rhop + p->added_mass_coef * rho0);
            d.a0c = (rhop - rho0) * aux;
            d.a1c = 0.5 * rho0 * aux;
            d.a2c = rho0 * (1. + p->added_mass_coef) * aux;
            d.a3c = aux;
        }
    }
    d.a0c32 = (float)d.a0c;
    d.a1c32 = (float)d.a1c;
    d.a2c32 = (float)d.a2c;
    d.nux32 = (float)d.nux;
    d.nuz32 = (float)d.nuz;
    d.tl_h32 = (float)d.tl_h;
    d.tl_v32 = (float)d.tl_v;
    d.drag_coef32 = (float)d.drag_coef;
}

// ---------------------------------------------------------------------------
// per-particle scratch of a run: the walk queue (2D LSM1) and the element-
// sorted working copies (their size follows the particle count)
// ---------------------------------------------------------------------------
// caller-owned particle state counted against the budget: five [n, dim]
// FP64 arrays, four int32, the diameter and the PCG32 state
static uint64_t state_bytes_of(int32_t n, int dim) {
    return (uint64_t)n * (5ull * dim * 8 + 4 * 4 + 8 + 8);
}

// the particles that the next step initializes: the first init_n
static DevState added_view(const cg_run* r) {
    DevState v = r->st;
    v.n = r->init_n;
    return v;
}

struct ScratchPlan {
    bool use_queue = false, use_sort = false;
    size_t queue_bytes = 0, sort_bytes = 0;
    size_t off_sums = 0, off_perm = 0, off_w[2] = {0, 0}, off_aux = 0, off_v2 = 0;
    int nkeys = 0, nl_key = 1, work = 0, dim = 2;
    size_t n = 0;
};

static size_t al256(size_t v) { return (v + 255) & ~(size_t)255; }

static ScratchPlan plan_scratch(const cg_ctx* c, const cg_params* p, int32_t n32, bool depth) {
    ScratchPlan q;
    const size_t n = (size_t)(n32 > 0 ? n32 : 0);
    q.n = n;
    q.dim = p->dim;
    // deferred 2D walk: LSM1 2D particles (its queue entry carries no
    // velocities and no elevation)
    q.use_queue = p->dim == 2 && n > 0 && p->model == 1;
    q.queue_bytes = q.use_queue ? 256 + n * sizeof(WalkEntry) : 0;
    // element sort: keys tri * layers + layer (+1 for inactive) within 4096
    // scan tiles of 4096; the optional working arrays are those the model
    // reads every step
    q.nl_key = c->fdim == 3 ? (c->nlayers > 1 ? c->nlayers - 1 : 1) : 1;
    const int64_t nkeys64 = (int64_t)c->mesh.nt * q.nl_key + 1;
    q.use_sort = p->sort_period > 0 && n > 0 && nkeys64 < (1ll << 30) &&
                 scan_scratch_ints((int)nkeys64) <= 4096;
    q.nkeys = (int)std::min<int64_t>(nkeys64, 1ll << 30);
    // velocity: read by the next call's last step (LSM1: the last velocity)
    // or every step (LSM2/LSM3); the outputs no step reads (W_AUXW) in
    // element order too, so that no step writes through the caller's slots
    q.work |= W_VEL | W_AUXW;
    if (p->model >= 2) q.work |= W_DIAM;
    if (p->model == 3) q.work |= W_FVS;
    if (p->dim == 3) q.work |= W_LAYER | W_DIAM;
    // mixed LSM1 2D: working positions as split FP32 pairs (same 16 bytes)
    if (p->precision == CG_PRECISION_MIXED && p->dim == 2 && p->model == 1) q.work |= W_SPLIT;
    // 2D LSM1: two working velocity arrays (the last velocity without
    // copies); its velocity is the fluid velocity seen (in 3D the settling
    // velocity is added to the velocity alone).  Every W_SPLIT run has them
    // (the split step kernels are compiled for it).
    if (p->model == 1 && p->dim == 2) q.work |= W_VEL2;
    // mixed LSM2/LSM3: FP32 working velocities (and fluid velocities seen)
    if (p->precision == CG_PRECISION_MIXED && p->model >= 2) q.work |= W_V32;
    // ... and, for the 3D direct integrators without compute_depth, FP32-pair
    // working positions (step_split3_kernel): LSM3, and LSM2 with its
    // velocity diffusion (the integrator that moves the position itself)
    if (p->precision == CG_PRECISION_MIXED && p->dim == 3 && p->time_scheme == 5 && !depth &&
        (p->model == 3 ||
         (p->model == 2 && p->diffusion_model != 0 && p->diffusion_lsm2_option >= 2)))
        q.work |= W_SPLIT3;
    const size_t D = (size_t)p->dim;
    const size_t vb = (q.work & W_V32) ? 4 : 8;
    const size_t work_bytes = al256(n * 8 * D) + 4 * al256(n * 8) +
                              ((q.work & W_VEL) ? al256(n * vb * D) : 0) +
                              ((q.work & W_FVS) ? al256(n * vb * D) : 0) +
                              ((q.work & W_LAYER) ? al256(n * 4) : 0) +
                              ((q.work & W_DIAM) ? al256(n * 8) : 0) +
                              ((q.work & W_AUXW) ? al256(n * 4) : 0);
    // the outputs the re-sort does not move: one set shared by both copies
    // (no fluid-velocity-seen array for W_VEL2 runs: it is the velocity)
    const size_t aux_bytes = (q.work & W_AUXW)
        ? 2 * al256(n * 8 * D) + ((q.work & (W_FVS | W_VEL2)) ? 0 : al256(n * 8 * D)) : 0;
    if (q.use_sort) {
        q.off_sums = al256((size_t)q.nkeys * 4);
        q.off_perm = al256(q.off_sums + (size_t)scan_scratch_ints(q.nkeys) * 4);
        q.off_w[0] = al256(q.off_perm + n * 4);
        q.off_w[1] = q.off_w[0] + work_bytes;
        q.off_aux = q.off_w[1] + work_bytes;
        // W_VEL2: the two copies' second velocity arrays after the rest (the
        // copies' other arrays keep the offsets they have without them)
        q.off_v2 = q.off_aux + aux_bytes;
        q.sort_bytes = q.off_v2 + ((q.work & W_VEL2) ? 2 * al256(n * 8 * D) : 0);
    }
    return q;
}

// allocates the planned scratch into r (r->queue and r->sortbuf must be empty)
static int take_scratch(cg_ctx* c, cg_run* r, const ScratchPlan& q) {
    int rc;
    r->use_queue = false;
    r->sb = SortBuffers{};
    r->sort_period = 0;
    r->resident = false;
    r->since_sort = 0;
    if ((rc = dalloc(c, r->queue, q.queue_bytes)) || (rc = dalloc(c, r->sortbuf, q.sort_bytes)))
        return rc;
    r->use_queue = q.use_queue;
    if (!q.use_sort) return CG_OK;
    const size_t n = q.n, D = (size_t)q.dim;
    char* b = (char*)r->sortbuf.p;
    r->sb.count = (int*)b;
    r->sb.block_sums = (int*)(b + q.off_sums);
    r->sb.perm = (int*)(b + q.off_perm);
    r->sb.dim = q.dim;
    r->sb.nl = q.nl_key;
    r->sb.work = q.work;
    r->sb.vpar = 0;
    WorkState* ws[2] = {&r->sb.a, &r->sb.b};
    char* aux = b + q.off_aux;
    auto take_aux = [&](size_t bytes) { char* t = aux; aux += al256(bytes); return t; };
    double* lpos = (q.work & W_AUXW) ? (double*)take_aux(n * 8 * D) : nullptr;
    double* lvel = (q.work & W_AUXW) ? (double*)take_aux(n * 8 * D) : nullptr;
    double* fvs_out = ((q.work & W_AUXW) && !(q.work & (W_FVS | W_VEL2)))
                          ? (double*)take_aux(n * 8 * D) : nullptr;
    for (int k = 0; k < 2; ++k) {
        char* w = b + q.off_w[k];
        auto take = [&](size_t bytes) { char* t = w; w += al256(bytes); return t; };
        ws[k]->pos = (double*)take(n * 8 * D);
        ws[k]->rng = (unsigned long long*)take(n * 8);
        ws[k]->tri = (int*)take(n * 8);
        ws[k]->tag = (int*)take(n * 8);
        ws[k]->slot = (int*)take(n * 8);
        const size_t vb = (q.work & W_V32) ? 4 : 8;
        ws[k]->vel = (q.work & W_VEL) ? (double*)take(n * vb * D) : nullptr;
        ws[k]->vel2 = (q.work & W_VEL2) ? (double*)(b + q.off_v2 + k * al256(n * 8 * D))
                                        : nullptr;
        ws[k]->fvs = (q.work & W_FVS) ? (double*)take(n * vb * D) : fvs_out;
        ws[k]->layer = (q.work & W_LAYER) ? (int*)take(n * 4) : nullptr;
        ws[k]->diam = (q.work & W_DIAM) ? (double*)take(n * 8) : nullptr;
        ws[k]->ltri = (q.work & W_AUXW) ? (int*)take(n * 4) : nullptr;
        ws[k]->lpos = lpos;
        ws[k]->lvel = lvel;
    }
    r->sort_period = r->prm.sort_period;
    return CG_OK;
}

// The bounds-checked build's error word (ERR_BOUNDS), read and cleared; 0 in
// normal builds, which never set it (call after synchronizing the stream).
static uint32_t take_bounds_error(cg_ctx* c) {
#ifdef CG_DEBUG_BOUNDS
    uint32_t b = 0;
    if (c->mesh.dbg && cudaMemcpy(&b, c->mesh.dbg, sizeof b, cudaMemcpyDeviceToHost) == cudaSuccess &&
        b)
        cudaMemset(c->mesh.dbg, 0, sizeof b);
    return b;
#else
    (void)c;
    return 0;
#endif
}

// The walk queue of the next step (or chunk): a run's steps alternate
// between two counters, so that no step needs a separate reset.  The one a
// step uses is zero when it starts (the call zeroed it, or the previous step
// kernel did); the step kernel zeroes the other, whose walk has finished.
static WalkQueue next_queue(cg_run* r, int* counters, WalkEntry* entries) {
    WalkQueue wq{nullptr, nullptr, nullptr};
    if (!r->use_queue) return wq;
    wq.count = counters + r->qpar;
    wq.e = entries;
    wq.reset = counters + (1 - r->qpar);
    r->qpar ^= 1;
    return wq;
}

// a call's first step: its counter zeroed, whatever ran on the array before
static int start_queue(cg_run* r, int* counters) {
    if (!r->use_queue) return CG_OK;
    CUDA_TRY(r->ctx, cudaMemsetAsync(counters + r->qpar, 0, sizeof(int), r->ctx->stream));
    return CG_OK;
}

// The per-step statistics rows of a call: grown to at least 1024 rows and by
// doubling, so that a call longer than the last one does not reallocate
// (cudaFree and cudaMalloc synchronize the device) inside a timed loop.
static int ensure_stats(cg_run* r, int nsteps, int row) {
    if (r->stats_rows >= nsteps && r->stats_cols == row) return CG_OK;
    const int rows = std::max(nsteps, std::max(2 * r->stats_rows, 1024));
    dfree(r->stats);
    int rc = dalloc(r->ctx, r->stats, (size_t)rows * row * sizeof(int));
    if (rc) return rc;
    r->stats_rows = rows;
    r->stats_cols = row;
    return CG_OK;
}

// Working copies -> the caller's arrays (stream-ordered), after which the
// caller's arrays are the run's state again and the next step gathers them.
static int write_back(cg_run* r) {
    if (!r->resident) return CG_OK;
    NvtxRange nvtx("write back");
    cg_ctx* c = r->ctx;
    launch_sort_scatter(r->st, r->sb, c->stream);
    r->resident = false;
    CUDA_TRY(c, cudaGetLastError());
    return CG_OK;
}

extern "C" {

int cg_ctx_create(int32_t device, uint64_t hbm_budget_bytes, cg_ctx** out) {
    if (!out) return CG_EINVAL;
    *out = nullptr;
    cg_ctx* c = new (std::nothrow) cg_ctx();
    if (!c) return CG_EINVAL;
    c->device = device;
    c->budget = hbm_budget_bytes;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        return CG_ECUDA;
    }
    c->stream = c->own_stream;
    *out = c;
    return CG_OK;
}

int cg_ctx_destroy(cg_ctx* c) {
    if (!c) return CG_EINVAL;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    for (auto& b : c->mesh_bufs) dfree(b);
    dfree(c->frames_buf);
    dfree(c->frames32_buf);
    cudaStreamSynchronize(c->own_stream);
    cudaStreamDestroy(c->own_stream);
    delete c;
    return CG_OK;
}

int cg_last_error(const cg_ctx* c, char* buf, uint64_t len) {
    if (!c || !buf || len == 0) return CG_EINVAL;
    snprintf(buf, (size_t)len, "%s", c->err.c_str());
    return CG_OK;
}

uint64_t cg_ctx_stream(const cg_ctx* c) { return c ? (uint64_t)(uintptr_t)c->stream : 0; }

int cg_ctx_set_stream(cg_ctx* c, uint64_t stream) {
    if (!c) return CG_EINVAL;
    CUDA_TRY(c, cudaSetDevice(c->device));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    c->stream = stream ? (cudaStream_t)(uintptr_t)stream : c->own_stream;
    return CG_OK;
}

int cg_ctx_sync(cg_ctx* c) {
    if (!c) return CG_EINVAL;
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return CG_OK;
}

// ---------------------------------------------------------------------------
// mesh (cylag/geom/triangular_mesh.pyx:75-179)
// ---------------------------------------------------------------------------
int cg_mesh_upload(cg_ctx* c, const cg_mesh_desc* d) {
    if (!c || !d) return CG_EINVAL;
    if (d->nv <= 0 || d->nt <= 0 || d->ne <= 0 || !d->x || !d->y || !d->triangles || !d->gradx ||
        !d->grady || !d->det || !d->edges || !d->triedge_map || !d->edgetri_map ||
        !d->edges_labels || !d->grid_start || !d->grid_tris || d->grid_nx <= 0 || d->grid_ny <= 0)
        return set_err(c, CG_EINVAL, "cg_mesh_upload: incomplete mesh description");
    CUDA_TRY(c, cudaSetDevice(c->device));
    for (auto& b : c->mesh_bufs) dfree(b);
    c->mesh_bufs.clear();
    int nv = d->nv, nt = d->nt, ne = d->ne;
    // range checks: every index the kernels follow must stay in bounds
    for (int64_t k = 0; k < 3LL * nt; ++k) {
        if (d->triangles[k] < 0 || d->triangles[k] >= nv)
            return set_err(c, CG_EINVAL, "triangle vertex out of range at %lld", (long long)k);
        if (d->triedge_map[k] < 0 || d->triedge_map[k] >= ne)
            return set_err(c, CG_EINVAL, "triedge_map out of range at %lld", (long long)k);
    }
    for (int64_t j = 0; j < ne; ++j) {
        int a = d->edges[2 * j], b = d->edges[2 * j + 1];
        int t0 = d->edgetri_map[2 * j], t1 = d->edgetri_map[2 * j + 1];
        if (a < 0 || a >= nv || b < 0 || b >= nv || t0 < 0 || t0 >= nt || t1 < -1 || t1 >= nt)
            return set_err(c, CG_EINVAL, "edge %lld out of range", (long long)j);
    }
    int64_t ncell = (int64_t)d->grid_nx * d->grid_ny;
    int64_t ngt = d->grid_start[ncell];
    for (int64_t q = 0; q < ncell; ++q)
        if (d->grid_start[q] < 0 || d->grid_start[q] > d->grid_start[q + 1])
            return set_err(c, CG_EINVAL, "grid_start not monotonic");
    for (int64_t q = 0; q < ngt; ++q)
        if (d->grid_tris[q] < 0 || d->grid_tris[q] >= nt)
            return set_err(c, CG_EINVAL, "grid triangle out of range");
    for (int64_t v = 0; v < nv; ++v)
        if (!std::isfinite(d->x[v]) || !std::isfinite(d->y[v]))
            return set_err(c, CG_EINVAL, "non-finite vertex coordinate at %lld", (long long)v);

    std::vector<double2> xy(nv);
    for (int v = 0; v < nv; ++v) xy[v] = make_double2(d->x[v], d->y[v]);
    std::vector<int4> tv(2 * (size_t)nt);
    std::vector<double2> basis(5 * (size_t)nt);
    for (int k = 0; k < nt; ++k) {
        const int32_t* t = d->triangles + 3 * k;
        const int32_t* e = d->triedge_map + 3 * k;
        tv[2 * k] = make_int4(t[0], t[1], t[2], e[0]);
        tv[2 * k + 1] = make_int4(e[1], e[2], 0, 0);
        const double *de = d->det + 3 * k, *gx = d->gradx + 3 * k, *gy = d->grady + 3 * k;
        basis[5 * k + 0] = make_double2(de[0], de[1]);
        basis[5 * k + 1] = make_double2(de[2], gx[0]);
        basis[5 * k + 2] = make_double2(gx[1], gx[2]);
        basis[5 * k + 3] = make_double2(gy[0], gy[1]);
        basis[5 * k + 4] = make_double2(gy[2], 0.0);
    }
    // exact-test geometry: vertices and edge vectors, FP64 subtractions as in
    // utils.pyx:332-361; FP32 P1 gradients for the mixed form
    std::vector<double2> geo(6 * (size_t)nt);
    std::vector<float4> g32(2 * (size_t)nt);
    for (int k = 0; k < nt; ++k) {
        const int32_t* t = d->triangles + 3 * k;
        double xa = d->x[t[0]], ya = d->y[t[0]], xb = d->x[t[1]], yb = d->y[t[1]];
        double xc = d->x[t[2]], yc = d->y[t[2]];
        geo[6 * k + 0] = make_double2(xa, ya);
        geo[6 * k + 1] = make_double2(xb, yb);
        geo[6 * k + 2] = make_double2(xc, yc);
        geo[6 * k + 3] = make_double2(xb - xa, yb - ya);
        geo[6 * k + 4] = make_double2(xc - xb, yc - yb);
        geo[6 * k + 5] = make_double2(xa - xc, ya - yc);
        const double *gx = d->gradx + 3 * k, *gy = d->grady + 3 * k;
        g32[2 * k] = make_float4((float)gx[0], (float)gx[1], (float)gx[2], (float)gy[0]);
        g32[2 * k + 1] = make_float4((float)gy[1], (float)gy[2], 0.f, 0.f);
    }
    // neighbour across the edge opposite each vertex
    std::vector<int4> nbr((size_t)nt);
    for (int k = 0; k < nt; ++k) {
        const int32_t* t = d->triangles + 3 * k;
        int n[3] = {-1, -1, -1};
        for (int i = 0; i < 3; ++i) {
            int eid = d->triedge_map[3 * k + i];
            int a = d->edges[2 * eid], b = d->edges[2 * eid + 1];
            int t0 = d->edgetri_map[2 * eid], t1 = d->edgetri_map[2 * eid + 1];
            for (int j = 0; j < 3; ++j)
                if (t[j] != a && t[j] != b) n[j] = (t0 == k) ? t1 : t0;
        }
        nbr[k] = make_int4(n[0], n[1], n[2], 0);
    }
    // packed 64-byte mixed-form record (see DevMesh::t64)
    std::vector<int4> t64(4 * (size_t)nt);
    for (int k = 0; k < nt; ++k) {
        const int32_t* t = d->triangles + 3 * k;
        const int32_t* e = d->triedge_map + 3 * k;
        double xa = d->x[t[0]], ya = d->y[t[0]];
        long long bx, by;
        memcpy(&bx, &xa, 8);
        memcpy(&by, &ya, 8);
        t64[4 * k + 0] = make_int4(t[0], t[1], t[2], e[0]);
        t64[4 * k + 1] = make_int4((int)(bx & 0xffffffffLL), (int)(bx >> 32),
                                   (int)(by & 0xffffffffLL), (int)(by >> 32));
        float4 g0 = g32[2 * k], g1 = g32[2 * k + 1];
        int4 gi0, gi1;
        memcpy(&gi0, &g0, 16);
        memcpy(&gi1, &g1, 8);
        gi1.z = e[1];
        gi1.w = e[2];
        t64[4 * k + 2] = gi0;
        t64[4 * k + 3] = gi1;
    }
    // the same records with vertex a as FP32 pairs hi + lo, and the
    // neighbour across each edge in place of the edge ids (the split step's
    // hops read them from the record they already hold)
    std::vector<int4> t64s(t64);
    for (int k = 0; k < nt; ++k) {
        const int32_t* t = d->triangles + 3 * k;
        double xa = d->x[t[0]], ya = d->y[t[0]];
        float q[4];
        q[0] = (float)xa;
        q[1] = (float)ya;
        q[2] = (float)(xa - (double)q[0]);
        q[3] = (float)(ya - (double)q[1]);
        memcpy(&t64s[4 * k + 1], q, 16);
        t64s[4 * k].w = nbr[k].x;
        t64s[4 * k + 3].z = nbr[k].y;
        t64s[4 * k + 3].w = nbr[k].z;
    }
    // walk records (DevMesh::wrec, WalkRec): vertices, FP32 gradients, edge
    // ids, the two elements of each edge and its end points' local indices
    std::vector<int4> wrec(8 * (size_t)nt, make_int4(0, 0, 0, 0));
    for (int k = 0; k < nt; ++k) {
        const int32_t* t = d->triangles + 3 * k;
        const int32_t* e = d->triedge_map + 3 * k;
        int4* w = &wrec[8 * (size_t)k];
        for (int v = 0; v < 3; ++v) {
            const double xv = d->x[t[v]], yv = d->y[t[v]];
            long long bx, by;
            memcpy(&bx, &xv, 8);
            memcpy(&by, &yv, 8);
            w[v] = make_int4((int)(bx & 0xffffffffLL), (int)(bx >> 32), (int)(by & 0xffffffffLL),
                             (int)(by >> 32));
        }
        memcpy(&w[3], &g32[2 * k], 16);
        const float4 g1 = g32[2 * k + 1];
        memcpy(&w[4].x, &g1.x, 4);
        memcpy(&w[4].y, &g1.y, 4);
        int ez[3], ew[3], order = 0;
        for (int i = 0; i < 3; ++i) {
            const int j = e[i];
            ez[i] = d->edgetri_map[2 * j];
            ew[i] = d->edgetri_map[2 * j + 1];
            int la = 0, lb = 0;
            for (int v = 0; v < 3; ++v) {
                if (t[v] == d->edges[2 * j]) la = v;
                if (t[v] == d->edges[2 * j + 1]) lb = v;
            }
            order |= (la << (4 * i)) | (lb << (4 * i + 2));
        }
        w[4].z = e[0];
        w[4].w = e[1];
        w[5] = make_int4(e[2], ez[0], ew[0], ez[1]);
        w[6] = make_int4(ew[1], ez[2], ew[2], order);
    }
    std::vector<int4> edge(ne);
    std::vector<int> lab(ne);
    for (int j = 0; j < ne; ++j) {
        edge[j] = make_int4(d->edges[2 * j], d->edges[2 * j + 1], d->edgetri_map[2 * j],
                            d->edgetri_map[2 * j + 1]);
        lab[j] = d->edges_labels[j];
    }
    // error word of the bounds-checked build (ERR_BOUNDS)
    c->mesh_bufs.emplace_back();
    {
        int rc0 = dalloc(c, c->mesh_bufs.back(), 256);
        if (rc0) return rc0;
        CUDA_TRY(c, cudaMemset(c->mesh_bufs.back().p, 0, 256));
    }
    uint32_t* dbg_word = (uint32_t*)c->mesh_bufs.back().p;
    std::vector<int> gstart(d->grid_start, d->grid_start + ncell + 1);
    std::vector<int> gtris(d->grid_tris, d->grid_tris + ngt);
    DevMesh m{};
    m.nv = nv; m.nt = nt; m.ne = ne;
    int rc;
    const double2 *p_xy, *p_basis, *p_geo;
    const float4* p_g32;
    const int4 *p_tv, *p_edge, *p_t64, *p_t64s, *p_nbr, *p_wrec;
    const int *p_lab, *p_gs, *p_gt;
    if ((rc = upload(c, xy, p_xy))) return rc;
    if ((rc = upload(c, tv, p_tv))) return rc;
    if ((rc = upload(c, basis, p_basis))) return rc;
    if ((rc = upload(c, geo, p_geo))) return rc;
    if ((rc = upload(c, g32, p_g32))) return rc;
    if ((rc = upload(c, t64, p_t64))) return rc;
    if ((rc = upload(c, t64s, p_t64s))) return rc;
    if ((rc = upload(c, edge, p_edge))) return rc;
    if ((rc = upload(c, nbr, p_nbr))) return rc;
    if ((rc = upload(c, wrec, p_wrec))) return rc;
    if ((rc = upload(c, lab, p_lab))) return rc;
    if ((rc = upload(c, gstart, p_gs))) return rc;
    if ((rc = upload(c, gtris, p_gt))) return rc;
    m.xy = p_xy; m.tv = p_tv; m.basis = p_basis; m.edge = p_edge; m.elabel = p_lab;
    m.geo = p_geo; m.g32 = p_g32; m.t64 = p_t64; m.t64s = p_t64s; m.nbr = p_nbr;
    m.gstart = p_gs; m.gtris = p_gt; m.wrec = p_wrec;
    m.dbg = dbg_word;
    m.gx0 = d->grid_x0;
    m.gy0 = d->grid_y0;
    m.ginv = d->grid_inv_cell;
    m.gnx = d->grid_nx;
    m.gny = d->grid_ny;
    c->mesh = m;
    c->nopen = d->nopen;
    c->have_mesh = true;
    return CG_OK;
}

// ---------------------------------------------------------------------------
// fields (cylag/core/eulerian_field_set.pyx:125-256)
// ---------------------------------------------------------------------------
int cg_fields_upload(cg_ctx* c, const cg_fields_desc* d) {
    if (!c || !d) return CG_EINVAL;
    if (!c->have_mesh) return set_err(c, CG_ESTATE, "cg_fields_upload before cg_mesh_upload");
    if (d->dim != 2 && d->dim != 3)
        return set_err(c, CG_EINVAL, "field dim must be 2 or 3");
    if (d->npoints != c->mesh.nv)
        return set_err(c, CG_EINVAL, "npoints (%d) != mesh nv (%d)", d->npoints, c->mesh.nv);
    if (d->nlayers < 1 || d->ntimes < 1 || !d->times || !d->elevation || !d->velocity_x ||
        !d->velocity_y || (d->dim == 3 && !d->velocity_z))
        return set_err(c, CG_EINVAL, "incomplete field description");
    if (d->dim == 2 && d->nlayers != 1) return set_err(c, CG_EINVAL, "2D fields need nlayers == 1");
    for (int t = 0; t + 1 < d->ntimes; ++t)
        if (!(d->times[t + 1] - d->times[t] > EPSILON))
            return set_err(c, CG_EINVAL, "times must be strictly increasing (at %d)", t);
    CUDA_TRY(c, cudaSetDevice(c->device));
    const double* src[RF_COUNT] = {d->elevation, d->velocity_x, d->velocity_y,
                                   d->dim == 3 ? d->velocity_z : nullptr,
                                   d->turbulent_energy, d->dissipation, d->bottom};
    DevFrames fr{};
    fr.nraw = 0;
    for (int f = 0; f < RF_COUNT; ++f) fr.raw_slot[f] = src[f] ? fr.nraw++ : -1;
    fr.nnodes = (int64_t)d->npoints * d->nlayers;
    fr.dim = d->dim;
    int64_t per = fr.nnodes;
    std::vector<double> h((size_t)d->ntimes * fr.nraw * per);
    for (int t = 0; t < d->ntimes; ++t)
        for (int f = 0; f < RF_COUNT; ++f) {
            if (!src[f]) continue;
            memcpy(&h[((size_t)t * fr.nraw + fr.raw_slot[f]) * per], src[f] + (size_t)t * per,
                   per * sizeof(double));
        }
    // a re-upload replaces the frames (and their budget share)
    if (c->frames32_buf.p) c->used -= c->frames32_buf.bytes;
    if (c->frames_buf.p) c->used -= c->frames_buf.bytes;
    dfree(c->frames32_buf);
    dfree(c->frames_buf);
    int rc = dalloc(c, c->frames_buf, h.size() * sizeof(double));
    if (rc) return rc;
    CUDA_TRY(c, cudaMemcpy(c->frames_buf.p, h.data(), c->frames_buf.bytes, cudaMemcpyHostToDevice));
    c->used += c->frames_buf.bytes;
    fr.frames = (const double*)c->frames_buf.p;
    // FP32 copy for the mixed form's per-step blend
    {
        std::vector<float> h32(h.size());
        for (size_t k = 0; k < h.size(); ++k) h32[k] = (float)h[k];
        dfree(c->frames32_buf);
        if ((rc = dalloc(c, c->frames32_buf, h32.size() * sizeof(float)))) return rc;
        CUDA_TRY(c, cudaMemcpy(c->frames32_buf.p, h32.data(), c->frames32_buf.bytes,
                               cudaMemcpyHostToDevice));
        c->used += c->frames32_buf.bytes;
        fr.frames32 = (const float*)c->frames32_buf.p;
    }
    c->frames = fr;
    c->times.assign(d->times, d->times + d->ntimes);
    c->fdim = d->dim;
    c->nlayers = d->nlayers;
    c->npoints = d->npoints;
    c->has_keps = d->turbulent_energy && d->dissipation;
    c->has_bottom = d->bottom != nullptr;
    if (d->friction_model < 0 || d->friction_model > 3)
        return set_err(c, CG_EINVAL, "Invalid friction model %d", d->friction_model);
    c->friction_model = d->friction_model;
    c->friction_coef = d->friction_coefficient;
    c->have_fields = true;
    return CG_OK;
}

// ---------------------------------------------------------------------------
// runs (cylag/core/solver.pyx:74-236)
// ---------------------------------------------------------------------------
// zlocalizer.pyx:125-151
static int lower_index(const std::vector<double>& t, double value, int last) {
    int ni = (int)t.size();
    for (int i = last; i < ni - 1; ++i)
        if (value >= t[i] && value < t[i + 1]) return i;
    if (ni > 1 && value >= t[ni - 1]) return ni - 2;
    return 0;
}

int cg_run_create(cg_ctx* c, const cg_params* p, const cg_state_desc* s, cg_run** out) {
    if (!c || !p || !s || !out) return CG_EINVAL;
    *out = nullptr;
    if (!c->have_mesh || !c->have_fields)
        return set_err(c, CG_ESTATE, "cg_run_create before mesh/field upload");
    int rc0 = check_params(c, p);
    if (rc0) return rc0;
    if (!(p->time_step > 0.) || !(p->final_time > p->initial_time))
        return set_err(c, CG_EINVAL, "bad time interval");
    if (s->n < 0 || (s->n > 0 && (!s->position || !s->velocity || !s->fluid_velocity_seen ||
                                  !s->last_position || !s->last_velocity || !s->tri ||
                                  !s->last_tri || !s->lowerlayer || !s->tag || !s->diameter ||
                                  !s->rng_state)))
        return set_err(c, CG_EINVAL, "incomplete particle state description");
    bool frozen = p->frozen_eulerian_fields || c->times.size() == 1;
    if (c->times.size() == 1 && !p->frozen_eulerian_fields)
        return set_err(c, CG_EINVAL,
                       "EulerianFieldSet has only one time step, use frozen_eulerian_fields=True");
    if (!p->frozen_eulerian_fields && p->final_time > c->times.back())
        return set_err(c, CG_EINVAL, "final_time > EulerianFieldSet maximum time");
    CUDA_TRY(c, cudaSetDevice(c->device));

    // the record layout follows the particles' dimension (3D particles on 2D
    // fields read the 3D layout with one layer, the bed in its ZB slot)
    size_t rec_bytes = record_bytes(p->dim, p->precision) * c->frames.nnodes;
    // LSM2/LSM3 with k-epsilon diffusion read k and eps themselves
    bool need_turb = p->model >= 2 && (p->diffusion_model == 2 || p->diffusion_model == 3);
    size_t turb_bytes = need_turb ? 2 * c->frames.nnodes * (p->precision ? 4 : 8) : 0;
    uint64_t state_bytes = state_bytes_of(s->n, p->dim);
    const ScratchPlan plan = plan_scratch(c, p, s->n, s->depth != nullptr);
    uint64_t need = state_bytes + 2 * rec_bytes + turb_bytes + 64 + plan.queue_bytes + plan.sort_bytes;
    if (c->budget && c->used + need > c->budget)
        return set_err(c, CG_ENOMEM_BUDGET, "run needs %llu bytes, %llu of %llu in use",
                       (unsigned long long)need, (unsigned long long)c->used,
                       (unsigned long long)c->budget);

    cg_run* r = new (std::nothrow) cg_run();
    if (!r) return set_err(c, CG_EINVAL, "out of host memory");
    r->ctx = c;
    r->prm = *p;
    int rc;
    if ((rc = dalloc(c, r->cur, rec_bytes)) || (rc = dalloc(c, r->prev, rec_bytes)) ||
        (rc = dalloc(c, r->errw, 64)) || (rc = dalloc(c, r->turb, turb_bytes)) ||
        (rc = take_scratch(c, r, plan))) {
        dfree(r->cur); dfree(r->prev); dfree(r->errw); dfree(r->queue); dfree(r->sortbuf);
        dfree(r->turb);
        delete r;
        return rc;
    }
    cudaMemsetAsync(r->errw.p, 0, 64, c->stream);
    r->bytes = need;
    r->scratch_bytes = plan.queue_bytes + plan.sort_bytes;
    c->used += need;

    make_dev_params(c, p, r->dp);

    DevState& st = r->st;
    st.n = s->n;
    st.pos = s->position;
    st.vel = s->velocity;
    st.fvs = s->fluid_velocity_seen;
    st.last_pos = s->last_position;
    st.last_vel = s->last_velocity;
    st.tri = s->tri;
    st.last_tri = s->last_tri;
    st.lowerlayer = s->lowerlayer;
    st.tag = s->tag;
    st.diameter = s->diameter;
    st.rng = s->rng_state;
    st.depth = (s->depth && r->prm.dim == 3) ? s->depth : nullptr;

    // simutime.pyx:46-75
    r->time = p->initial_time;
    r->nt = (int64_t)((p->final_time - p->initial_time) / p->time_step);
    r->frozen = frozen;
    // solver.pyx:144-152 and 188-191
    r->record = frozen ? 0 : lower_index(c->times, p->initial_time, 0);
    r->interp_done = false;
    r->prev_valid = false;
    *out = r;
    return CG_OK;
}

int cg_run_destroy(cg_run* r) {
    if (!r) return CG_EINVAL;
    cg_ctx* c = r->ctx;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    dfree(r->cur);
    dfree(r->prev);
    dfree(r->turb);
    dfree(r->stats);
    dfree(r->csec);
    dfree(r->strand);
    dfree(r->errw);
    dfree(r->queue);
    dfree(r->sortbuf);
    for (auto e : r->ev) cudaEventDestroy(e);
    for (auto e : r->hev) cudaEventDestroy(e);
    if (r->h2d) cudaStreamDestroy(r->h2d);
    if (r->d2h) cudaStreamDestroy(r->d2h);
    if (r->bstream) cudaStreamDestroy(r->bstream);
    if (r->step_started) cudaEventDestroy(r->step_started);
    if (r->blended) cudaEventDestroy(r->blended);
    c->used -= r->bytes;
    delete r;
    return CG_OK;
}

int cg_run_seed(cg_run* r) {
    if (!r) return CG_EINVAL;
    cg_ctx* c = r->ctx;
    CUDA_TRY(c, cudaSetDevice(c->device));
    int rc = write_back(r);
    if (rc) return rc;
    launch_seed(r->st.tag, r->st.rng, r->st.n, r->prm.seed, c->stream);
    CUDA_TRY(c, cudaGetLastError());
    return CG_OK;
}

static double keps_fac(const cg_run* r) { return CMU / r->prm.schmidt_number; }

static FieldView field_view(const cg_run* r) {
    const cg_ctx* c = r->ctx;
    return FieldView{r->cur.p, r->prev.p, r->turb.p, c->npoints, c->nlayers, c->fdim,
                     r->prev_valid ? 1 : 0};
}

// eulerian_field_set.pyx:866-938: saves the previous temps (pointer swap)
// and interpolates at `time` into the current ones.
static int time_interpolation(cg_run* r, double time, cudaStream_t st = nullptr) {
    cg_ctx* c = r->ctx;
    if (!st) st = c->stream;
    if (r->frozen) {
        if (!r->fields_ready) {
            launch_blend(c->frames, 0, 1.0, true, keps_fac(r), r->cur.p, r->turb.p, r->prm.precision,
                     r->prm.dim, c->stream);
            CUDA_TRY(c, cudaMemcpyAsync(r->prev.p, r->cur.p, r->cur.bytes,
                                        cudaMemcpyDeviceToDevice, c->stream));
            r->fields_ready = true;
        }
        return CG_OK;
    }
    std::swap(r->cur, r->prev);
    r->prev_valid = r->interp_done;
    r->interp_done = true;
    r->record = lower_index(c->times, time, r->record);
    int rec = r->record;
    double dt = c->times[rec] - c->times[rec + 1];
    if (std::fabs(dt) < EPSILON)
        return set_err(c, CG_EINVAL, "Time interpolation failed: duplicate times at record %d", rec);
    double tf = (time - c->times[rec + 1]) / dt;
    launch_blend(c->frames, rec, tf, false, keps_fac(r), r->cur.p, r->turb.p, r->prm.precision,
                 r->prm.dim, st);
    r->fields_time = time;
    r->fields_ready = true;
    CUDA_TRY(c, cudaGetLastError());
    return CG_OK;
}

static int ensure_fields(cg_run* r) {
    if (r->fields_ready) return CG_OK;
    cg_ctx* c = r->ctx;
    if (r->frozen) return time_interpolation(r, r->time);
    // EulerianFieldSet._init_tmp (743-776): both temps hold record 0, then
    // Solver.__init__ interpolates at initial_time (solver.pyx:190-191).
    launch_blend(c->frames, 0, 1.0, true, keps_fac(r), r->cur.p, r->turb.p, r->prm.precision,
                     r->prm.dim, c->stream);
    CUDA_TRY(c, cudaMemcpyAsync(r->prev.p, r->cur.p, r->cur.bytes, cudaMemcpyDeviceToDevice,
                                c->stream));
    return time_interpolation(r, r->prm.initial_time);
}

int cg_run_init(cg_run* r) {
    if (!r) return CG_EINVAL;
    cg_ctx* c = r->ctx;
    CUDA_TRY(c, cudaSetDevice(c->device));
    int rc = write_back(r);
    if (rc) return rc;
    if ((rc = ensure_fields(r))) return rc;
    launch_init(r->prm.precision, c->mesh, field_view(r), r->dp, r->st,
                r->prm.particle_velocity_init, -1, (uint32_t*)r->errw.p, c->stream);
    CUDA_TRY(c, cudaGetLastError());
    return CG_OK;
}

// the stranding records of the call just finished, in the reference's order
static int collect_stranded(cg_run* r) {
    if (!r->strand_on) return CG_OK;
    cg_ctx* c = r->ctx;
    int cnt = 0;
    CUDA_TRY(c, cudaMemcpy(&cnt, r->strand.p, sizeof(int), cudaMemcpyDeviceToHost));
    cnt = std::min(cnt, r->dp.strand_cap);
    r->strand_host.resize(cnt);
    if (cnt)
        CUDA_TRY(c, cudaMemcpy(r->strand_host.data(), r->dp.strand_rec,
                               (size_t)cnt * sizeof(StrandRec), cudaMemcpyDeviceToHost));
    // the reference appends in its particle loop: by step, then index
    std::sort(r->strand_host.begin(), r->strand_host.end(),
              [](const StrandRec& a, const StrandRec& b) {
                  return a.step != b.step ? a.step < b.step : a.index < b.index;
              });
    return CG_OK;
}

int cg_run_step(cg_run* r, int32_t nsteps, int32_t* bnd_stats_host) {
    NvtxRange nvtx_call("cg_run_step");
    if (!r || nsteps < 0) return CG_EINVAL;
    cg_ctx* c = r->ctx;
    if (nsteps == 0) return CG_OK;
    CUDA_TRY(c, cudaSetDevice(c->device));
    int rc = ensure_fields(r);
    if (rc) return rc;
    // a step's statistics row: max(1, nopen) exit counts, then the control
    // sections' counts
    const int nopen = c->nopen > 0 ? c->nopen : 1;
    const int row = nopen + r->dp.ncsec;
    if ((rc = ensure_stats(r, nsteps, row))) return rc;
    CUDA_TRY(c, cudaMemsetAsync(r->stats.p, 0, (size_t)nsteps * row * sizeof(int), c->stream));
    if (r->strand_on) CUDA_TRY(c, cudaMemsetAsync(r->strand.p, 0, sizeof(int), c->stream));
    // three timing events per step (before the step kernel, between it and
    // the walk, after the walk), created ahead by doubling (as the rows)
    const int nev = 3 * nsteps;
    if ((int)r->ev.size() < nev) {
        const int want = std::max(nev, std::max(2 * (int)r->ev.size(), 512));
        while ((int)r->ev.size() < want) {
            cudaEvent_t e;
            CUDA_TRY(c, cudaEventCreate(&e));
            r->ev.push_back(e);
        }
    }
    // element-sorted working state: gathered from the caller's arrays at the
    // first step after a write-back, re-sorted every sort_period steps
    // (counted across calls), kept resident between calls
    const bool sorted = r->sort_period > 0 && r->st.n > 0;
    if ((rc = start_queue(r, (int*)r->queue.p))) return rc;
    int launches = 0;   // kernels launched by this call
    // LSM1 2D runs (a walk queue; neither kernel reads the previous record):
    // step s + 1's blend writes the record that step s - 1 used, so it runs
    // on its own stream from the start of step s, overlapping the step's
    // tail and its walk
    const bool pre_blend = r->use_queue && !r->frozen && nsteps > 1;
    if (pre_blend && !r->bstream) {
        CUDA_TRY(c, cudaStreamCreateWithFlags(&r->bstream, cudaStreamNonBlocking));
        CUDA_TRY(c, cudaEventCreateWithFlags(&r->step_started, cudaEventDisableTiming));
        CUDA_TRY(c, cudaEventCreateWithFlags(&r->blended, cudaEventDisableTiming));
    }
    bool blended = false;   // this step's fields were blended during the last one
    for (int s = 0; s < nsteps; ++s) {
        // solver.pyx:440: fields at the step-start time
        if (blended) {
            CUDA_TRY(c, cudaStreamWaitEvent(c->stream, r->blended, 0));
            blended = false;
        } else if ((rc = time_interpolation(r, r->time))) {
            return rc;
        }
        if (!r->frozen) launches += 1;   // field blend
        // particles added since the last step: initialized with this step's
        // fields, then advanced by it (solver.pyx:443-470)
        if (s == 0 && r->pending_init) {
            if ((rc = write_back(r))) return rc;
            launch_init(r->prm.precision, c->mesh, field_view(r), r->dp, added_view(r),
                        r->prm.particle_velocity_init, -2 - (int)r->iteration,
                        (uint32_t*)r->errw.p, c->stream);
            r->pending_init = false;
            launches += 1;
        }
        if (sorted && (!r->resident || r->since_sort >= r->sort_period)) {
            NvtxRange nvtx_sort("element sort");
            if (!r->resident) launch_sort_gather(r->st, c->mesh.nt, r->sb, c->stream);
            else launch_sort_resort(r->st.n, c->mesh.nt, r->sb, c->stream);
            r->resident = true;
            r->since_sort = 0;
            launches += 6;   // histogram, 3 scan passes, index scatter, gather
        }
        const DevState run_state = sorted ? sorted_view(r->st, r->sb) : r->st;
        int aux = (s == nsteps - 1) ? 2 : (s == nsteps - 2 ? 1 : 0);
        int* stats = (int*)r->stats.p + (size_t)s * row;
        CUDA_TRY(c, cudaEventRecord(r->ev[3 * s], c->stream));
        const WalkQueue wq = next_queue(r, (int*)r->queue.p,
                                        (WalkEntry*)((char*)r->queue.p + 256));
        const FieldView fv = field_view(r);
        uint32_t* errw = (uint32_t*)r->errw.p;
        const int it = (int)r->iteration;
        if (pre_blend && s + 1 < nsteps) {
            // the next step's fields (the records swap in time_interpolation;
            // this step keeps the view taken above)
            CUDA_TRY(c, cudaEventRecord(r->step_started, c->stream));
            CUDA_TRY(c, cudaStreamWaitEvent(r->bstream, r->step_started, 0));
            if ((rc = time_interpolation(r, r->time + r->prm.time_step, r->bstream))) return rc;
            CUDA_TRY(c, cudaEventRecord(r->blended, r->bstream));
            blended = true;
        }
        if (r->prm.precision == CG_PRECISION_MIXED)
            launch_step_mixed(c->mesh, fv, r->dp, run_state, wq, aux, it, stats, errw, c->stream);
        else
            launch_step_plain(c->mesh, fv, r->dp, run_state, wq, aux, it, stats, errw, c->stream);
        CUDA_TRY(c, cudaEventRecord(r->ev[3 * s + 1], c->stream));
        if (r->use_queue) {
            if (r->prm.precision == CG_PRECISION_MIXED)
                launch_walk_mixed(c->mesh, fv, r->dp, run_state, wq, aux, it, stats, errw, c->stream);
            else
                launch_walk_plain(c->mesh, fv, r->dp, run_state, wq, aux, it, stats, errw, c->stream);
        }
        CUDA_TRY(c, cudaEventRecord(r->ev[3 * s + 2], c->stream));
        CUDA_TRY(c, cudaGetLastError());
        launches += r->st.n > 0 ? (r->use_queue ? 2 : 1) : 0;   // step (+ walk)
        if (sorted) r->since_sort += 1;
        // W_VEL2: this step's velocity array is now the newest
        if (sorted && (r->sb.work & W_VEL2) && aux >= 1) r->sb.vpar ^= 1;
        // simutime.pyx:77-84
        r->time += r->prm.time_step;
        r->iteration += 1;
    }
    if (r->st.depth) {
        // solver.pyx:526-538 after the call's last step
        launch_depth(r->prm.precision, c->mesh, field_view(r),
                     r->resident ? sorted_view(r->st, r->sb) : r->st, c->stream);
        launches += 1;
    }
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    double tot = 0., tstep = 0.;
    for (int s = 0; s < nsteps; ++s) {
        float ms = 0.f, ms1 = 0.f;
        CUDA_TRY(c, cudaEventElapsedTime(&ms, r->ev[3 * s], r->ev[3 * s + 2]));
        CUDA_TRY(c, cudaEventElapsedTime(&ms1, r->ev[3 * s], r->ev[3 * s + 1]));
        tot += ms;
        tstep += ms1;
    }
    r->last_ms = tot / nsteps;
    r->last_step_ms = tstep / nsteps;
    r->last_walk_ms = (tot - tstep) / nsteps;
    r->last_launches = launches;
    if (bnd_stats_host && c->nopen > 0)
        CUDA_TRY(c, cudaMemcpy2D(bnd_stats_host, (size_t)c->nopen * sizeof(int), r->stats.p,
                                 (size_t)row * sizeof(int), (size_t)c->nopen * sizeof(int),
                                 nsteps, cudaMemcpyDeviceToHost));
    if ((rc = collect_stranded(r))) return rc;
    if (r->dp.ncsec > 0) {
        r->csec_counts.resize((size_t)nsteps * r->dp.ncsec);
        CUDA_TRY(c, cudaMemcpy2D(r->csec_counts.data(), (size_t)r->dp.ncsec * sizeof(int),
                                 (const int*)r->stats.p + nopen, (size_t)row * sizeof(int),
                                 (size_t)r->dp.ncsec * sizeof(int), nsteps,
                                 cudaMemcpyDeviceToHost));
        r->csec_steps = nsteps;
    }
    uint32_t flags = 0;
    CUDA_TRY(c, cudaMemcpy(&flags, r->errw.p, sizeof flags, cudaMemcpyDeviceToHost));
    flags |= take_bounds_error(c);
    if (flags) return set_err(c, CG_EDEVICE, "device error flags 0x%x", flags);
    return CG_OK;
}

int cg_run_set_sections(cg_run* r, int32_t ncsec, const double* segments) {
    if (!r || ncsec < 0 || (ncsec > 0 && !segments)) return CG_EINVAL;
    cg_ctx* c = r->ctx;
    if (ncsec > CG_MAX_SECTIONS)
        return set_err(c, CG_EINVAL, "%d control sections, at most %d", ncsec, CG_MAX_SECTIONS);
    CUDA_TRY(c, cudaSetDevice(c->device));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    dfree(r->csec);
    r->dp.ncsec = 0;
    r->dp.csec = nullptr;
    r->csec_counts.clear();
    r->csec_steps = 0;
    if (ncsec == 0) return CG_OK;
    int rc = dalloc(c, r->csec, (size_t)ncsec * sizeof(SectionSeg));
    if (rc) return rc;
    CUDA_TRY(c, cudaMemcpy(r->csec.p, segments, (size_t)ncsec * sizeof(SectionSeg),
                           cudaMemcpyHostToDevice));
    r->dp.ncsec = ncsec;
    r->dp.csec = (const SectionSeg*)r->csec.p;
    return CG_OK;
}

// stranding record buffer for r->st.n particles (a stranded particle is
// deleted, so one call records each particle at most once)
static int alloc_strand(cg_ctx* c, cg_run* r) {
    dfree(r->strand);
    r->dp.strand_cap = 0;
    r->dp.strand_count = nullptr;
    r->dp.strand_rec = nullptr;
    r->strand_host.clear();
    if (!r->strand_on) return CG_OK;
    const size_t cap = r->st.n > 0 ? (size_t)r->st.n : 1;
    int rc = dalloc(c, r->strand, 256 + cap * sizeof(StrandRec));
    if (rc) return rc;
    r->dp.strand_cap = (int)cap;
    r->dp.strand_count = (int*)r->strand.p;
    r->dp.strand_rec = (StrandRec*)((char*)r->strand.p + 256);
    return CG_OK;
}

int cg_run_set_stranding_output(cg_run* r, int32_t on) {
    if (!r) return CG_EINVAL;
    cg_ctx* c = r->ctx;
    CUDA_TRY(c, cudaSetDevice(c->device));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    r->strand_on = on != 0;
    return alloc_strand(c, r);
}

int cg_run_stranded(const cg_run* r, double* xyz, int32_t* count) {
    if (!r) return CG_EINVAL;
    if (count) *count = (int32_t)r->strand_host.size();
    if (xyz)
        for (size_t k = 0; k < r->strand_host.size(); ++k) {
            xyz[3 * k] = r->strand_host[k].x;
            xyz[3 * k + 1] = r->strand_host[k].y;
            xyz[3 * k + 2] = r->strand_host[k].z;
        }
    return CG_OK;
}

int cg_run_section_stats(const cg_run* r, int32_t* counts, int32_t* nsteps) {
    if (!r) return CG_EINVAL;
    if (nsteps) *nsteps = r->csec_steps;
    if (counts && !r->csec_counts.empty())
        std::memcpy(counts, r->csec_counts.data(), r->csec_counts.size() * sizeof(int32_t));
    return CG_OK;
}

int cg_run_resize(cg_run* r, const cg_state_desc* s) {
    if (!r || !s || s->n < 0) return CG_EINVAL;
    cg_ctx* c = r->ctx;
    if (s->n > 0 && (!s->position || !s->velocity || !s->fluid_velocity_seen ||
                     !s->last_position || !s->last_velocity || !s->tri || !s->last_tri ||
                     !s->lowerlayer || !s->tag || !s->diameter || !s->rng_state))
        return set_err(c, CG_EINVAL, "incomplete particle state description");
    if (r->resident)
        return set_err(c, CG_ESTATE,
                       "cg_run_resize: the run's newest state is in its working copies; "
                       "call cg_run_writeback before replacing the particle arrays");
    CUDA_TRY(c, cudaSetDevice(c->device));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    const ScratchPlan plan = plan_scratch(c, &r->prm, s->n, s->depth != nullptr);
    const uint64_t old_state = state_bytes_of(r->st.n, r->prm.dim);
    const uint64_t new_state = state_bytes_of(s->n, r->prm.dim);
    const uint64_t old_bytes = r->bytes;
    const uint64_t new_bytes = old_bytes - old_state - r->scratch_bytes + new_state +
                               plan.queue_bytes + plan.sort_bytes;
    if (c->budget && c->used - old_bytes + new_bytes > c->budget)
        return set_err(c, CG_ENOMEM_BUDGET, "resized run needs %llu bytes, budget %llu",
                       (unsigned long long)new_bytes, (unsigned long long)c->budget);
    dfree(r->queue);
    dfree(r->sortbuf);
    int rc = take_scratch(c, r, plan);
    if (rc) {
        // the caller's old arrays are gone: the run keeps no particles
        r->st = DevState{};
        return rc;
    }
    c->used = c->used - old_bytes + new_bytes;
    r->bytes = new_bytes;
    r->scratch_bytes = plan.queue_bytes + plan.sort_bytes;
    DevState& st = r->st;
    st.n = s->n;
    st.pos = s->position;
    st.vel = s->velocity;
    st.fvs = s->fluid_velocity_seen;
    st.last_pos = s->last_position;
    st.last_vel = s->last_velocity;
    st.tri = s->tri;
    st.last_tri = s->last_tri;
    st.lowerlayer = s->lowerlayer;
    st.tag = s->tag;
    st.diameter = s->diameter;
    st.rng = s->rng_state;
    st.depth = (s->depth && r->prm.dim == 3) ? s->depth : nullptr;
    return alloc_strand(c, r);
}

int cg_run_added(cg_run* r, int32_t n_init) {
    if (!r || n_init < 0) return CG_EINVAL;
    cg_ctx* c = r->ctx;
    CUDA_TRY(c, cudaSetDevice(c->device));
    int rc = write_back(r);
    if (rc) return rc;
    launch_seed_added(r->st.tri, r->st.tag, r->st.rng, r->st.n, r->prm.seed, c->stream);
    CUDA_TRY(c, cudaGetLastError());
    r->pending_init = n_init > 0;
    r->init_n = n_init < r->st.n ? n_init : r->st.n;
    return CG_OK;
}

int cg_run_writeback(cg_run* r) {
    if (!r) return CG_EINVAL;
    cg_ctx* c = r->ctx;
    if (!r->resident) return CG_OK;
    CUDA_TRY(c, cudaSetDevice(c->device));
    return write_back(r);
}

int cg_rng_draws(cg_ctx* c, uint64_t seed, uint64_t stream, int32_t kind, int32_t method,
                 int64_t n, double* out_host) {
    if (!c || !out_host || n < 0 || kind < 0 || kind > 4 || method < 1 || method > 3)
        return set_err(c, CG_EINVAL, "cg_rng_draws: bad arguments");
    if (n == 0) return CG_OK;
    CUDA_TRY(c, cudaSetDevice(c->device));
    const size_t vals = (size_t)n * (kind == 3 ? 2 : 1);
    DevBuf buf, err;
    int rc;
    if ((rc = dalloc(c, buf, vals * sizeof(double))) || (rc = dalloc(c, err, 256))) {
        dfree(buf);
        return rc;
    }
    cudaMemsetAsync(err.p, 0, sizeof(uint32_t), c->stream);
    launch_rng_draws(seed, stream, kind, method, n, (double*)buf.p, (uint32_t*)err.p, c->stream);
    uint32_t flags = 0;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess) e = cudaMemcpy(out_host, buf.p, vals * sizeof(double), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&flags, err.p, sizeof flags, cudaMemcpyDeviceToHost);
    dfree(buf);
    dfree(err);
    if (e != cudaSuccess) return set_err(c, CG_ECUDA, "cg_rng_draws: %s", cudaGetErrorString(e));
    if (flags) return set_err(c, CG_EDEVICE, "device error flags 0x%x", flags);
    return CG_OK;
}

int cg_run_time(const cg_run* r, double* time, int64_t* iteration) {
    if (!r) return CG_EINVAL;
    if (time) *time = r->time;
    if (iteration) *iteration = r->iteration;
    return CG_OK;
}

// Allocation-free variant of cg_run_step: see include/cylag_gpu.h.
int cg_run_step_noalloc(cg_run* r, int32_t nsteps) {
    NvtxRange nvtx_call("cg_run_step_noalloc");
    if (!r || nsteps < 0) return CG_EINVAL;
    cg_ctx* c = r->ctx;
    if (r->st.n > CG_NOALLOC_MAX_PARTICLES)
        return set_err(c, CG_EINVAL,
                       "cg_run_step_noalloc: run has %d particles, the allocation-free "
                       "scratch holds at most %d (use cg_run_step)",
                       r->st.n, CG_NOALLOC_MAX_PARTICLES);
    // section counts and stranding records are per-call device buffers of
    // cg_run_step; this entry point produces neither, so it refuses runs
    // that asked for them rather than dropping them
    if (r->dp.ncsec > 0 || r->strand_on)
        return set_err(c, CG_EINVAL,
                       "cg_run_step_noalloc: the run has control sections or stranding output "
                       "on, which only cg_run_step records");
    r->last_ms = r->last_step_ms = r->last_walk_ms = 0.;
    r->last_launches = 0;
    if (nsteps == 0) return CG_OK;
    CUDA_TRY(c, cudaSetDevice(c->device));
    NoallocScratch* scratch = nullptr;
    int rc = noalloc_scratch(c, &scratch);
    if (rc) return rc;
    int launches = r->resident ? 1 : 0;   // the write-back of sorted working copies
    if ((rc = write_back(r))) return rc;
    if ((rc = ensure_fields(r))) return rc;
    if ((rc = start_queue(r, scratch->count))) return rc;
    for (int s = 0; s < nsteps; ++s) {
        if ((rc = time_interpolation(r, r->time))) return rc;
        if (!r->frozen) launches += 1;
        if (s == 0 && r->pending_init) {
            launch_init(r->prm.precision, c->mesh, field_view(r), r->dp, added_view(r),
                        r->prm.particle_velocity_init, -2 - (int)r->iteration,
                        (uint32_t*)r->errw.p, c->stream);
            r->pending_init = false;
            launches += 1;
        }
        int aux = (s == nsteps - 1) ? 2 : (s == nsteps - 2 ? 1 : 0);
        const WalkQueue wq = next_queue(r, scratch->count, scratch->entries);
        const FieldView fv = field_view(r);
        uint32_t* errw = (uint32_t*)r->errw.p;
        const int it = (int)r->iteration;
        if (r->prm.precision == CG_PRECISION_MIXED)
            launch_step_mixed(c->mesh, fv, r->dp, r->st, wq, aux, it, nullptr, errw, c->stream);
        else
            launch_step_plain(c->mesh, fv, r->dp, r->st, wq, aux, it, nullptr, errw, c->stream);
        if (wq.e) {
            if (r->prm.precision == CG_PRECISION_MIXED)
                launch_walk_mixed(c->mesh, fv, r->dp, r->st, wq, aux, it, nullptr, errw, c->stream);
            else
                launch_walk_plain(c->mesh, fv, r->dp, r->st, wq, aux, it, nullptr, errw, c->stream);
        }
        CUDA_TRY(c, cudaGetLastError());
        launches += r->st.n > 0 ? (wq.e ? 2 : 1) : 0;
        r->time += r->prm.time_step;
        r->iteration += 1;
    }
    if (r->st.depth) {
        launch_depth(r->prm.precision, c->mesh, field_view(r), r->st, c->stream);
        launches += 1;
    }
    r->last_launches = launches;
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    uint32_t flags = 0;
    CUDA_TRY(c, cudaMemcpy(&flags, r->errw.p, sizeof flags, cudaMemcpyDeviceToHost));
    flags |= take_bounds_error(c);
    if (flags) return set_err(c, CG_EDEVICE, "device error flags 0x%x", flags);
    return CG_OK;
}

// entries [a, a + m) of the particle state, as a state of m particles
static DevState slice_state(const DevState& s, int a, int m, int dim) {
    DevState v = s;
    const size_t av = (size_t)a * dim;
    v.n = m;
    v.pos += av;
    v.vel += av;
    v.fvs += av;
    v.last_pos += av;
    v.last_vel += av;
    v.tri += a;
    v.last_tri += a;
    v.lowerlayer += a;
    v.tag += a;
    v.diameter += a;
    v.rng += a;
    v.slot = nullptr;
    v.work = 0;
    v.base = s.base + a;
    return v;
}

// copies of entries [a, a + m) between the host arrays h and the run's state
static cudaError_t copy_chunk(const cg_run* r, const cg_host_arrays* h, bool to_device, int a,
                              int m, cudaStream_t st) {
    const int D = r->prm.dim;
    const DevState& d = r->st;
    struct A {
        void* host;
        void* dev;
        size_t elem;
    } arr[] = {{h->position, d.pos, 8u * D},       {h->velocity, d.vel, 8u * D},
               {h->fluid_velocity_seen, d.fvs, 8u * D}, {h->tri, d.tri, 4},
               {h->lowerlayer, d.lowerlayer, 4},   {h->tag, d.tag, 4},
               {h->rng_state, d.rng, 8}};
    for (const A& x : arr) {
        if (!x.host) continue;
        char* hp = (char*)x.host + (size_t)a * x.elem;
        char* dp = (char*)x.dev + (size_t)a * x.elem;
        cudaError_t e = to_device
            ? cudaMemcpyAsync(dp, hp, (size_t)m * x.elem, cudaMemcpyHostToDevice, st)
            : cudaMemcpyAsync(hp, dp, (size_t)m * x.elem, cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

int cg_run_step_host(cg_run* r, int32_t nsteps, const cg_host_arrays* in,
                     const cg_host_arrays* out, int32_t chunk, int32_t* bnd_stats_host) {
    NvtxRange nvtx_call("cg_run_step_host");
    if (!r || nsteps < 0 || !in || !out || chunk < 0) return CG_EINVAL;
    cg_ctx* c = r->ctx;
    if (nsteps == 0) return CG_OK;
    if (r->pending_init)
        return set_err(c, CG_ESTATE, "particles await initialization: step them with cg_run_step");
    CUDA_TRY(c, cudaSetDevice(c->device));
    int rc = write_back(r);
    if (rc) return rc;
    if ((rc = ensure_fields(r))) return rc;
    const int n = r->st.n, D = r->prm.dim;
    // chunk boundaries: `chunk` particles each, or (chunk == 0) four equal
    // chunks on 256-particle boundaries.  A chunk's copies overlap the other
    // chunks' steps and copies, across steps too (chunk j of step s + 1 waits
    // only for chunk j of step s), so the pipeline fills once per call; each
    // chunk costs a step and a walk launch, and the walk's duration hardly
    // depends on its queue: few chunks (measured with 1e7 particles: 4
    // chunks 4.91e9 particle-steps/s, 5: 4.86e9, 2: 4.63e9, 11: 4.46e9).
    // Boundaries off 256-particle multiples leave copies misaligned (3
    // chunks of 3,333,334: 4.1e9).
    std::vector<int> bounds{0};
    if (chunk > 0) {
        for (int a = chunk; a < n; a += chunk) bounds.push_back(a);
    } else if (n >= (1 << 20)) {
        const int c4 = (int)(((int64_t)n + 3) / 4 + 255) / 256 * 256;
        for (int a = c4; a < n; a += c4) bounds.push_back(a);
    } else {
        const int c8 = std::max(1 << 16, ((n + 7) / 8 + 255) / 256 * 256);
        for (int a = c8; a < n; a += c8) bounds.push_back(a);
    }
    if (n > 0) bounds.push_back(n);
    const int nch = (int)bounds.size() - 1;
    if (!r->h2d) CUDA_TRY(c, cudaStreamCreateWithFlags(&r->h2d, cudaStreamNonBlocking));
    if (!r->d2h) CUDA_TRY(c, cudaStreamCreateWithFlags(&r->d2h, cudaStreamNonBlocking));
    while ((int)r->hev.size() < 3 * nch + 1) {
        cudaEvent_t e;
        CUDA_TRY(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        r->hev.push_back(e);
    }
    cudaEvent_t* ev_in = r->hev.data();
    cudaEvent_t* ev_comp = ev_in + nch;
    cudaEvent_t* ev_out = ev_comp + nch;
    cudaEvent_t ev_start = r->hev[3 * nch];
    const int nopen = c->nopen > 0 ? c->nopen : 1;
    const int row = nopen + r->dp.ncsec;
    if ((rc = ensure_stats(r, nsteps, row))) return rc;
    CUDA_TRY(c, cudaMemsetAsync(r->stats.p, 0, (size_t)nsteps * row * sizeof(int), c->stream));
    if (r->strand_on) CUDA_TRY(c, cudaMemsetAsync(r->strand.p, 0, sizeof(int), c->stream));
    // the copy streams start after what is queued on the run's stream
    CUDA_TRY(c, cudaEventRecord(ev_start, c->stream));
    CUDA_TRY(c, cudaStreamWaitEvent(r->h2d, ev_start, 0));
    CUDA_TRY(c, cudaStreamWaitEvent(r->d2h, ev_start, 0));
    uint32_t* errw = (uint32_t*)r->errw.p;
    if ((rc = start_queue(r, (int*)r->queue.p))) return rc;
    for (int s = 0; s < nsteps; ++s) {
        if ((rc = time_interpolation(r, r->time))) return rc;
        const int aux = (s == nsteps - 1) ? 2 : (s == nsteps - 2 ? 1 : 0);
        int* stats = (int*)r->stats.p + (size_t)s * row;
        const FieldView fv = field_view(r);
        const int it = (int)r->iteration;
        for (int j = 0; j < nch; ++j) {
            const int a = bounds[j], m = bounds[j + 1] - bounds[j];
            // in: after the previous step's copy out of this chunk (the host
            // arrays may be the same)
            if (s > 0) CUDA_TRY(c, cudaStreamWaitEvent(r->h2d, ev_out[j], 0));
            CUDA_TRY(c, copy_chunk(r, in, true, a, m, r->h2d));
            CUDA_TRY(c, cudaEventRecord(ev_in[j], r->h2d));
            // step
            CUDA_TRY(c, cudaStreamWaitEvent(c->stream, ev_in[j], 0));
            const DevState v = slice_state(r->st, a, m, D);
            const WalkQueue wq = next_queue(r, (int*)r->queue.p,
                                            (WalkEntry*)((char*)r->queue.p + 256));
            if (r->prm.precision == CG_PRECISION_MIXED) {
                launch_step_mixed(c->mesh, fv, r->dp, v, wq, aux, it, stats, errw, c->stream);
                if (wq.e) launch_walk_mixed(c->mesh, fv, r->dp, v, wq, aux, it, stats, errw, c->stream);
            } else {
                launch_step_plain(c->mesh, fv, r->dp, v, wq, aux, it, stats, errw, c->stream);
                if (wq.e) launch_walk_plain(c->mesh, fv, r->dp, v, wq, aux, it, stats, errw, c->stream);
            }
            CUDA_TRY(c, cudaGetLastError());
            CUDA_TRY(c, cudaEventRecord(ev_comp[j], c->stream));
            // out
            CUDA_TRY(c, cudaStreamWaitEvent(r->d2h, ev_comp[j], 0));
            CUDA_TRY(c, copy_chunk(r, out, false, a, m, r->d2h));
            CUDA_TRY(c, cudaEventRecord(ev_out[j], r->d2h));
        }
        r->time += r->prm.time_step;
        r->iteration += 1;
    }
    if (r->st.depth) {
        // after every chunk's last step (the device state of the whole pool)
        for (int j = 0; j < nch; ++j) CUDA_TRY(c, cudaStreamWaitEvent(c->stream, ev_comp[j], 0));
        launch_depth(r->prm.precision, c->mesh, field_view(r), r->st, c->stream);
    }
    CUDA_TRY(c, cudaStreamSynchronize(r->d2h));
    CUDA_TRY(c, cudaStreamSynchronize(r->h2d));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if (bnd_stats_host && c->nopen > 0)
        CUDA_TRY(c, cudaMemcpy2D(bnd_stats_host, (size_t)c->nopen * sizeof(int), r->stats.p,
                                 (size_t)row * sizeof(int), (size_t)c->nopen * sizeof(int),
                                 nsteps, cudaMemcpyDeviceToHost));
    if (r->dp.ncsec > 0) {
        r->csec_counts.resize((size_t)nsteps * r->dp.ncsec);
        CUDA_TRY(c, cudaMemcpy2D(r->csec_counts.data(), (size_t)r->dp.ncsec * sizeof(int),
                                 (const int*)r->stats.p + nopen, (size_t)row * sizeof(int),
                                 (size_t)r->dp.ncsec * sizeof(int), nsteps,
                                 cudaMemcpyDeviceToHost));
        r->csec_steps = nsteps;
    }
    if ((rc = collect_stranded(r))) return rc;
    uint32_t flags = 0;
    CUDA_TRY(c, cudaMemcpy(&flags, r->errw.p, sizeof flags, cudaMemcpyDeviceToHost));
    flags |= take_bounds_error(c);
    if (flags) return set_err(c, CG_EDEVICE, "device error flags 0x%x", flags);
    return CG_OK;
}

int cg_run_errors(cg_run* r, uint32_t* flags) {
    if (!r || !flags) return CG_EINVAL;
    cg_ctx* c = r->ctx;
    CUDA_TRY(c, cudaSetDevice(c->device));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    CUDA_TRY(c, cudaMemcpy(flags, r->errw.p, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    CUDA_TRY(c, cudaMemset(r->errw.p, 0, sizeof(uint32_t)));
    return CG_OK;
}

int cg_run_last_kernel_ms(const cg_run* r, double* ms, int32_t* launches) {
    if (!r) return CG_EINVAL;
    if (ms) *ms = r->last_ms;
    if (launches) *launches = r->last_launches;
    return CG_OK;
}

int cg_run_last_kernel_split_ms(const cg_run* r, double* step_ms, double* walk_ms) {
    if (!r) return CG_EINVAL;
    if (step_ms) *step_ms = r->last_step_ms;
    if (walk_ms) *walk_ms = r->last_walk_ms;
    return CG_OK;
}

int cg_run_clock(const cg_run* r, double* time, double* fields_time, int64_t* iteration) {
    if (!r) return CG_EINVAL;
    if (time) *time = r->time;
    if (fields_time) *fields_time = r->frozen ? NAN : r->fields_time;
    if (iteration) *iteration = r->iteration;
    return CG_OK;
}

int cg_run_resume(cg_run* r, double time, double fields_time, int64_t iteration) {
    if (!r) return CG_EINVAL;
    cg_ctx* c = r->ctx;
    CUDA_TRY(c, cudaSetDevice(c->device));
    if (r->pending_init)
        return set_err(c, CG_ESTATE, "particles await initialization: resume a stepped run");
    int rc = write_back(r);
    if (rc) return rc;
    if ((rc = ensure_fields(r))) return rc;
    r->time = time;
    r->iteration = iteration;
    if (!r->frozen && std::isfinite(fields_time)) {
        // the current record as the checkpointed run held it (blended at
        // its last step's time): the first resumed step's previous record,
        // as in the uninterrupted run
        r->record = 0;
        if ((rc = time_interpolation(r, fields_time))) return rc;
    }
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return CG_OK;
}

}  // extern "C"
