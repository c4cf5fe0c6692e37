// cg_server.cu -- the serving pool behind cg_server_* (include/cylag_gpu.h).
//
// Many dispersion runs share one context (mesh and frozen field records
// resident in HBM) and one pool of particle state.  A run is admitted when a
// contiguous range of warps is free in the pool (memory admission), steps in
// the same launch as every other admitted run (serve_step_kernel, captured
// once in a CUDA graph and replayed each step), and is read back and
// released when its horizon is reached, so runs that arrive while others
// are on the GPU start at the next step (continuous batching).
//
// Ordering: kernels and the run-table / active-list uploads go on the
// context stream; a new run's positions are copied on a second stream,
// which the context stream then waits for, so admissions overlap the steps
// already queued; results are read on the second stream after an event
// recorded behind the run's last step.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <new>
#include <vector>

#include "cg_host.h"

namespace cg {

// a newly admitted run's range: awaiting initialization (tri = -2), tags
// 0..n-1 (its PCG32 stream ids), zero velocities and last state, diameters
// (dflt <= 0: the diameters were copied in already)
__global__ void serve_prepare_kernel(DevState v, double dflt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.n) return;
    v.tri[i] = -2;
    v.last_tri[i] = -1;
    v.lowerlayer[i] = 0;
    v.tag[i] = i;
    if (dflt > 0.) v.diameter[i] = dflt;
    reinterpret_cast<double2*>(v.vel)[i] = make_double2(0., 0.);
    reinterpret_cast<double2*>(v.fvs)[i] = make_double2(0., 0.);
    reinterpret_cast<double2*>(v.last_vel)[i] = make_double2(0., 0.);
    reinterpret_cast<double2*>(v.last_pos)[i] = reinterpret_cast<const double2*>(v.pos)[i];
}

}  // namespace cg

namespace {

constexpr size_t BYTES_PER_PARTICLE = 5 * 16 + 4 * 4 + 8 + 8;   // 2D pool arrays
constexpr int NUM_EVENTS = 64;

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

}  // namespace

struct cg_server {
    cg_ctx* ctx = nullptr;
    int precision = 0;
    int64_t capacity = 0;   // particles, multiple of 32
    int max_runs = 0;
    DevBuf pool_buf, rec_buf, turb_buf, runs_buf, active_buf, nactive_buf, clock_buf, err_buf;
    DevState pool{};
    double sigc = 1.0;      // Schmidt number of the nodal k-epsilon diffusivity in the records
    int grid = 0;
    cudaStream_t copy = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t issued = 0;     // steps launched
    // free warps: start -> length
    std::map<int, int> free_warps;
    struct Run {
        bool used = false;
        int first = 0, count = 0, nwarps = 0, horizon = 0;
        int64_t start = 0;
    };
    std::vector<Run> runs;
    std::vector<int> free_ids;
    std::vector<int2> active;
    // pinned staging
    int2* active_h[2] = {nullptr, nullptr};
    cudaEvent_t active_ev[2] = {nullptr, nullptr};
    int active_flip = 0;
    ServeRun* runs_h = nullptr;
    std::vector<cudaEvent_t> table_ev;   // per run slot: its last table upload
    double* stage_h = nullptr;
    size_t stage_cap = 0;
    cudaEvent_t stage_ev = nullptr, cancel_ev = nullptr;
    bool cancel_pending = false;
    // events behind step calls: (global step after the call, event)
    std::vector<std::pair<int64_t, cudaEvent_t>> marks;
    std::vector<cudaEvent_t> spare;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    int last_nsteps = 0;
    uint64_t bytes = 0;
};

static FieldView server_view(const cg_server* s) {
    const cg_ctx* c = s->ctx;
    return FieldView{s->rec_buf.p, s->rec_buf.p, s->turb_buf.p, c->npoints, c->nlayers, c->fdim, 0};
}

static DevState range_view(const cg_server* s, int first, int n) {
    DevState v = s->pool;
    v.n = n;
    v.pos += 2 * (size_t)first;
    v.vel += 2 * (size_t)first;
    v.fvs += 2 * (size_t)first;
    v.last_pos += 2 * (size_t)first;
    v.last_vel += 2 * (size_t)first;
    v.tri += first;
    v.last_tri += first;
    v.lowerlayer += first;
    v.tag += first;
    v.diameter += first;
    v.rng += first;
    v.slot = nullptr;
    return v;
}

// uploads the active-warp list (pinned double buffer)
static int upload_active(cg_server* s) {
    cg_ctx* c = s->ctx;
    int b = s->active_flip;
    s->active_flip ^= 1;
    CUDA_TRY(c, cudaEventSynchronize(s->active_ev[b]));   // the buffer's previous copy is done
    int n = (int)s->active.size();
    if (n) std::memcpy(s->active_h[b], s->active.data(), n * sizeof(int2));
    s->active_h[b][s->capacity / 32].x = n;                // count travels in the spare slot
    if (n)
        CUDA_TRY(c, cudaMemcpyAsync(s->active_buf.p, s->active_h[b], n * sizeof(int2),
                                    cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(s->nactive_buf.p, &s->active_h[b][s->capacity / 32].x,
                                sizeof(int), cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(c, cudaEventRecord(s->active_ev[b], c->stream));
    return CG_OK;
}

static cudaEvent_t take_event(cg_server* s) {
    if (!s->spare.empty()) {
        cudaEvent_t e = s->spare.back();
        s->spare.pop_back();
        return e;
    }
    // recycle the oldest mark (wait for it: later marks cover later steps)
    cudaEvent_t e = s->marks.front().second;
    cudaEventSynchronize(e);
    s->marks.erase(s->marks.begin());
    return e;
}

static void destroy_server(cg_server* s) {
    if (!s) return;
    cg_ctx* c = s->ctx;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    if (s->copy) cudaStreamSynchronize(s->copy);
    if (s->exec) cudaGraphExecDestroy(s->exec);
    for (DevBuf* b : {&s->pool_buf, &s->rec_buf, &s->turb_buf, &s->runs_buf, &s->active_buf,
                      &s->nactive_buf, &s->clock_buf, &s->err_buf})
        dfree(*b);
    for (cudaEvent_t e : s->table_ev)
        if (e) cudaEventDestroy(e);
    for (int k = 0; k < 2; ++k) {
        if (s->active_h[k]) cudaFreeHost(s->active_h[k]);
        if (s->active_ev[k]) cudaEventDestroy(s->active_ev[k]);
    }
    if (s->runs_h) cudaFreeHost(s->runs_h);
    if (s->stage_h) cudaFreeHost(s->stage_h);
    for (cudaEvent_t e : {s->stage_ev, s->cancel_ev, s->t0, s->t1})
        if (e) cudaEventDestroy(e);
    for (auto& m : s->marks) cudaEventDestroy(m.second);
    for (auto e : s->spare) cudaEventDestroy(e);
    if (s->copy) cudaStreamDestroy(s->copy);
    c->used -= s->bytes;
    delete s;
}

extern "C" {

int cg_server_create(cg_ctx* c, int32_t precision, int64_t capacity, int32_t max_runs,
                     double schmidt_number, cg_server** out) {
    if (!c || !out || capacity <= 0 || max_runs <= 0 || !(schmidt_number > 0.)) return CG_EINVAL;
    *out = nullptr;
    if (!c->have_mesh || !c->have_fields)
        return set_err(c, CG_ESTATE, "cg_server_create before mesh/field upload");
    if (c->fdim != 2) return set_err(c, CG_EINVAL, "the serving pool steps 2D runs");
    if (precision != CG_PRECISION_FP64 && precision != CG_PRECISION_MIXED)
        return set_err(c, CG_EINVAL, "unknown precision %d", precision);
    if (capacity > ((int64_t)1 << 31) - 64)
        return set_err(c, CG_EINVAL, "pool capacity above 2^31 particles");
    CUDA_TRY(c, cudaSetDevice(c->device));
    capacity = (capacity + 31) / 32 * 32;
    const int64_t nwarps = capacity / 32;
    const size_t rec = record_bytes(2, precision) * c->frames.nnodes;
    const size_t turb = c->has_keps ? 2 * c->frames.nnodes * (precision ? 4 : 8) : 0;
    const size_t pool_bytes = align256((size_t)capacity * BYTES_PER_PARTICLE) + 11 * 256;
    const uint64_t need = pool_bytes + rec + turb + (size_t)max_runs * (sizeof(ServeRun) + 4) +
                          (size_t)nwarps * sizeof(int2) + 512;
    if (c->budget && c->used + need > c->budget)
        return set_err(c, CG_ENOMEM_BUDGET, "serving pool needs %llu bytes, %llu of %llu in use",
                       (unsigned long long)need, (unsigned long long)c->used,
                       (unsigned long long)c->budget);
    cg_server* s = new (std::nothrow) cg_server();
    if (!s) return set_err(c, CG_EINVAL, "out of host memory");
    s->ctx = c;
    s->precision = precision;
    s->sigc = schmidt_number;
    s->capacity = capacity;
    s->max_runs = max_runs;
    int rc;
    if ((rc = dalloc(c, s->pool_buf, pool_bytes)) || (rc = dalloc(c, s->rec_buf, rec)) ||
        (rc = dalloc(c, s->turb_buf, turb)) ||
        (rc = dalloc(c, s->runs_buf, (size_t)max_runs * sizeof(ServeRun))) ||
        (rc = dalloc(c, s->active_buf, (size_t)nwarps * sizeof(int2))) ||
        (rc = dalloc(c, s->nactive_buf, 256)) || (rc = dalloc(c, s->clock_buf, 256)) ||
        (rc = dalloc(c, s->err_buf, (size_t)max_runs * 4))) {
        destroy_server(s);
        return rc;
    }
    s->bytes = need;
    c->used += need;
    // pool arrays, 256-byte aligned
    char* p = (char*)s->pool_buf.p;
    auto take = [&](size_t b) { char* q = p; p += align256(b); return q; };
    const size_t n = (size_t)capacity;
    s->pool.n = (int)capacity;
    s->pool.pos = (double*)take(n * 16);
    s->pool.vel = (double*)take(n * 16);
    s->pool.fvs = (double*)take(n * 16);
    s->pool.last_pos = (double*)take(n * 16);
    s->pool.last_vel = (double*)take(n * 16);
    s->pool.tri = (int*)take(n * 4);
    s->pool.last_tri = (int*)take(n * 4);
    s->pool.lowerlayer = (int*)take(n * 4);
    s->pool.tag = (int*)take(n * 4);
    s->pool.diameter = (double*)take(n * 8);
    s->pool.rng = (uint64_t*)take(n * 8);
    s->pool.slot = nullptr;
    CUDA_TRY(c, cudaMemsetAsync(s->pool.tri, 0xff, n * 4, c->stream));   // -1: empty
    CUDA_TRY(c, cudaMemsetAsync(s->nactive_buf.p, 0, 256, c->stream));
    CUDA_TRY(c, cudaMemsetAsync(s->clock_buf.p, 0, 256, c->stream));
    CUDA_TRY(c, cudaMemsetAsync(s->err_buf.p, 0, (size_t)max_runs * 4, c->stream));
    // frozen field records (record 0) and, with k-epsilon fields, {k, eps}
    launch_blend(c->frames, 0, 1.0, true, CMU / schmidt_number, s->rec_buf.p, s->turb_buf.p,
                 precision, 2, c->stream);
    CUDA_TRY(c, cudaGetLastError());
    CUDA_TRY(c, cudaStreamCreateWithFlags(&s->copy, cudaStreamNonBlocking));
    for (int k = 0; k < 2; ++k) {
        CUDA_TRY(c, cudaMallocHost(&s->active_h[k], (size_t)(nwarps + 1) * sizeof(int2)));
        CUDA_TRY(c, cudaEventCreateWithFlags(&s->active_ev[k], cudaEventDisableTiming));
    }
    CUDA_TRY(c, cudaMallocHost(&s->runs_h, (size_t)max_runs * sizeof(ServeRun)));
    for (cudaEvent_t* e : {&s->stage_ev, &s->cancel_ev})
        CUDA_TRY(c, cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    CUDA_TRY(c, cudaEventCreate(&s->t0));
    CUDA_TRY(c, cudaEventCreate(&s->t1));
    for (int k = 0; k < NUM_EVENTS; ++k) {
        cudaEvent_t e;
        CUDA_TRY(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        s->spare.push_back(e);
    }
    s->runs.resize(max_runs);
    s->table_ev.assign(max_runs, nullptr);
    for (int k = 0; k < max_runs; ++k)
        CUDA_TRY(c, cudaEventCreateWithFlags(&s->table_ev[k], cudaEventDisableTiming));
    for (int k = max_runs - 1; k >= 0; --k) s->free_ids.push_back(k);
    s->free_warps[0] = (int)nwarps;
    s->grid = precision ? serve_grid_mixed() : serve_grid_plain();
    // the step, captured once
    DevMesh m = c->mesh;
    FieldView fv = server_view(s);
    cudaGraph_t g = nullptr;
    CUDA_TRY(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    if (precision)
        launch_serve_mixed(s->grid, m, fv, s->pool, (const ServeRun*)s->runs_buf.p,
                           (const int2*)s->active_buf.p, (const int*)s->nactive_buf.p,
                           (ServeClock*)s->clock_buf.p, (uint32_t*)s->err_buf.p, c->stream);
    else
        launch_serve_plain(s->grid, m, fv, s->pool, (const ServeRun*)s->runs_buf.p,
                           (const int2*)s->active_buf.p, (const int*)s->nactive_buf.p,
                           (ServeClock*)s->clock_buf.p, (uint32_t*)s->err_buf.p, c->stream);
    cudaError_t e1 = cudaStreamEndCapture(c->stream, &g);
    if (e1 != cudaSuccess) {
        destroy_server(s);
        return set_err(c, CG_ECUDA, "graph capture failed: %s", cudaGetErrorString(e1));
    }
    e1 = cudaGraphInstantiate(&s->exec, g, 0);
    cudaGraphDestroy(g);
    if (e1 != cudaSuccess) {
        destroy_server(s);
        return set_err(c, CG_ECUDA, "graph instantiation failed: %s", cudaGetErrorString(e1));
    }
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    *out = s;
    return CG_OK;
}

int cg_server_destroy(cg_server* s) {
    if (!s) return CG_EINVAL;
    destroy_server(s);
    return CG_OK;
}

int cg_server_admit(cg_server* s, const cg_params* prm, int32_t n, const double* position,
                    double particle_diameter, const double* diameter, int32_t horizon,
                    int32_t* run_id) {
    NvtxRange nvtx("cg_server_admit");
    if (!s || !prm || !position || !run_id || n <= 0 || horizon <= 0) return CG_EINVAL;
    cg_ctx* c = s->ctx;
    *run_id = -1;
    int rc = check_params(c, prm);
    if (rc) return rc;
    if (prm->precision != s->precision)
        return set_err(c, CG_EINVAL, "run precision %d differs from the pool's %d",
                       prm->precision, s->precision);
    if (!prm->frozen_eulerian_fields && c->times.size() > 1)
        return set_err(c, CG_EINVAL, "the serving pool steps runs on frozen fields");
    if (!(prm->time_step > 0.)) return set_err(c, CG_EINVAL, "bad time_step");
    if (!(particle_diameter > 0.) && !diameter)
        return set_err(c, CG_EINVAL, "particle_diameter must be > 0");
    // the records hold K for one Schmidt number (eulerian_field_set.pyx:1995-1997)
    const bool uses_k = (prm->diffusion_model == 2 || prm->diffusion_model == 3) &&
                        (prm->model == 1 || (prm->model == 2 && prm->diffusion_lsm2_option == 1));
    if (uses_k && prm->schmidt_number != s->sigc)
        return set_err(c, CG_EINVAL, "schmidt_number %g differs from the pool's %g",
                       prm->schmidt_number, s->sigc);
    const int nw = (n + 31) / 32;
    auto it = std::find_if(s->free_warps.begin(), s->free_warps.end(),
                           [&](const std::pair<const int, int>& e) { return e.second >= nw; });
    if (it == s->free_warps.end())
        return set_err(c, CG_ENOMEM_BUDGET, "no free range of %d particles in the pool", n);
    if (s->free_ids.empty()) return set_err(c, CG_ENOMEM_BUDGET, "run table full");
    CUDA_TRY(c, cudaSetDevice(c->device));
    const int w0 = it->first, len = it->second;
    s->free_warps.erase(it);
    if (len > nw) s->free_warps[w0 + nw] = len - nw;
    const int id = s->free_ids.back();
    s->free_ids.pop_back();
    const int first = w0 * 32;
    // positions (and diameters) through pinned staging on the copy stream
    const size_t pos_bytes = (size_t)n * 16, dia_bytes = diameter ? (size_t)n * 8 : 0;
    CUDA_TRY(c, cudaEventSynchronize(s->stage_ev));
    if (s->stage_cap < pos_bytes + dia_bytes) {
        if (s->stage_h) cudaFreeHost(s->stage_h);
        s->stage_h = nullptr;
        s->stage_cap = 0;
        CUDA_TRY(c, cudaMallocHost(&s->stage_h, pos_bytes + dia_bytes));
        s->stage_cap = pos_bytes + dia_bytes;
    }
    std::memcpy(s->stage_h, position, pos_bytes);
    if (diameter) std::memcpy((char*)s->stage_h + pos_bytes, diameter, dia_bytes);
    if (s->cancel_pending) CUDA_TRY(c, cudaStreamWaitEvent(s->copy, s->cancel_ev, 0));
    DevState v = range_view(s, first, n);
    CUDA_TRY(c, cudaMemcpyAsync(v.pos, s->stage_h, pos_bytes, cudaMemcpyHostToDevice, s->copy));
    if (diameter)
        CUDA_TRY(c, cudaMemcpyAsync(v.diameter, (char*)s->stage_h + pos_bytes, dia_bytes,
                                    cudaMemcpyHostToDevice, s->copy));
    CUDA_TRY(c, cudaEventRecord(s->stage_ev, s->copy));
    CUDA_TRY(c, cudaStreamWaitEvent(c->stream, s->stage_ev, 0));
    // prepare, seed, initialize (Solver.__init__ + initialize_particle_state)
    DevParams dp;
    make_dev_params(c, prm, dp);
    serve_prepare_kernel<<<(n + 255) / 256, 256, 0, c->stream>>>(v, diameter ? 0. : particle_diameter);
    launch_seed(v.tag, v.rng, n, prm->seed, c->stream);
    CUDA_TRY(c, cudaMemsetAsync((uint32_t*)s->err_buf.p + id, 0, 4, c->stream));
    launch_init(s->precision, c->mesh, server_view(s), dp, v, prm->particle_velocity_init, -1,
                (uint32_t*)s->err_buf.p + id, c->stream);
    CUDA_TRY(c, cudaGetLastError());
    // run table entry: step 0 at the next launched step (the pinned slot's
    // previous upload must have been read before it is rewritten)
    CUDA_TRY(c, cudaEventSynchronize(s->table_ev[id]));
    ServeRun& R = s->runs_h[id];
    R.p = dp;
    R.first = first;
    R.count = n;
    R.horizon = horizon;
    R.pad = 0;
    R.start = (long long)s->issued;
    CUDA_TRY(c, cudaMemcpyAsync((ServeRun*)s->runs_buf.p + id, &R, sizeof(ServeRun),
                                cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(c, cudaEventRecord(s->table_ev[id], c->stream));
    for (int w = 0; w < nw; ++w) s->active.push_back(make_int2(w0 + w, id));
    if ((rc = upload_active(s))) return rc;
    cg_server::Run& H = s->runs[id];
    H.used = true;
    H.first = first;
    H.count = n;
    H.nwarps = nw;
    H.horizon = horizon;
    H.start = s->issued;
    *run_id = id;
    return CG_OK;
}

int cg_server_step(cg_server* s, int32_t nsteps) {
    NvtxRange nvtx("cg_server_step");
    if (!s || nsteps < 0) return CG_EINVAL;
    cg_ctx* c = s->ctx;
    if (nsteps == 0) return CG_OK;
    CUDA_TRY(c, cudaSetDevice(c->device));
    CUDA_TRY(c, cudaEventRecord(s->t0, c->stream));
    for (int k = 0; k < nsteps; ++k) CUDA_TRY(c, cudaGraphLaunch(s->exec, c->stream));
    CUDA_TRY(c, cudaEventRecord(s->t1, c->stream));
    s->issued += nsteps;
    s->last_nsteps = nsteps;
    cudaEvent_t e = take_event(s);
    CUDA_TRY(c, cudaEventRecord(e, c->stream));
    s->marks.emplace_back(s->issued, e);
    return CG_OK;
}

int cg_server_run_status(const cg_server* s, int32_t id, int32_t* steps_left) {
    if (!s || !steps_left || id < 0 || id >= s->max_runs || !s->runs[id].used) return CG_EINVAL;
    const cg_server::Run& H = s->runs[id];
    int64_t left = H.start + H.horizon - s->issued;
    *steps_left = (int32_t)(left > 0 ? left : 0);
    return CG_OK;
}

int cg_server_read(cg_server* s, int32_t id, double* position, double* velocity, double* fvs,
                   int32_t* tri, int32_t* tag, uint64_t* rng_state, uint32_t* err_flags) {
    if (!s || id < 0 || id >= s->max_runs || !s->runs[id].used) return CG_EINVAL;
    cg_ctx* c = s->ctx;
    const cg_server::Run& H = s->runs[id];
    const int64_t end = H.start + H.horizon;
    if (s->issued < end)
        return set_err(c, CG_ESTATE, "run %d has %lld steps left", id,
                       (long long)(end - s->issued));
    CUDA_TRY(c, cudaSetDevice(c->device));
    auto mk = std::find_if(s->marks.begin(), s->marks.end(),
                           [&](const std::pair<int64_t, cudaEvent_t>& m) { return m.first >= end; });
    if (mk == s->marks.end()) return set_err(c, CG_ESTATE, "no step event behind run %d", id);
    CUDA_TRY(c, cudaStreamWaitEvent(s->copy, mk->second, 0));
    DevState v = range_view(s, H.first, H.count);
    const size_t n = (size_t)H.count;
    if (position) CUDA_TRY(c, cudaMemcpyAsync(position, v.pos, n * 16, cudaMemcpyDeviceToHost, s->copy));
    if (velocity) CUDA_TRY(c, cudaMemcpyAsync(velocity, v.vel, n * 16, cudaMemcpyDeviceToHost, s->copy));
    if (fvs) CUDA_TRY(c, cudaMemcpyAsync(fvs, v.fvs, n * 16, cudaMemcpyDeviceToHost, s->copy));
    if (tri) CUDA_TRY(c, cudaMemcpyAsync(tri, v.tri, n * 4, cudaMemcpyDeviceToHost, s->copy));
    if (tag) CUDA_TRY(c, cudaMemcpyAsync(tag, v.tag, n * 4, cudaMemcpyDeviceToHost, s->copy));
    if (rng_state) CUDA_TRY(c, cudaMemcpyAsync(rng_state, v.rng, n * 8, cudaMemcpyDeviceToHost, s->copy));
    uint32_t flags = 0;
    CUDA_TRY(c, cudaMemcpyAsync(&flags, (uint32_t*)s->err_buf.p + id, 4, cudaMemcpyDeviceToHost,
                                s->copy));
    CUDA_TRY(c, cudaStreamSynchronize(s->copy));
    if (err_flags) *err_flags = flags;
    if (flags) return set_err(c, CG_EDEVICE, "run %d: device error flags 0x%x", id, flags);
    return CG_OK;
}

int cg_server_release(cg_server* s, int32_t id) {
    if (!s || id < 0 || id >= s->max_runs || !s->runs[id].used) return CG_EINVAL;
    cg_ctx* c = s->ctx;
    CUDA_TRY(c, cudaSetDevice(c->device));
    cg_server::Run& H = s->runs[id];
    const bool finished = s->issued >= H.start + H.horizon;
    s->active.erase(std::remove_if(s->active.begin(), s->active.end(),
                                   [&](const int2& e) { return e.y == id; }),
                    s->active.end());
    int rc = upload_active(s);
    if (rc) return rc;
    if (!finished) {
        // steps already queued may still write the range: a later admission
        // into it waits for this point of the context stream
        CUDA_TRY(c, cudaEventRecord(s->cancel_ev, c->stream));
        s->cancel_pending = true;
    }
    // return the range, merging with free neighbours
    int w0 = H.first / 32, len = H.nwarps;
    auto nx = s->free_warps.lower_bound(w0);
    if (nx != s->free_warps.end() && nx->first == w0 + len) {
        len += nx->second;
        nx = s->free_warps.erase(nx);
    }
    if (nx != s->free_warps.begin()) {
        auto pv = std::prev(nx);
        if (pv->first + pv->second == w0) {
            w0 = pv->first;
            len += pv->second;
            s->free_warps.erase(pv);
        }
    }
    s->free_warps[w0] = len;
    H = cg_server::Run{};
    s->free_ids.push_back(id);
    return CG_OK;
}

int cg_server_stats(cg_server* s, int32_t* active_runs, int64_t* active_particles,
                    int64_t* largest_free, int64_t* steps_issued, double* last_step_ms) {
    if (!s) return CG_EINVAL;
    cg_ctx* c = s->ctx;
    int nr = 0;
    int64_t np = 0, lf = 0;
    for (const auto& H : s->runs)
        if (H.used) {
            ++nr;
            np += H.count;
        }
    for (const auto& f : s->free_warps) lf = std::max<int64_t>(lf, (int64_t)f.second * 32);
    if (active_runs) *active_runs = nr;
    if (active_particles) *active_particles = np;
    if (largest_free) *largest_free = lf;
    if (steps_issued) *steps_issued = s->issued;
    if (last_step_ms) {
        *last_step_ms = 0.;
        if (s->last_nsteps > 0) {
            CUDA_TRY(c, cudaEventSynchronize(s->t1));
            float ms = 0.f;
            CUDA_TRY(c, cudaEventElapsedTime(&ms, s->t0, s->t1));
            *last_step_ms = ms / s->last_nsteps;
        }
    }
    return CG_OK;
}

}  // extern "C"
