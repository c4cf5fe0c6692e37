// cg_host.h -- host-side pieces shared by the C-ABI translation units
// (cg_api.cu: contexts and runs; cg_server.cu: the serving pool).  Not part
// of the public ABI.
#pragma once

#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/cylag_gpu.h"
#include "cg_internal.h"

using namespace cg;

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

struct cg_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;      // stream all work is issued on
    cudaStream_t own_stream = nullptr;  // the context's own stream
    uint64_t budget = 0;
    uint64_t used = 0;
    std::string err;
    // mesh
    bool have_mesh = false;
    DevMesh mesh{};
    int nopen = 0;
    std::vector<DevBuf> mesh_bufs;
    // fields
    bool have_fields = false;
    DevFrames frames{};
    DevBuf frames_buf;
    DevBuf frames32_buf;
    std::vector<double> times;
    int fdim = 2, nlayers = 1, npoints = 0;
    bool has_keps = false;
    bool has_bottom = false;
    int friction_model = 1;
    double friction_coef = 40.;
};

inline int set_err(cg_ctx* c, int code, const char* fmt, ...) {
    if (c) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        c->err = buf;
    }
    return code;
}

#define CUDA_TRY(c, call)                                                                    \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            return set_err((c), CG_ECUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

inline int dalloc(cg_ctx* c, DevBuf& b, size_t bytes) {
    b.bytes = bytes;
    if (bytes == 0) { b.p = nullptr; return CG_OK; }
    CUDA_TRY(c, cudaMalloc(&b.p, bytes));
    return CG_OK;
}

inline void dfree(DevBuf& b) {
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
}


// parameters.pyx:208-279 (model / scheme / option combinations) and the
// GPU-specific restrictions; CG_OK or CG_EINVAL with the message set
int check_params(cg_ctx* c, const cg_params* p);
// device copy of the run parameters and particle coefficients
// (lagrangian_particle_set.pyx:355-375, update_state_lsm1.pyx:708-713)
void make_dev_params(const cg_ctx* c, const cg_params* p, DevParams& d);
