// Internal definition of the C-ABI context (include/meso_gpu.h).
#pragma once

#include <cuda_runtime.h>

#include <ctime>
#include <new>
#include <memory>
#include <string>
#include <vector>

#include "host/case.h"
#include "host/renumber.h"
#include "host/tiles.h"
#include "kernels/fp32_step.h"
#include "kernels/plain_fp64.h"
#include "meso_gpu.h"

namespace meso_host {

// The device allocations of one context: small arrays are carved (256-byte aligned) out of 8 MiB
// blocks and large ones get their own allocation, so a context costs a few cudaMalloc / cudaFree
// calls rather than one per array (admission and retirement of served solves).  `bytes` counts
// what the blocks and large arrays hold on the device.
struct DevArena {
    static constexpr size_t kBlock = (size_t)8 << 20, kAlign = 256;
    std::vector<void *> ptrs;
    size_t bytes = 0;
    char *cur = nullptr;
    size_t left = 0;
    template <class T> T *alloc(size_t n) {
        if (n == 0) n = 1;
        const size_t want = (n * sizeof(T) + kAlign - 1) / kAlign * kAlign;
        if (want > kBlock / 4) return static_cast<T *>(raw(want));
        if (want > left) {
            cur = static_cast<char *>(raw(kBlock));
            left = kBlock;
        }
        T *r = reinterpret_cast<T *>(cur);
        cur += want;
        left -= want;
        return r;
    }
    void *raw(size_t nbytes) {
        void *p = nullptr;
        if (cudaMalloc(&p, nbytes) != cudaSuccess) throw std::bad_alloc();
        ptrs.push_back(p);
        bytes += nbytes;
        return p;
    }
    void release();
    ~DevArena() { release(); }
};

void set_error(const std::string &msg);
const char *last_error_cstr();
int fail(int code, const std::string &msg);

void derive_kparams(const meso_params &p, int dim, meso::KParams &k);

// Context helpers shared with the batch and server front ends (capi.cpp).
int ctx_read_status(meso_ctx *c);    // device status -> c->h_status (syncs the context's stream)
int ctx_residual_check(meso_ctx *c); // residual + convergence counter of do_step
int ctx_read_resid(meso_ctx *c);     // FP32: the device residual state -> host fields
void batch_forget(meso_batch *b, meso_ctx *c);  // batch.cpp
bool tuned_shape(int ncell, int nface, int nv, int &tile_cells, int &vpl, int &ngroup);  // autotune.cpp

}  // namespace meso_host

struct meso_ctx {
    meso_params params{};
    std::unique_ptr<meso_case> kase;  // set for contexts made from a case file
    int dim = 2, C = 0, F = 0, NV = 0, nb = 0;
    meso_host::Renumbering rn;
    std::vector<meso_mark_desc> marks;
    std::vector<uint8_t> mask;
    std::vector<double> vol;  // original order, for residuals
    double min_cell_size = 0, total_volume = 0, dvs_max_mag = 0;

    // device
    int device = 0, num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    meso_host::DevArena arena;
    meso::DMesh dm{};
    meso::DStatus *d_status = nullptr;
    meso::DStatus *h_status = nullptr;  // pinned mirror
    double *h_mac = nullptr;            // pinned staging of the macros: rho [C], u [3C], T [C], q [3C]
    double *d_mac = nullptr;            // the same on the device, in original cell order (gather_macros)
    int *d_new2old = nullptr;           // renumbered -> original cell index
    meso::PlainState ps{};
    meso::F32Inst f32{};               // FP32 instance (device pointers), when precision == MESO_FP32
    meso::Fp32State fs{};              // its single-instance launch state
    std::vector<void *> fs_owned;
    meso_host::TilePlan plan;

    // host step state (the reference's step / solution_time / run_state / converge_state)
    int step = 0;
    double solution_time = 0.0;
    int run_state = 0;
    int converged = 0;
    int converge_state = 0;
    bool initialized = false;
    std::vector<double> rho_res, u_res, T_res, q_res;
    double last_res[8] = {0};
    int nres = 0;
    double last_ms = 0.0;
    int64_t last_launches = 0;
    std::time_t case_mtime = 0;
    int f32_version = 0;  // bumped when the FP32 instance's settings change on the device
    cudaGraphExec_t f32_graph = nullptr;  // the FP32 step's launches, captured once
    meso::StepFork f32_fork;              // side stream and events of the captured step's branch
    int f32_graph_version = -1;
    int64_t f32_graph_launches = 0;
    cudaGraphExec_t plain_graph = nullptr;  // the FP64 step's launches, captured for these kp
    meso::KParams plain_graph_kp{};
    int64_t plain_graph_launches = 0;
    meso_batch *batch = nullptr;  // the batch this context is a member of, if any
    // FP32 defect correction (meso_fp32_refine): every refine_interval steps one FP64 step from the
    // same state (ps, with its own buffers) measures the FP32 step's error
    int refine_interval = 0;
    meso::PlainState ps64{};      // the FP64 step's own buffers (ps aliases the FP32 instance's macros)
    meso::DStatus *d_status_save = nullptr;
    float2 *corrS_mem = nullptr;  // the corrections' device arrays, kept while the correction is off
    double *corrW_mem = nullptr, *corrq_mem = nullptr;
    float2 *corrR_mem = nullptr;
};
