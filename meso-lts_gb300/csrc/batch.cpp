// Batched FP32 Shakhov solves (include/meso_gpu.h, meso_batch_*).
//
// A batch steps many FP32 contexts with one set of launches: the phase
// kernels take an instance array and a work list of (instance, tile, velocity
// group) items, so solves of different mesh and velocity-set sizes share every
// launch.  The launches of one step are captured once as a CUDA graph and
// replayed; the graph needs no per-step arguments because each instance picks
// its current state buffer from its own device step counter.
//
// Each member keeps the reference's per-solve bookkeeping (step, solution
// time, residual every residual_interval of its own steps, the 10-check
// convergence counter, cdugks_shakhov.cpp:724-764).  The check runs on the
// device after each step (k32_residual); a member that converges is halted
// there at once and leaves the work list at the next call.
#include <algorithm>
#include <climits>
#include <cstring>
#include <string>
#include <vector>

#include "capi_internal.h"
#include "host/fp32_host.h"

using meso_host::fail;

struct meso_batch {
    std::vector<meso_ctx *> members;
    std::vector<int> version;   // members' f32_version at the last upload
    std::vector<char> active;   // member is in the current work list
    meso::Fp32State fs{};
    std::vector<void *> owned;
    int device = 0, num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    meso::StepFork fork;  // side stream and events of the captured step's branch
    int launches_per_step = 0;
    double last_ms = 0.0;
    int64_t last_launches = 0;
    bool use_graph = true;
};

namespace {

void drop_graph(meso_batch *b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

bool running(const meso_ctx *c) { return c->run_state != 0; }

// Work list over the running members; the step graph is recaptured.
int rebuild(meso_batch *b) {
    drop_graph(b);
    meso_host::free_fp32_launch(b->fs, b->owned);
    std::vector<meso::F32Inst> insts;
    for (size_t i = 0; i < b->members.size(); ++i) {
        meso_ctx *c = b->members[i];
        b->active[i] = running(c) ? 1 : 0;
        b->version[i] = c->f32_version;
        if (b->active[i]) insts.push_back(c->f32);
    }
    if (insts.empty()) return MESO_OK;
    if (meso_host::build_fp32_launch(insts, b->num_sms, b->fs, b->owned))
        return fail(MESO_ERR_OOM, "batch work-list allocation failed");
    if (!b->use_graph) return MESO_OK;
    int64_t n = 0;
    cudaError_t e = cudaSuccess;
    if (!b->fork.side) {
        e = cudaStreamCreateWithFlags(&b->fork.side, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork.fork, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork.join, cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        const int rc = meso::fp32_step(b->fs, b->stream, &n, nullptr, &b->fork);
        e = cudaStreamEndCapture(b->stream, &b->graph);
        if (rc == 0 && e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
    }
    if (e != cudaSuccess || !b->exec) {  // launch the kernels directly instead
        cudaGetLastError();
        drop_graph(b);
        b->use_graph = false;
    }
    b->launches_per_step = (int)n;
    return MESO_OK;
}

int launch(meso_batch *b) {
    if (b->exec) {
        if (cudaGraphLaunch(b->exec, b->stream) != cudaSuccess)
            return fail(MESO_ERR_CUDA, std::string("graph launch: ") + cudaGetErrorString(cudaGetLastError()));
        b->last_launches += b->launches_per_step;
        return MESO_OK;
    }
    if (meso::fp32_step(b->fs, b->stream, &b->last_launches))
        return fail(MESO_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(cudaGetLastError()));
    return MESO_OK;
}

// Members whose run state or parameters changed since the last upload: rebuild the work list.
int refresh(meso_batch *b) {
    bool stale = false;
    for (size_t i = 0; i < b->members.size(); ++i) {
        meso_ctx *c = b->members[i];
        if (!c) continue;
        cudaStreamSynchronize(c->stream);
        stale = stale || b->active[i] != (running(c) ? 1 : 0) || b->version[i] != c->f32_version;
    }
    return stale ? rebuild(b) : MESO_OK;
}

// After the steps of one call: the members' step, solution time, run state and residuals.
int finish(meso_batch *b, const std::vector<int> &start, int32_t *nrunning) {
    if (cudaStreamSynchronize(b->stream) != cudaSuccess)
        return fail(MESO_ERR_CUDA, std::string("batch step: ") + cudaGetErrorString(cudaGetLastError()));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, b->ev0, b->ev1);
    b->last_ms = ms;
    int still = 0;
    for (size_t i = 0; i < b->members.size(); ++i) {
        meso_ctx *c = b->members[i];
        if (!c || !b->active[i]) continue;
        int rc = meso_host::ctx_read_status(c);
        if (rc) return rc;
        const int done = c->h_status->step - start[i];
        for (int k = 0; k < done; ++k) c->solution_time += c->params.dt;  // as do_step accumulates it
        c->step = c->h_status->step;
        if ((rc = meso_host::ctx_read_resid(c))) return rc;
        if (c->h_status->stop_step != INT_MAX || c->h_status->timeout) c->run_state = 0;
        still += running(c) ? 1 : 0;
    }
    if (nrunning) *nrunning = still;
    return MESO_OK;
}

}  // namespace

extern "C" {

int meso_batch_create(meso_ctx *const *ctxs, int32_t n, meso_batch **out) {
    if (!out) return fail(MESO_ERR_INVALID, "null output handle");
    *out = nullptr;
    if (!ctxs || n <= 0) return fail(MESO_ERR_INVALID, "a batch needs at least one context");
    std::vector<meso_ctx *> m(ctxs, ctxs + n);
    for (int i = 0; i < n; ++i) {
        meso_ctx *c = m[i];
        if (!c) return fail(MESO_ERR_INVALID, "null context in the batch");
        if (c->params.precision != MESO_FP32)
            return fail(MESO_ERR_UNSUPPORTED, "batches step FP32 contexts only");
        if (!c->initialized) return fail(MESO_ERR_INVALID, "batch member " + std::to_string(i) + " is not initialised");
        if (c->batch) return fail(MESO_ERR_INVALID, "context is already in a batch");
        if (c->f32.corrS)
            return fail(MESO_ERR_UNSUPPORTED, "a context with defect correction (meso_fp32_refine) steps alone");
        if (c->device != m[0]->device) return fail(MESO_ERR_INVALID, "batch members must share a device");
        for (int j = 0; j < i; ++j)
            if (m[j] == c) return fail(MESO_ERR_INVALID, "context listed twice");
    }
    if (cudaSetDevice(m[0]->device) != cudaSuccess) return fail(MESO_ERR_CUDA, "cannot select the batch's device");
    auto *b = new meso_batch();
    b->members = m;
    b->version.assign(n, -1);
    b->active.assign(n, 0);
    b->device = m[0]->device;
    b->num_sms = m[0]->num_sms;
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess) {
        delete b;
        return fail(MESO_ERR_CUDA, "cannot create the batch stream");
    }
    for (meso_ctx *c : m) cudaStreamSynchronize(c->stream);
    int rc = rebuild(b);
    if (rc) {
        meso_batch_destroy(b);
        return rc;
    }
    for (meso_ctx *c : m) c->batch = b;
    *out = b;
    return MESO_OK;
}

void meso_batch_destroy(meso_batch *b) {
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    drop_graph(b);
    meso_host::free_fp32_launch(b->fs, b->owned);
    for (meso_ctx *c : b->members)
        if (c && c->batch == b) c->batch = nullptr;
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->fork.side) cudaStreamDestroy(b->fork.side);
    if (b->fork.fork) cudaEventDestroy(b->fork.fork);
    if (b->fork.join) cudaEventDestroy(b->fork.join);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

int meso_batch_step(meso_batch *b, int32_t nsteps, int32_t *nrunning) {
    if (!b) return fail(MESO_ERR_INVALID, "null batch");
    if (nsteps < 0) return fail(MESO_ERR_INVALID, "nsteps must be >= 0");
    if (cudaSetDevice(b->device) != cudaSuccess) return fail(MESO_ERR_CUDA, "cannot select the batch's device");
    const int n = (int)b->members.size();
    int rc = refresh(b);
    if (rc) return rc;
    std::vector<int> start(n);
    for (int i = 0; i < n; ++i) start[i] = b->members[i] ? b->members[i]->step : 0;
    b->last_launches = 0;
    cudaEventRecord(b->ev0, b->stream);
    int nact = 0;
    for (int i = 0; i < n; ++i) nact += b->active[i] && running(b->members[i]);
    // The residual check and the convergence counter run on the device (k32_residual), so the
    // steps go out back to back; a member that converges or fails is halted there and its kernels
    // skip it from the next step on.
    for (int it = 0; it < nsteps && nact > 0; ++it)
        if ((rc = launch(b))) return rc;
    cudaEventRecord(b->ev1, b->stream);
    return finish(b, start, nrunning);
}

int meso_batch_phase_times(meso_batch *b, int32_t nsteps, double *ms, int32_t max_phases, int32_t *nphases) {
    if (!b) return fail(MESO_ERR_INVALID, "null batch");
    if (nsteps <= 0 || !ms) return fail(MESO_ERR_INVALID, "nsteps must be > 0 and ms non-null");
    if (cudaSetDevice(b->device) != cudaSuccess) return fail(MESO_ERR_CUDA, "cannot select the batch's device");
    int rc = refresh(b);
    if (rc) return rc;
    const int np = meso::F32_NPHASE;
    if (nphases) *nphases = np;
    const int n = (int)b->members.size();
    std::vector<int> start(n);
    for (int i = 0; i < n; ++i) start[i] = b->members[i] ? b->members[i]->step : 0;
    std::vector<cudaEvent_t> ev((size_t)np + 1);
    for (auto &e : ev)
        if (cudaEventCreate(&e) != cudaSuccess) return fail(MESO_ERR_CUDA, "cannot create the phase events");
    std::vector<double> acc(np, 0.0);
    b->last_launches = 0;
    int nact = 0;
    for (int i = 0; i < n; ++i) nact += b->active[i] && running(b->members[i]);
    cudaEventRecord(b->ev0, b->stream);
    for (int s = 0; s < nsteps && nact > 0 && rc == MESO_OK; ++s) {
        if (meso::fp32_step(b->fs, b->stream, &b->last_launches, ev.data()) ||
            cudaEventSynchronize(ev[np]) != cudaSuccess) {
            rc = fail(MESO_ERR_CUDA, std::string("batch phase timing: ") + cudaGetErrorString(cudaGetLastError()));
            break;
        }
        for (int k = 0; k < np; ++k) {
            float t = 0.f;
            cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
            acc[k] += t;
        }
    }
    cudaEventRecord(b->ev1, b->stream);
    for (auto &e : ev) cudaEventDestroy(e);
    if (rc) return rc;
    for (int k = 0; k < np && k < max_phases; ++k) ms[k] = acc[k] / nsteps;
    return finish(b, start, nullptr);
}

double meso_batch_last_step_ms(meso_batch *b) { return b ? b->last_ms : 0.0; }

int64_t meso_batch_last_step_launches(meso_batch *b) { return b ? b->last_launches : 0; }

int32_t meso_batch_size(meso_batch *b) { return b ? (int32_t)b->members.size() : 0; }

}  // extern "C"

namespace meso_host {
// A member context is going away: it leaves its batch (which rebuilds at its next step).
void batch_forget(meso_batch *b, meso_ctx *c) {
    if (!b) return;
    cudaStreamSynchronize(b->stream);
    for (size_t i = 0; i < b->members.size(); ++i)
        if (b->members[i] == c) {
            b->members.erase(b->members.begin() + (long)i);
            b->version.erase(b->version.begin() + (long)i);
            b->active.erase(b->active.begin() + (long)i);
            break;
        }
    rebuild(b);
}
}  // namespace meso_host
