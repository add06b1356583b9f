// Served solves with continuous batching (include/meso_gpu.h, meso_server_*).
//
// Requests are case files.  A request is admitted when the device has room
// for it (an HBM budget and the free memory the runtime reports) and a member
// slot is free; admitted solves keep their state resident on the device and
// are stepped together by one batch (one set of launches per step, batch.cpp),
// so requests that arrive while others run overlap with them on the GPU.  A
// solve leaves the batch when it converges, fails (unmasked NaN / T < 0) or
// reaches the case's max-step; its macros are copied out, its device memory is
// freed, and the next pending requests take its place.
//
// The per-solve loop is the reference's handle_solver loop
// (src/meso/exec.cpp:141-165: do_step until run_state turns false or step
// reaches max_step), run for many solves at once.  No counterpart in the
// reference, which serves one solve per process.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <deque>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "capi_internal.h"

using meso_host::fail;
using Clock = std::chrono::steady_clock;

namespace {

enum class ReqState { pending, running, done };

struct Request {
    int64_t tag = 0;
    meso_case *kase = nullptr;
    meso_params params{};
    int32_t max_step = 0;
    size_t est_bytes = 0;
    meso_ctx *ctx = nullptr;
    ReqState state = ReqState::pending;
    Clock::time_point t_submit, t_admit, t_done;
    // results, original cell order
    std::vector<double> rho, u, T, q;
    meso_status status{};
    ~Request() {
        if (ctx) meso_ctx_destroy(ctx);
        if (kase) meso_case_free(kase);
    }
};

// Device bytes of an FP32 solve: two state buffers, the stored face values, boundary face buffers,
// per-face and per-cell work arrays and the geometry tables.
size_t estimate_bytes(const meso_mesh_desc &m, const meso_dvs_desc &d) {
    const size_t NVp = ((size_t)d.nv + 63) / 64 * 64;
    const size_t C = m.ncell, F = m.nface;
    const size_t nb = 4 * (size_t)std::sqrt((double)C) + 64;  // boundary faces of a 2-D domain, with margin
    const size_t state = 2 * C * NVp * 8;
    const size_t faces = F * NVp * 8;  // stored face reconstructions
    const size_t bnd = 2 * nb * NVp * 8;
    const size_t work = F * (8 * 11 * 4 + 200) + C * 400;  // face partials (up to 4 groups), tables
    return state + faces + bnd + work + ((size_t)16 << 20);
}

}  // namespace

struct meso_server {
    int device = 0;
    int64_t budget = 0;
    int32_t max_members = 0;
    int64_t next_tag = 1;
    std::deque<std::unique_ptr<Request>> pending;
    std::vector<std::unique_ptr<Request>> running;
    std::map<int64_t, std::unique_ptr<Request>> done;
    meso_batch *batch = nullptr;
    bool dirty = true;
    int64_t used = 0;
    double last_ms = 0.0;
    int64_t steps_issued = 0;
    double gpu_ms = 0.0, poll_ms = 0.0;  // device time of the batch steps / wall time inside polls
};

namespace {

int admit(meso_server *s) {
    while (!s->pending.empty() && (int)s->running.size() < s->max_members) {
        Request *r = s->pending.front().get();
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return fail(MESO_ERR_CUDA, "cudaMemGetInfo failed");
        const size_t margin = (size_t)1 << 30;
        if (s->used + (int64_t)r->est_bytes > s->budget || r->est_bytes + margin > free_b) break;
        meso_mesh_desc m;
        meso_dvs_desc d;
        const meso_mark_desc *marks = nullptr;
        int32_t nmarks = 0;
        meso_case_mesh(r->kase, &m);
        meso_case_dvs(r->kase, &d);
        meso_case_marks(r->kase, &marks, &nmarks);
        std::vector<double> rho(m.ncell), u(3 * (size_t)m.ncell), T(m.ncell);
        std::vector<uint8_t> mask(m.ncell);
        int rc = meso_case_initial_fields(r->kase, rho.data(), u.data(), T.data(), mask.data());
        if (rc) return rc;
        meso_ctx *c = nullptr;
        rc = meso_ctx_create(&m, &d, marks, nmarks, &r->params, mask.data(), &c);
        if (rc == MESO_ERR_OOM) break;  // retry when a running solve has left
        if (rc) return rc;
        rc = meso_init_macros(c, rho.data(), u.data(), T.data(), nullptr, 0);
        if (rc) {
            meso_ctx_destroy(c);
            return rc;
        }
        r->ctx = c;
        r->state = ReqState::running;
        r->t_admit = Clock::now();
        s->used += (int64_t)meso_ctx_device_bytes(c);
        s->running.push_back(std::move(s->pending.front()));
        s->pending.pop_front();
        s->dirty = true;
    }
    return MESO_OK;
}

int retire(meso_server *s, std::vector<int64_t> &finished) {
    for (size_t i = 0; i < s->running.size();) {
        Request *r = s->running[i].get();
        meso_status st;
        int rc = meso_get_status(r->ctx, &st);
        if (rc) return rc;
        const bool over = r->max_step > 0 && st.step >= r->max_step;
        if (st.run_state && !over) {
            ++i;
            continue;
        }
        if (s->batch) {  // membership changes: the batch is rebuilt at the next poll
            meso_batch_destroy(s->batch);
            s->batch = nullptr;
        }
        const int C = r->ctx->C;
        r->rho.resize(C);
        r->u.resize(3 * (size_t)C);
        r->T.resize(C);
        r->q.resize(3 * (size_t)C);
        if ((rc = meso_get_macros(r->ctx, r->rho.data(), r->u.data(), r->T.data(), r->q.data()))) return rc;
        r->status = st;
        s->used -= (int64_t)meso_ctx_device_bytes(r->ctx);
        meso_ctx_destroy(r->ctx);  // leaves the batch
        r->ctx = nullptr;
        meso_case_free(r->kase);
        r->kase = nullptr;
        r->state = ReqState::done;
        r->t_done = Clock::now();
        finished.push_back(r->tag);
        s->done[r->tag] = std::move(s->running[i]);
        s->running.erase(s->running.begin() + (long)i);
        s->dirty = true;
    }
    return MESO_OK;
}

}  // namespace

extern "C" {

int meso_server_create(int64_t hbm_budget_bytes, int32_t max_members, meso_server **out) {
    if (!out) return fail(MESO_ERR_INVALID, "null output handle");
    *out = nullptr;
    if (hbm_budget_bytes <= 0 || max_members <= 0) return fail(MESO_ERR_INVALID, "budget and member count must be > 0");
    auto *s = new meso_server();
    if (cudaGetDevice(&s->device) != cudaSuccess) {
        delete s;
        return fail(MESO_ERR_CUDA, "no CUDA device");
    }
    s->budget = hbm_budget_bytes;
    s->max_members = max_members;
    *out = s;
    return MESO_OK;
}

void meso_server_destroy(meso_server *s) {
    if (!s) return;
    cudaSetDevice(s->device);
    if (s->batch) meso_batch_destroy(s->batch);
    s->running.clear();
    s->pending.clear();
    s->done.clear();
    delete s;
}

int meso_server_submit(meso_server *s, const char *case_file, const meso_params *params, int64_t *tag) {
    if (!s || !case_file) return fail(MESO_ERR_INVALID, "null argument");
    auto r = std::make_unique<Request>();
    int rc = meso_case_load(case_file, &r->kase);
    if (rc) return rc;
    meso_params p;
    meso_case_params(r->kase, &p);
    if (params) p = *params;
    p.precision = MESO_FP32;
    if (p.solver != MESO_SOLVER_CDUGKS_SHAKHOV) return fail(MESO_ERR_UNSUPPORTED, "served solves are FP32 Shakhov solves");
    // One velocity group per tile unless the request sets a shape: the batch of running solves
    // supplies the parallelism, and whole-velocity-range items carry the least per-item overhead.
    if (p.tile_cells == 0 && p.vpl == 0 && p.ngroup == 0) p.ngroup = 1;
    r->params = p;
    int32_t ws = 0, rnp = 0, ol = 0, onp = 0;
    meso_case_loop_settings(r->kase, &r->max_step, &ws, &rnp, &ol, &onp);
    meso_mesh_desc m;
    meso_dvs_desc d;
    meso_case_mesh(r->kase, &m);
    meso_case_dvs(r->kase, &d);
    r->est_bytes = estimate_bytes(m, d);
    if ((int64_t)r->est_bytes > s->budget) return fail(MESO_ERR_CAPACITY, "request larger than the server's HBM budget");
    r->tag = s->next_tag++;
    r->t_submit = Clock::now();
    if (tag) *tag = r->tag;
    s->pending.push_back(std::move(r));
    return MESO_OK;
}

int meso_server_poll(meso_server *s, int32_t nsteps, int64_t *done_tags, int32_t max_done, int32_t *ndone) {
    if (!s) return fail(MESO_ERR_INVALID, "null server");
    if (ndone) *ndone = 0;
    const auto t0 = Clock::now();
    struct PollTimer {  // wall time of the poll, whichever way it returns
        meso_server *s;
        Clock::time_point t0;
        ~PollTimer() { s->poll_ms += std::chrono::duration<double, std::milli>(Clock::now() - t0).count(); }
    } timer{s, t0};
    if (cudaSetDevice(s->device) != cudaSuccess) return fail(MESO_ERR_CUDA, "cannot select the server's device");
    std::vector<int64_t> finished;
    int rc = retire(s, finished);  // solves that ended in the previous poll
    if (rc) return rc;
    if ((rc = admit(s))) return rc;
    if (s->dirty) {
        if (s->batch) meso_batch_destroy(s->batch);
        s->batch = nullptr;
        if (!s->running.empty()) {
            std::vector<meso_ctx *> m;
            for (auto &r : s->running) m.push_back(r->ctx);
            if ((rc = meso_batch_create(m.data(), (int32_t)m.size(), &s->batch))) return rc;
        }
        s->dirty = false;
    }
    s->last_ms = 0.0;
    if (s->batch && nsteps > 0) {
        // do not step a solve past its max_step: the batch stops at the nearest one
        int32_t n = nsteps;
        for (auto &r : s->running)
            if (r->max_step > 0) n = std::min<int32_t>(n, std::max(1, r->max_step - r->ctx->step));
        int32_t nrun = 0;
        if ((rc = meso_batch_step(s->batch, n, &nrun))) return rc;
        s->last_ms = meso_batch_last_step_ms(s->batch);
        s->gpu_ms += s->last_ms;
        s->steps_issued += n;
    }
    if ((rc = retire(s, finished))) return rc;
    const int32_t k = (int32_t)std::min<size_t>(finished.size(), (size_t)std::max(0, max_done));
    for (int32_t i = 0; i < k; ++i)
        if (done_tags) done_tags[i] = finished[i];
    if (ndone) *ndone = k;
    if ((int32_t)finished.size() > k) return fail(MESO_ERR_CAPACITY, "done_tags too small for the finished solves");
    return MESO_OK;
}

int meso_server_counts(meso_server *s, int32_t *npending, int32_t *nrunning, int32_t *ndone) {
    if (!s) return fail(MESO_ERR_INVALID, "null server");
    if (npending) *npending = (int32_t)s->pending.size();
    if (nrunning) *nrunning = (int32_t)s->running.size();
    if (ndone) *ndone = (int32_t)s->done.size();
    return MESO_OK;
}

int meso_server_result(meso_server *s, int64_t tag, double *rho, double *u, double *T, double *q, meso_status *st,
                       double *seconds) {
    if (!s) return fail(MESO_ERR_INVALID, "null server");
    auto it = s->done.find(tag);
    if (it == s->done.end()) return fail(MESO_ERR_INVALID, "no finished request with this tag");
    const Request &r = *it->second;
    if (rho) std::copy(r.rho.begin(), r.rho.end(), rho);
    if (u) std::copy(r.u.begin(), r.u.end(), u);
    if (T) std::copy(r.T.begin(), r.T.end(), T);
    if (q) std::copy(r.q.begin(), r.q.end(), q);
    if (st) *st = r.status;
    if (seconds) {
        seconds[0] = std::chrono::duration<double>(r.t_done - r.t_submit).count();  // submit -> finished
        seconds[1] = std::chrono::duration<double>(r.t_admit - r.t_submit).count(); // queueing
    }
    return MESO_OK;
}

int meso_server_release(meso_server *s, int64_t tag) {
    if (!s) return fail(MESO_ERR_INVALID, "null server");
    s->done.erase(tag);
    return MESO_OK;
}

int64_t meso_server_device_bytes(meso_server *s) { return s ? s->used : 0; }

int meso_server_stats(meso_server *s, double *gpu_ms, double *poll_ms, int64_t *batch_steps) {
    if (!s) return fail(MESO_ERR_INVALID, "null server");
    if (gpu_ms) *gpu_ms = s->gpu_ms;
    if (poll_ms) *poll_ms = s->poll_ms;
    if (batch_steps) *batch_steps = s->steps_issued;
    return MESO_OK;
}

}  // extern "C"
