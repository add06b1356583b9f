// C ABI of the step library (include/meso_gpu.h): context lifecycle, upload,
// the do_step loop with the reference's residual / convergence logic, and the
// read-back of macroscopic fields in the original cell order.
//
// Reference correspondence (meso-lts):
//   step loop              src/meso/exec.cpp:141-165
//   do_step bookkeeping    cdugks_shakhov.cpp:724-764, cdugks.cpp:337-371, dugks.cpp:346-383
//   residual               src/solver/field.cpp:223-249, src/core/core.cpp:45-51
//   derived constants      cdugks.cpp:41-47, 171, 306-308; dugks.cpp:41-48, 300, 331;
//                          cdugks_shakhov.cpp:29-32
#include "capi_internal.h"

#include <sys/stat.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <fstream>
#include <sstream>

#include "host/fp32_host.h"
#include "host/output.h"

namespace meso_host {

namespace {
thread_local std::string g_error;
}

const char *last_error_cstr() { return g_error.c_str(); }

void set_error(const std::string &msg) { g_error = msg; }
int fail(int code, const std::string &msg) {
    g_error = msg;
    return code;
}

void DevArena::release() {
    for (void *p : ptrs) cudaFree(p);
    ptrs.clear();
    bytes = 0;
    cur = nullptr;
    left = 0;
}

void derive_kparams(const meso_params &p, int dim, meso::KParams &k) {
    std::memset(&k, 0, sizeof(k));
    k.dt = p.dt;
    k.hdt = p.dt * 0.5;
    k.R = p.R;
    k.T0 = p.T0;
    k.Kd = (double)p.K;
    k.Dd = (double)dim;
    k.Pr = p.Pr;
    k.mu0 = p.mu0;
    k.vhs = p.vhs_index;
    k.gamma = (p.K + 5.0) / (p.K + 3.0);
    k.Cv = (p.K + 3.0) * p.R * 0.5;
    k.venkata_k = p.venkata_k;
    k.gradient = p.gradient_switch;
    k.limiter = p.limiter_switch;
    if (p.solver != MESO_SOLVER_CDUGKS_SHAKHOV) {
        k.RT = p.R * p.T0;
        k.over_RT = 1.0 / k.RT;
        double c_sound = std::sqrt(k.RT);
        k.tau = (p.L0 * p.Ma) / (p.Re * c_sound);
        k.hdt = 0.5 * p.dt;
        k.cm = k.hdt / (k.hdt - 2.0 * k.tau);
        k.Cc = k.tau / (k.tau + k.hdt);
        k.c_eq = k.hdt / (2.0 * k.tau);
        k.c_eq_face = k.hdt / (2.0 * k.tau + k.hdt);
        k.C_bp_to_t = (p.dt + k.hdt) / (k.hdt - 2.0 * k.tau);
        k.C_t_to_bp = (p.dt + k.hdt) / (2.0 * k.tau + p.dt);
    }
}

}  // namespace meso_host

using namespace meso_host;

namespace {

#define CUDA_TRY(expr)                                                                   \
    do {                                                                                 \
        cudaError_t e_ = (expr);                                                         \
        if (e_ != cudaSuccess)                                                           \
            return fail(MESO_ERR_CUDA, std::string(#expr ": ") + cudaGetErrorString(e_)); \
    } while (0)

bool valid_params(const meso_params &p, std::string &why) {
    if (p.solver < 0 || p.solver > 2) { why = "unknown solver kind"; return false; }
    if (p.precision != MESO_FP64 && p.precision != MESO_FP32) { why = "unknown precision"; return false; }
    if (!(p.dt > 0.0) || !std::isfinite(p.dt)) { why = "timeStep must be positive"; return false; }
    if (p.residual_interval < 0) { why = "residual_interval must be >= 0"; return false; }
    return true;
}

template <class T> void upload(T *dst, const std::vector<T> &src, cudaStream_t s) {
    if (!src.empty()) cudaMemcpyAsync(dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice, s);
}

int check_desc(const meso_mesh_desc *m, const meso_dvs_desc *d, const meso_mark_desc *marks, int nmarks) {
    if (!m || !d) return fail(MESO_ERR_INVALID, "null mesh or DVS descriptor");
    if (m->dim != 2 && m->dim != 3) return fail(MESO_ERR_INVALID, "mesh dim must be 2 or 3");
    if (m->ncell <= 0 || m->nface <= 0) return fail(MESO_ERR_INVALID, "empty mesh");
    if (d->nv <= 0 || !d->xi || !d->w) return fail(MESO_ERR_INVALID, "empty DVS");
    if (!m->cell_pos || !m->cell_vol || !m->cell_face_ptr || !m->cell_face || !m->cell_nbr_ptr ||
        !m->lsq_c || !m->face_cell || !m->face_pos || !m->face_area || !m->face_normal || !m->face_mark)
        return fail(MESO_ERR_INVALID, "mesh descriptor has a null table");
    if (nmarks <= 0 || !marks) return fail(MESO_ERR_INVALID, "mark table is empty");
    for (int c = 0; c < m->ncell; ++c) {
        if (m->cell_face_ptr[c + 1] < m->cell_face_ptr[c] || m->cell_nbr_ptr[c + 1] < m->cell_nbr_ptr[c])
            return fail(MESO_ERR_INVALID, "CSR pointers must be non-decreasing");
        if (!(m->cell_vol[c] > 0.0)) return fail(MESO_ERR_INVALID, "cell volume must be positive");
    }
    const int nf = m->cell_face_ptr[m->ncell], nn = m->cell_nbr_ptr[m->ncell];
    for (int j = 0; j < nf; ++j)
        if (m->cell_face[j] < 0 || m->cell_face[j] >= m->nface) return fail(MESO_ERR_INVALID, "cell_face out of range");
    for (int j = 0; j < nn; ++j)
        if (m->cell_nbr[j] < 0 || m->cell_nbr[j] >= m->ncell) return fail(MESO_ERR_INVALID, "cell_nbr out of range");
    if (nn > 0 && (!m->lsq_w || !m->lsq_dr)) return fail(MESO_ERR_INVALID, "least-squares tables missing");
    for (int f = 0; f < m->nface; ++f) {
        for (int s = 0; s < 2; ++s)
            if (m->face_cell[2 * f + s] < 0 || m->face_cell[2 * f + s] >= m->ncell)
                return fail(MESO_ERR_INVALID, "face_cell out of range");
        if (m->face_mark[f] < 0 || m->face_mark[f] >= nmarks) return fail(MESO_ERR_INVALID, "face_mark out of range");
    }
    for (int i = 0; i < nmarks; ++i)
        if (marks[i].type < 0 || marks[i].type > MESO_BC_SYMMETRY) return fail(MESO_ERR_INVALID, "bad mark type");
    if (d->sym)
        for (int p = 0; p < 3 * d->nv; ++p)
            if (d->sym[p] < 0 || d->sym[p] >= d->nv) return fail(MESO_ERR_INVALID, "DVS symmetry index out of range");
    for (int i = 0; i < nmarks; ++i)
        if ((marks[i].type == MESO_BC_SYMMETRY || marks[i].type == MESO_BC_SLIP_WALL) &&
            (marks[i].direction < 0 || marks[i].direction > 2))
            return fail(MESO_ERR_INVALID, "symmetry direction must be 0, 1 or 2");
    return MESO_OK;
}

// Host macro arrays in renumbered order <-> original order.
void to_orig(const meso_ctx *c, const std::vector<double> &dev, double *out, int ncomp) {
    for (int i = 0; i < c->C; ++i) {
        int o = c->rn.cell_new2old[i];
        for (int k = 0; k < ncomp; ++k) out[(size_t)o * ncomp + k] = dev[(size_t)i * ncomp + k];
    }
}
void to_new(const meso_ctx *c, const double *in, std::vector<double> &dev, int ncomp) {
    dev.resize((size_t)c->C * ncomp);
    for (int i = 0; i < c->C; ++i) {
        int o = c->rn.cell_new2old[i];
        for (int k = 0; k < ncomp; ++k) dev[(size_t)i * ncomp + k] = in[(size_t)o * ncomp + k];
    }
}

int build_device(meso_ctx *c, const meso_mesh_desc *m, const meso_dvs_desc *d) {
    CUDA_TRY(cudaGetDevice(&c->device));
    CUDA_TRY(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device));
    CUDA_TRY(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    CUDA_TRY(cudaEventCreate(&c->ev0));
    CUDA_TRY(cudaEventCreate(&c->ev1));
    CUDA_TRY(cudaMallocHost(&c->h_status, sizeof(meso::DStatus)));
    const int C = m->ncell, F = m->nface, NV = d->nv, D = m->dim;
    CUDA_TRY(cudaMallocHost(&c->h_mac, sizeof(double) * 8 * (size_t)C));
    const auto &rn = c->rn;
    c->d_mac = c->arena.alloc<double>(8 * (size_t)C);
    c->d_new2old = c->arena.alloc<int>(C);
    CUDA_TRY(cudaMemcpyAsync(c->d_new2old, rn.cell_new2old.data(), sizeof(int) * (size_t)C, cudaMemcpyHostToDevice,
                             c->stream));
    // ---- renumbered host tables
    std::vector<double> vol(C), cpos(3 * C), lsq_c(9 * C), lsq_w, lsq_dr, farea(F), fpos(3 * F), fn(3 * F);
    std::vector<int> cf_ptr(1, 0), cf_face, cn_ptr(1, 0), cn_cell, fown(F), fnei(F), fmark(F), bface;
    std::vector<uint8_t> mask(C, 0);
    for (int i = 0; i < C; ++i) {
        int o = rn.cell_new2old[i];
        vol[i] = m->cell_vol[o];
        for (int k = 0; k < 3; ++k) cpos[3 * i + k] = m->cell_pos[3 * o + k];
        for (int k = 0; k < 9; ++k) lsq_c[9 * i + k] = m->lsq_c[9 * o + k];
        for (int j = m->cell_face_ptr[o]; j < m->cell_face_ptr[o + 1]; ++j) cf_face.push_back(rn.face_old2new[m->cell_face[j]]);
        cf_ptr.push_back((int)cf_face.size());
        for (int j = m->cell_nbr_ptr[o]; j < m->cell_nbr_ptr[o + 1]; ++j) {
            cn_cell.push_back(rn.cell_old2new[m->cell_nbr[j]]);
            lsq_w.push_back(m->lsq_w[j]);
            for (int k = 0; k < 3; ++k) lsq_dr.push_back(m->lsq_dr[3 * j + k]);
        }
        cn_ptr.push_back((int)cn_cell.size());
        if (!c->mask.empty()) mask[i] = c->mask[o];
    }
    for (int f = 0; f < F; ++f) {
        int o = rn.face_new2old[f];
        fown[f] = rn.cell_old2new[m->face_cell[2 * o]];
        fnei[f] = rn.cell_old2new[m->face_cell[2 * o + 1]];
        farea[f] = m->face_area[o];
        for (int k = 0; k < 3; ++k) {
            fpos[3 * f + k] = m->face_pos[3 * o + k];
            fn[3 * f + k] = m->face_normal[3 * o + k];
        }
        fmark[f] = m->face_mark[o];
        if (c->marks[fmark[f]].type != MESO_BC_FLUID_INTERIOR) bface.push_back(f);
    }
    std::vector<double> xix(NV), xiy(NV), xiz(NV), w(NV);
    std::vector<int> sym(3 * NV, 0);
    for (int p = 0; p < NV; ++p) {
        xix[p] = d->xi[3 * p];
        xiy[p] = d->xi[3 * p + 1];
        xiz[p] = d->xi[3 * p + 2];
        w[p] = d->w[p];
        if (d->sym)
            for (int k = 0; k < 3; ++k) sym[3 * p + k] = d->sym[3 * p + k];
    }
    c->nb = (int)bface.size();
    // tensor-product velocity sets (2-D): every (x, y) of the distinct components present once
    std::vector<double> tX, tY;
    std::vector<int> tix(NV), tiy(NV);
    if (D == 2) {
        tX = xix;
        tY = xiy;
        std::sort(tX.begin(), tX.end());
        tX.erase(std::unique(tX.begin(), tX.end()), tX.end());
        std::sort(tY.begin(), tY.end());
        tY.erase(std::unique(tY.begin(), tY.end()), tY.end());
        bool tensor = tX.size() * tY.size() == (size_t)NV;
        std::vector<char> seen(tensor ? (size_t)NV : 0, 0);
        for (int p = 0; tensor && p < NV; ++p) {
            tix[p] = (int)(std::lower_bound(tX.begin(), tX.end(), xix[p]) - tX.begin());
            tiy[p] = (int)(std::lower_bound(tY.begin(), tY.end(), xiy[p]) - tY.begin());
            char &c2 = seen[(size_t)tiy[p] * tX.size() + tix[p]];
            tensor = !c2;
            c2 = 1;
        }
        if (!tensor) tX.clear(), tY.clear();
    }
    auto &A = c->arena;
    auto &dm = c->dm;
    dm.dim = D;
    dm.C = C;
    dm.F = F;
    dm.NV = NV;
    dm.nb = c->nb;
    try {
        double *p_vol = A.alloc<double>(C), *p_cpos = A.alloc<double>(3 * C), *p_lsqc = A.alloc<double>(9 * C);
        double *p_lw = A.alloc<double>(lsq_w.size()), *p_ldr = A.alloc<double>(lsq_dr.size());
        int *p_cfp = A.alloc<int>(C + 1), *p_cf = A.alloc<int>(cf_face.size()), *p_cnp = A.alloc<int>(C + 1);
        int *p_cn = A.alloc<int>(cn_cell.size());
        int *p_fo = A.alloc<int>(F), *p_fne = A.alloc<int>(F), *p_fm = A.alloc<int>(F), *p_bf = A.alloc<int>(bface.size());
        double *p_fa = A.alloc<double>(F), *p_fp = A.alloc<double>(3 * F), *p_fn = A.alloc<double>(3 * F);
        double *p_x = A.alloc<double>(NV), *p_y = A.alloc<double>(NV), *p_z = A.alloc<double>(NV), *p_w = A.alloc<double>(NV);
        int *p_sym = A.alloc<int>(3 * NV);
        meso_mark_desc *p_marks = A.alloc<meso_mark_desc>(c->marks.size());
        uint8_t *p_mask = A.alloc<uint8_t>(C);
        upload(p_vol, vol, c->stream);
        upload(p_cpos, cpos, c->stream);
        upload(p_lsqc, lsq_c, c->stream);
        upload(p_lw, lsq_w, c->stream);
        upload(p_ldr, lsq_dr, c->stream);
        upload(p_cfp, cf_ptr, c->stream);
        upload(p_cf, cf_face, c->stream);
        upload(p_cnp, cn_ptr, c->stream);
        upload(p_cn, cn_cell, c->stream);
        upload(p_fo, fown, c->stream);
        upload(p_fne, fnei, c->stream);
        upload(p_fm, fmark, c->stream);
        upload(p_bf, bface, c->stream);
        upload(p_fa, farea, c->stream);
        upload(p_fp, fpos, c->stream);
        upload(p_fn, fn, c->stream);
        upload(p_x, xix, c->stream);
        upload(p_y, xiy, c->stream);
        upload(p_z, xiz, c->stream);
        upload(p_w, w, c->stream);
        upload(p_sym, sym, c->stream);
        upload(p_marks, c->marks, c->stream);
        upload(p_mask, mask, c->stream);
        dm.vol = p_vol;
        dm.cpos = p_cpos;
        dm.cf_ptr = p_cfp;
        dm.cf_face = p_cf;
        dm.cn_ptr = p_cnp;
        dm.cn_cell = p_cn;
        dm.lsq_w = p_lw;
        dm.lsq_dr = p_ldr;
        dm.lsq_c = p_lsqc;
        dm.fown = p_fo;
        dm.fnei = p_fne;
        dm.farea = p_fa;
        dm.fpos = p_fp;
        dm.fn = p_fn;
        dm.fmark = p_fm;
        dm.bface = p_bf;
        dm.xix = p_x;
        dm.xiy = p_y;
        dm.xiz = p_z;
        dm.w = p_w;
        dm.sym = p_sym;
        dm.marks = p_marks;
        dm.mask = p_mask;
        if (!tX.empty()) {
            double *p_tx = A.alloc<double>(tX.size()), *p_ty = A.alloc<double>(tY.size());
            int *p_tix = A.alloc<int>(NV), *p_tiy = A.alloc<int>(NV);
            upload(p_tx, tX, c->stream);
            upload(p_ty, tY, c->stream);
            upload(p_tix, tix, c->stream);
            upload(p_tiy, tiy, c->stream);
            dm.ntx = (int)tX.size();
            dm.nty = (int)tY.size();
            dm.tx = p_tx;
            dm.ty = p_ty;
            dm.tix = p_tix;
            dm.tiy = p_tiy;
        }
        c->d_status = A.alloc<meso::DStatus>(1);

        const bool shakhov = c->params.solver == MESO_SOLVER_CDUGKS_SHAKHOV;
        const size_t cv = (size_t)C * NV, fv = (size_t)F * NV, bv = (size_t)std::max(c->nb, 1) * NV;
        if (c->params.precision == MESO_FP32) {
            c->ps.status = c->d_status;
            c->ps.mesh = dm;
            c->ps.solver = c->params.solver;
            c->ps.num_sms = c->num_sms;
            if (meso::fp32_configure(c->device)) return fail(MESO_ERR_CUDA, "FP32 kernel configuration failed");
            int rc = build_fp32_instance(c, m, d, c->plan, c->params.ngroup, c->params.vpl);
            if (rc) return rc;
            return MESO_OK;
        }
        auto &s = c->ps;
        s.solver = c->params.solver;
        s.num_sms = c->num_sms;
        s.mesh = dm;
        s.status = c->d_status;
        s.f0 = A.alloc<double>(cv);
        s.f1 = shakhov ? A.alloc<double>(cv) : nullptr;
        s.face0 = A.alloc<double>(fv);
        s.face1 = shakhov ? A.alloc<double>(fv) : nullptr;
        s.grad0 = A.alloc<double>(cv * D);
        s.grad1 = shakhov ? A.alloc<double>(cv * D) : nullptr;
        s.flux0 = c->params.solver != MESO_SOLVER_DUGKS ? A.alloc<double>(cv) : nullptr;
        s.flux1 = shakhov ? A.alloc<double>(cv) : nullptr;
        s.snap0 = A.alloc<double>(bv);
        s.snap1 = shakhov ? A.alloc<double>(bv) : nullptr;
        s.rho = A.alloc<double>(8 * (size_t)C);  // rho, u, T, q contiguous: one copy to the host
        s.u = s.rho + C;
        s.T = s.rho + 4 * (size_t)C;
        s.q = s.rho + 5 * (size_t)C;
        s.fm0 = A.alloc<double>(C);
        s.fm1 = A.alloc<double>(3 * C);
        s.fm2 = A.alloc<double>(C);
        s.repair_list = A.alloc<int>(C);
        CUDA_TRY(cudaMemsetAsync(s.T, 0, sizeof(double) * C, c->stream));
        CUDA_TRY(cudaMemsetAsync(s.q, 0, sizeof(double) * 3 * C, c->stream));
        CUDA_TRY(cudaMemsetAsync(s.fm0, 0, sizeof(double) * C, c->stream));
        CUDA_TRY(cudaMemsetAsync(s.fm1, 0, sizeof(double) * 3 * C, c->stream));
        CUDA_TRY(cudaMemsetAsync(s.fm2, 0, sizeof(double) * C, c->stream));
    } catch (const std::bad_alloc &) {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        cudaGetLastError();
        return fail(MESO_ERR_OOM, "device allocation failed (" + std::to_string(A.bytes) + " bytes held, " +
                                      std::to_string(fr) + " free)");
    }
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    return MESO_OK;
}

void reset_status(meso_ctx *c) {
    meso::DStatus s{};
    s.step = 0;
    s.stop_step = INT_MAX;
    s.first_bad = INT_MAX;
    std::memcpy(c->h_status, &s, sizeof(s));
    cudaMemcpyAsync(c->d_status, c->h_status, sizeof(s), cudaMemcpyHostToDevice, c->stream);
    cudaStreamSynchronize(c->stream);
}

int read_status(meso_ctx *c) {
    CUDA_TRY(cudaMemcpyAsync(c->h_status, c->d_status, sizeof(meso::DStatus), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    return MESO_OK;
}

// The macros in original cell order into the given host arrays (any may be null): one copy of the
// contiguous device block into pinned staging, then the permutation.
int fetch_macros(meso_ctx *c, double *rho, double *u, double *T, double *q) {
    const size_t C = (size_t)c->C;
    // permuted to the original cell order on the device, then one copy to the host; straight into
    // the caller's arrays when all of them are page-locked
    if (meso::gather_macros(c->ps.rho, c->ps.u, c->ps.T, c->ps.q, c->d_new2old, c->C, c->d_mac, c->num_sms, c->stream))
        return fail(MESO_ERR_CUDA, "macro gather failed");
    double *const dst[4] = {rho, u, T, q};
    const size_t off[4] = {0, C, 4 * C, 5 * C}, len[4] = {C, 3 * C, C, 3 * C};
    bool direct = true;
    for (double *p : dst) {
        if (!p) continue;
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, p) != cudaSuccess || a.type != cudaMemoryTypeHost) {
            cudaGetLastError();
            direct = false;
        }
    }
    if (direct) {
        for (int k = 0; k < 4; ++k)
            if (dst[k])
                CUDA_TRY(cudaMemcpyAsync(dst[k], c->d_mac + off[k], sizeof(double) * len[k], cudaMemcpyDeviceToHost,
                                         c->stream));
        CUDA_TRY(cudaStreamSynchronize(c->stream));
        return MESO_OK;
    }
    CUDA_TRY(cudaMemcpyAsync(c->h_mac, c->d_mac, sizeof(double) * 8 * C, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    for (int k = 0; k < 4; ++k)
        if (dst[k]) std::memcpy(dst[k], c->h_mac + off[k], sizeof(double) * len[k]);
    return MESO_OK;
}

int download_macros(meso_ctx *c, std::vector<double> &rho, std::vector<double> &u, std::vector<double> &T,
                    std::vector<double> &q) {
    const size_t C = (size_t)c->C;
    rho.resize(C);
    u.resize(3 * C);
    T.resize(C);
    q.resize(3 * C);
    return fetch_macros(c, rho.data(), u.data(), T.data(), q.data());
}

// Solver::residual (field.cpp:223-249): sum |(new-old)/old| V/V_total in cell order; old <- new.
double residual_scalar(const meso_ctx *c, std::vector<double> &old, const std::vector<double> &nw) {
    double r = 0.0;
    for (int i = 0; i < c->C; ++i) r += std::abs((nw[i] - old[i]) / old[i]) * (c->vol[i] / c->total_volume);
    old = nw;
    return r;
}
void residual_vector(const meso_ctx *c, std::vector<double> &old, const std::vector<double> &nw, double out[3]) {
    double rx = 0, ry = 0, rz = 0;
    for (int i = 0; i < c->C; ++i) {
        double vx = std::fabs((nw[3 * i] - old[3 * i]) / old[3 * i]);
        double vy = std::fabs((nw[3 * i + 1] - old[3 * i + 1]) / old[3 * i + 1]);
        double vz = std::fabs((nw[3 * i + 2] - old[3 * i + 2]) / old[3 * i + 2]);
        double s = c->vol[i] / c->total_volume;
        rx += vx * s;
        ry += vy * s;
        rz += vz * s;
    }
    old = nw;
    out[0] = rx;
    out[1] = ry;
    out[2] = rz;
}

// Volume-weighted L2-relative change ||new - old|| / ||old|| of component k of an ncomp field; old <- new
// after the last component.  The convergence measure MESO_RES_L2 selects instead of the reference's
// mean relative change, which divides by values near zero.
double residual_l2(const meso_ctx *c, const std::vector<double> &old, const std::vector<double> &nw, int ncomp, int k) {
    double num = 0.0, den = 0.0;
    for (int i = 0; i < c->C; ++i) {
        const double d = nw[(size_t)ncomp * i + k] - old[(size_t)ncomp * i + k], o = old[(size_t)ncomp * i + k];
        num += c->vol[i] * d * d;
        den += c->vol[i] * o * o;
    }
    return den > 0.0 ? std::sqrt(num / den) : std::sqrt(num);
}

// Residual check of do_step (e.g. cdugks_shakhov.cpp:729-757).
int residual_check(meso_ctx *c) {
    std::vector<double> rho, u, T, q;
    int rc = download_macros(c, rho, u, T, q);
    if (rc) return rc;
    if (c->params.residual_fields & MESO_RES_L2) {
        const int D = c->dim;
        std::vector<double> list = {residual_l2(c, c->rho_res, rho, 1, 0)};
        std::vector<int> field = {MESO_RES_RHO};
        if (c->params.solver == MESO_SOLVER_CDUGKS_SHAKHOV) list.push_back(residual_l2(c, c->T_res, T, 1, 0)), field.push_back(MESO_RES_T);
        for (int k = 0; k < D; ++k) list.push_back(residual_l2(c, c->u_res, u, 3, k)), field.push_back(MESO_RES_U);
        if (c->params.solver == MESO_SOLVER_CDUGKS_SHAKHOV)
            for (int k = 0; k < D; ++k) list.push_back(residual_l2(c, c->q_res, q, 3, k)), field.push_back(MESO_RES_Q);
        c->rho_res = rho;
        c->T_res = T;
        c->u_res = u;
        c->q_res = q;
        c->nres = (int)list.size();
        for (int i = 0; i < c->nres; ++i) c->last_res[i] = list[i];
        const int watch = c->params.residual_fields & (MESO_RES_RHO | MESO_RES_T | MESO_RES_U | MESO_RES_Q);
        bool conv = true;
        for (size_t i = 0; i < list.size(); ++i)
            if (watch == 0 || (watch & field[i])) conv = conv && (list[i] <= c->params.residual_limit);
        if (conv) c->converge_state++;
        else c->converge_state = 0;
        if (c->converge_state >= 10) {
            c->run_state = 0;
            c->converged = 1;
        }
        return MESO_OK;
    }
    double rr = residual_scalar(c, c->rho_res, rho);
    double ru[3];
    residual_vector(c, c->u_res, u, ru);
    std::vector<double> list;
    std::vector<int> field;  // MESO_RES_* of each entry
    const int D = c->dim;
    if (c->params.solver == MESO_SOLVER_CDUGKS_SHAKHOV) {
        double rT = residual_scalar(c, c->T_res, T);
        double rq[3];
        residual_vector(c, c->q_res, q, rq);
        list = {rr, rT};
        field = {MESO_RES_RHO, MESO_RES_T};
        for (int k = 0; k < D; ++k) list.push_back(ru[k]), field.push_back(MESO_RES_U);
        for (int k = 0; k < D; ++k) list.push_back(rq[k]), field.push_back(MESO_RES_Q);
    } else {
        list = {rr};
        field = {MESO_RES_RHO};
        for (int k = 0; k < D; ++k) list.push_back(ru[k]), field.push_back(MESO_RES_U);
    }
    c->nres = (int)list.size();
    for (int i = 0; i < c->nres; ++i) c->last_res[i] = list[i];
    const int watch = c->params.residual_fields & (MESO_RES_RHO | MESO_RES_T | MESO_RES_U | MESO_RES_Q);
    bool conv = true;
    for (size_t i = 0; i < list.size(); ++i)
        if (watch == 0 || (watch & field[i])) conv = conv && (list[i] <= c->params.residual_limit);
    if (conv) c->converge_state++;
    else c->converge_state = 0;
    if (c->converge_state >= 10) {
        c->run_state = 0;
        c->converged = 1;
    }
    return MESO_OK;
}

// The FP32 step's launches take no per-step arguments (each instance reads its state parity from
// its device step counter), so they are captured once as a CUDA graph and replayed.
bool capture_f32_graph(meso_ctx *c) {
    if (c->f32_graph) cudaGraphExecDestroy(c->f32_graph);
    c->f32_graph = nullptr;
    cudaGraph_t g = nullptr;
    int64_t n = 0;
    if (!c->f32_fork.side &&
        (cudaStreamCreateWithFlags(&c->f32_fork.side, cudaStreamNonBlocking) != cudaSuccess ||
         cudaEventCreateWithFlags(&c->f32_fork.fork, cudaEventDisableTiming) != cudaSuccess ||
         cudaEventCreateWithFlags(&c->f32_fork.join, cudaEventDisableTiming) != cudaSuccess)) {
        cudaGetLastError();
        return false;
    }
    if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return false;
    const int rc = meso::fp32_step(c->fs, c->stream, &n, nullptr, &c->f32_fork);
    const cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    bool ok = rc == 0 && e == cudaSuccess && cudaGraphInstantiate(&c->f32_graph, g, 0) == cudaSuccess;
    if (g) cudaGraphDestroy(g);
    if (!ok) {
        cudaGetLastError();
        c->f32_graph = nullptr;
        return false;
    }
    c->f32_graph_version = c->f32_version;
    c->f32_graph_launches = n;
    return true;
}

// The FP64 step's launches take the step constants (KParams) by value and fixed buffers, so they
// are captured as a graph for the current constants and recaptured when a parameter change (live
// reload, meso_set_params) alters them.
bool capture_plain_graph(meso_ctx *c) {
    if (c->plain_graph) cudaGraphExecDestroy(c->plain_graph);
    c->plain_graph = nullptr;
    cudaGraph_t g = nullptr;
    int64_t n = 0;
    if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return false;
    const int rc = meso::plain_step(c->ps, c->stream, &n);
    const cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    bool ok = rc == 0 && e == cudaSuccess && cudaGraphInstantiate(&c->plain_graph, g, 0) == cudaSuccess;
    if (g) cudaGraphDestroy(g);
    if (!ok) {
        cudaGetLastError();
        c->plain_graph = nullptr;
        return false;
    }
    c->plain_graph_kp = c->ps.kp;
    c->plain_graph_launches = n;
    return true;
}

int launch_step(meso_ctx *c) {
    if (c->params.precision != MESO_FP32 &&
        ((c->plain_graph && std::memcmp(&c->plain_graph_kp, &c->ps.kp, sizeof(meso::KParams)) == 0) ||
         capture_plain_graph(c))) {
        if (cudaGraphLaunch(c->plain_graph, c->stream) != cudaSuccess)
            return fail(MESO_ERR_CUDA, std::string("graph launch failed: ") + cudaGetErrorString(cudaGetLastError()));
        c->last_launches += c->plain_graph_launches;
        return MESO_OK;
    }
    if (c->params.precision == MESO_FP32 && (c->f32_graph_version == c->f32_version || capture_f32_graph(c))) {
        if (cudaGraphLaunch(c->f32_graph, c->stream) != cudaSuccess)
            return fail(MESO_ERR_CUDA, std::string("graph launch failed: ") + cudaGetErrorString(cudaGetLastError()));
        c->last_launches += c->f32_graph_launches;
        return MESO_OK;
    }
    int rc = c->params.precision == MESO_FP32 ? meso::fp32_step(c->fs, c->stream, &c->last_launches)
                                              : meso::plain_step(c->ps, c->stream, &c->last_launches);
    if (rc) return fail(MESO_ERR_CUDA, std::string("kernel launch failed: ") + cudaGetErrorString(cudaGetLastError()));
    return MESO_OK;
}

// New step settings into the FP32 instance: time step, Prandtl number, viscosity law and the
// gradient switch.  R, T0 and rho0 define the stored reference Maxwellian and stay fixed.
int refresh_f32(meso_ctx *c) {
    if (c->params.precision != MESO_FP32) return MESO_OK;
    meso::F32Inst &I = c->f32;
    const meso_params &p = c->params;
    I.dt = p.dt;
    I.hdt = p.dt * 0.5;
    I.hdt32 = (float)I.hdt;
    I.Pr = p.Pr;
    I.mu0 = p.mu0;
    I.vhs = p.vhs_index;
    I.gradient = p.gradient_switch;
    I.res_interval = p.residual_interval;
    I.res_fields = p.residual_fields;
    I.res_limit = p.residual_limit;
    CUDA_TRY(cudaMemcpyAsync(c->fs.d_inst, &I, sizeof(I), cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->f32_version++;
    return MESO_OK;
}

bool fp32_fixed_changed(const meso_params &a, const meso_params &b) {
    return a.R != b.R || a.T0 != b.T0 || a.rho0 != b.rho0 || a.K != b.K || a.limiter_switch != b.limiter_switch ||
           a.tile_cells != b.tile_cells || a.vpl != b.vpl || a.ngroup != b.ngroup;
}

// Live reload of [settings] (cdugks_shakhov.cpp:762): the reference re-reads
// the case file after every step; re-reading only when its mtime changed
// gives the same settings without a file read per step.
void maybe_reload(meso_ctx *c) {
    if (!c->kase || c->params.solver != MESO_SOLVER_CDUGKS_SHAKHOV) return;
    struct stat sb;
    if (stat(c->kase->config.path().c_str(), &sb) != 0) return;
    if (sb.st_mtime == c->case_mtime) return;
    c->case_mtime = sb.st_mtime;
    try {
        c->kase->params.precision = c->params.precision;
        if (c->kase->reload_settings()) {
            const meso_params prev = c->params;
            c->params = c->kase->params;
            if (c->params.precision == MESO_FP32 && fp32_fixed_changed(prev, c->params)) {
                c->params.R = prev.R;  // the FP32 form keeps its reference state
                c->params.T0 = prev.T0;
                c->params.rho0 = prev.rho0;
                c->params.K = prev.K;
                c->params.limiter_switch = prev.limiter_switch;
                c->params.tile_cells = prev.tile_cells;
                c->params.vpl = prev.vpl;
                c->params.ngroup = prev.ngroup;
            }
            derive_kparams(c->params, c->dim, c->ps.kp);
            refresh_f32(c);
        }
    } catch (...) {
        // a half-written file keeps the current settings; the next change retries
    }
}

meso_ctx *new_ctx(const meso_mesh_desc *m, const meso_dvs_desc *d, const meso_mark_desc *marks, int nmarks,
                  const meso_params *p, const uint8_t *mask, int *rc) {
    auto c = std::make_unique<meso_ctx>();
    c->params = *p;
    c->dim = m->dim;
    c->C = m->ncell;
    c->F = m->nface;
    c->NV = d->nv;
    c->marks.assign(marks, marks + nmarks);
    if (mask) c->mask.assign(mask, mask + m->ncell);
    c->vol.assign(m->cell_vol, m->cell_vol + m->ncell);
    c->min_cell_size = m->min_cell_size;
    c->total_volume = m->total_volume;
    if (!(c->total_volume > 0.0)) {
        c->total_volume = 0.0;
        for (double v : c->vol) c->total_volume += v;
    }
    c->dvs_max_mag = d->max_magnitude;
    if (c->params.solver == MESO_SOLVER_DUGKS) {
        double mm = d->max_magnitude;
        if (!(mm > 0.0)) {
            for (int i = 0; i < d->nv; ++i) {
                double v = std::sqrt(d->xi[3 * i] * d->xi[3 * i] + d->xi[3 * i + 1] * d->xi[3 * i + 1] +
                                     d->xi[3 * i + 2] * d->xi[3 * i + 2]);
                mm = std::max(mm, v);
            }
        }
        c->params.dt = c->params.CFL * (c->min_cell_size / mm);  // dugks.cpp:47
    }
    std::string why;
    if (!valid_params(c->params, why)) {
        *rc = fail(MESO_ERR_INVALID, why);
        return nullptr;
    }
    if (c->params.precision == MESO_FP32) {
        if (c->params.solver != MESO_SOLVER_CDUGKS_SHAKHOV || m->dim != 2 || c->params.limiter_switch) {
            *rc = fail(MESO_ERR_UNSUPPORTED,
                       "FP32 storage covers the 2-D Shakhov solver without the limiter; use MESO_FP64");
            return nullptr;
        }
        if (c->params.tile_cells == 0 && c->params.vpl == 0 && c->params.ngroup == 0) {
            int tc = 0, v = 0, ng = 0;  // a shape the autotuner measured for a solve of this size
            if (tuned_shape(m->ncell, m->nface, d->nv, tc, v, ng)) {
                c->params.tile_cells = tc;
                c->params.vpl = v;
                c->params.ngroup = ng;
            }
        }
        const int T = c->params.tile_cells > 0 ? c->params.tile_cells : meso::F32_DEFAULT_CELLS;
        if (T < 8 || T > meso::F32_MAX_CELLS || c->params.vpl < 0 || c->params.vpl > meso::F32_MAX_VPL ||
            c->params.ngroup < 0) {
            *rc = fail(MESO_ERR_INVALID, "FP32 kernel shape out of range (tile_cells 8.." +
                                             std::to_string(meso::F32_MAX_CELLS) + ", vpl 0..2, ngroup >= 0)");
            return nullptr;
        }
        if (!plan_fp32(*m, T, c->rn, c->plan)) {
            *rc = fail(MESO_ERR_UNSUPPORTED, "mesh connectivity exceeds the FP32 tile limits");
            return nullptr;
        }
    } else {
        c->rn = renumber(*m, false);
    }
    derive_kparams(c->params, c->dim, c->ps.kp);
    *rc = build_device(c.get(), m, d);
    if (*rc != MESO_OK) return nullptr;
    derive_kparams(c->params, c->dim, c->ps.kp);
    reset_status(c.get());
    return c.release();
}

int init_common(meso_ctx *c, const double *rho, const double *u, const double *T, const double *q, int mode) {
    const int C = c->C;
    if (!rho || !u) return fail(MESO_ERR_INVALID, "rho and u are required");
    const bool shakhov = c->params.solver == MESO_SOLVER_CDUGKS_SHAKHOV;
    if (shakhov && !T) return fail(MESO_ERR_INVALID, "T is required for the Shakhov solver");
    if (mode != 0 && mode != 1) return fail(MESO_ERR_INVALID, "mode must be 0 or 1");
    std::vector<double> r, uu, t(C, 0.0), qq(3 * (size_t)C, 0.0);
    to_new(c, rho, r, 1);
    to_new(c, u, uu, 3);
    if (T) to_new(c, T, t, 1);
    if (q && shakhov) to_new(c, q, qq, 3);
    CUDA_TRY(cudaMemcpyAsync(c->ps.rho, r.data(), sizeof(double) * C, cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(cudaMemcpyAsync(c->ps.u, uu.data(), sizeof(double) * 3 * C, cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(cudaMemcpyAsync(c->ps.T, t.data(), sizeof(double) * C, cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(cudaMemcpyAsync(c->ps.q, qq.data(), sizeof(double) * 3 * C, cudaMemcpyHostToDevice, c->stream));
    reset_status(c);  // step 0 first: the FP32 init writes S[step parity]
    if (c->params.precision == MESO_FP32) {
        if (meso::fp32_init(c->fs, mode, c->stream)) return fail(MESO_ERR_CUDA, "init kernel launch failed");
    } else if (meso::plain_init(c->ps, mode, c->stream)) {
        return fail(MESO_ERR_CUDA, "init kernel launch failed");
    }
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->step = 0;
    c->solution_time = 0.0;
    c->run_state = 1;
    c->converged = 0;
    c->converge_state = 0;
    c->initialized = true;
    if (c->params.precision == MESO_FP32) {  // the device residual check starts from these macros
        const meso::F32Inst &I = c->f32;
        const size_t C = (size_t)c->C;
        CUDA_TRY(cudaMemcpyAsync(I.rho_old, I.rho, sizeof(double) * C, cudaMemcpyDeviceToDevice, c->stream));
        CUDA_TRY(cudaMemcpyAsync(I.u_old, I.u, sizeof(double) * 3 * C, cudaMemcpyDeviceToDevice, c->stream));
        CUDA_TRY(cudaMemcpyAsync(I.T_old, I.T, sizeof(double) * C, cudaMemcpyDeviceToDevice, c->stream));
        CUDA_TRY(cudaMemcpyAsync(I.q_old, I.q, sizeof(double) * 3 * C, cudaMemcpyDeviceToDevice, c->stream));
        CUDA_TRY(cudaMemsetAsync(I.resid, 0, sizeof(meso::F32Resid), c->stream));
    }
    std::vector<double> T2, q2;
    int rc = download_macros(c, c->rho_res, c->u_res, T2, q2);
    if (rc) return rc;
    c->T_res = T2;
    c->q_res = q2;
    return MESO_OK;
}

std::vector<double> read_scalar_file(const std::string &f, int n) {
    MESO::Field<double> fld;
    fld.len = n;
    fld.values.assign(n, 0.0);
    MESO::read_np_data<double>(f, fld);
    return fld.values;
}
std::vector<double> read_vector_file(const std::string &f, int n) {
    MESO::Field<MESO::Vector> fld;
    fld.len = n;
    fld.values.assign(n, MESO::Vector());
    MESO::read_np_data<MESO::Vector>(f, fld);
    std::vector<double> out(3 * (size_t)n);
    for (int i = 0; i < n; ++i) {
        out[3 * i] = fld.values[i].x;
        out[3 * i + 1] = fld.values[i].y;
        out[3 * i + 2] = fld.values[i].z;
    }
    return out;
}

#define CTX_CHECK(c)                                                        \
    do {                                                                    \
        if (!(c)) return fail(MESO_ERR_INVALID, "null context");            \
        if (cudaSetDevice((c)->device) != cudaSuccess)                      \
            return fail(MESO_ERR_CUDA, "cannot select the context's device"); \
    } while (0)

}  // namespace

namespace meso_host {
int ctx_read_status(meso_ctx *c) { return read_status(c); }
int ctx_read_resid(meso_ctx *c) {
    meso::F32Resid r;
    CUDA_TRY(cudaMemcpyAsync(&r, c->f32.resid, sizeof(r), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->converge_state = r.converge_state;
    if (r.nres > 0) {
        c->nres = r.nres;
        for (int i = 0; i < r.nres && i < 8; ++i) c->last_res[i] = r.res[i];
    }
    if (r.converged) {
        c->run_state = 0;
        c->converged = 1;
    }
    return MESO_OK;
}
int ctx_residual_check(meso_ctx *c) { return residual_check(c); }
}  // namespace meso_host

extern "C" {

const char *meso_last_error(void) { return last_error_cstr(); }

const char *meso_version(void) { return "meso-gb300 1.0 sm_103a (FP64 plain step, FP32 tiled Shakhov step)"; }

int meso_case_load(const char *case_file, meso_case **out) {
    if (!case_file || !out) return fail(MESO_ERR_INVALID, "null argument");
    *out = nullptr;
    try {
        *out = load_case(case_file).release();
        return MESO_OK;
    } catch (const std::invalid_argument &e) {
        std::string msg = e.what();
        bool io = msg.find("file open error") != std::string::npos;
        return fail(io ? MESO_ERR_IO : MESO_ERR_INVALID, msg);
    } catch (const std::exception &e) {
        return fail(MESO_ERR_IO, std::string("case load failed: ") + e.what());
    }
}

void meso_case_free(meso_case *c) { delete c; }

int meso_case_mesh(const meso_case *c, meso_mesh_desc *m) {
    if (!c || !m) return fail(MESO_ERR_INVALID, "null argument");
    c->mesh_desc(*m);
    return MESO_OK;
}

int meso_case_dvs(const meso_case *c, meso_dvs_desc *d) {
    if (!c || !d) return fail(MESO_ERR_INVALID, "null argument");
    c->dvs_desc(*d);
    return MESO_OK;
}

int meso_case_marks(const meso_case *c, const meso_mark_desc **marks, int32_t *n) {
    if (!c || !marks || !n) return fail(MESO_ERR_INVALID, "null argument");
    *marks = c->marks.data();
    *n = (int32_t)c->marks.size();
    return MESO_OK;
}

int meso_case_params(const meso_case *c, meso_params *p) {
    if (!c || !p) return fail(MESO_ERR_INVALID, "null argument");
    *p = c->params;
    return MESO_OK;
}

int meso_case_initial_fields(const meso_case *c, double *rho, double *u, double *T, uint8_t *mask) {
    if (!c) return fail(MESO_ERR_INVALID, "null argument");
    try {
        c->initial_fields(rho, u, T, mask);
    } catch (const std::exception &e) {
        return fail(MESO_ERR_INVALID, e.what());
    }
    return MESO_OK;
}

int meso_case_loop_settings(const meso_case *c, int32_t *max_step, int32_t *write_interval, int32_t *read_np_data,
                            int32_t *output_latest, int32_t *output_np) {
    if (!c) return fail(MESO_ERR_INVALID, "null argument");
    if (max_step) *max_step = c->max_step;
    if (write_interval) *write_interval = c->write_interval;
    if (read_np_data) *read_np_data = c->read_np_data;
    if (output_latest) *output_latest = c->output_latest;
    if (output_np) *output_np = c->output_np;
    return MESO_OK;
}

int meso_case_output_grid(const meso_case *c, const char *path) {
    if (!c || !path) return fail(MESO_ERR_INVALID, "null argument");
    try {
        write_grid(*c, path);
    } catch (const std::exception &e) {
        return fail(MESO_ERR_IO, e.what());
    }
    return MESO_OK;
}

int meso_ctx_create(const meso_mesh_desc *mesh, const meso_dvs_desc *dvs, const meso_mark_desc *marks, int32_t nmarks,
                    const meso_params *params, const uint8_t *mask, meso_ctx **out) {
    if (!out || !params) return fail(MESO_ERR_INVALID, "null argument");
    *out = nullptr;
    int rc = check_desc(mesh, dvs, marks, nmarks);
    if (rc) return rc;
    try {
        meso_ctx *c = new_ctx(mesh, dvs, marks, nmarks, params, mask, &rc);
        if (!c) return rc;
        *out = c;
        return MESO_OK;
    } catch (const std::exception &e) {
        return fail(MESO_ERR_INVALID, e.what());
    }
}

int meso_ctx_create_from_case(const char *case_file, int32_t precision, meso_ctx **out) {
    if (!out) return fail(MESO_ERR_INVALID, "null argument");
    *out = nullptr;
    meso_case *k = nullptr;
    int rc = meso_case_load(case_file, &k);
    if (rc) return rc;
    std::unique_ptr<meso_case> kase(k);
    if (precision == MESO_FP64 || precision == MESO_FP32) kase->params.precision = precision;
    meso_mesh_desc m;
    meso_dvs_desc d;
    kase->mesh_desc(m);
    kase->dvs_desc(d);
    std::vector<uint8_t> mask(kase->mesh.NCELL, 0);
    try {
        kase->initial_fields(nullptr, nullptr, nullptr, mask.data());
    } catch (const std::exception &e) {
        return fail(MESO_ERR_INVALID, e.what());
    }
    rc = meso_ctx_create(&m, &d, kase->marks.data(), (int)kase->marks.size(), &kase->params, mask.data(), out);
    if (rc) return rc;
    struct stat sb;
    if (stat(kase->config.path().c_str(), &sb) == 0) (*out)->case_mtime = sb.st_mtime;
    (*out)->kase = std::move(kase);
    return MESO_OK;
}

void meso_ctx_destroy(meso_ctx *c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->batch) meso_host::batch_forget(c->batch, c);
    if (c->f32_graph) cudaGraphExecDestroy(c->f32_graph);
    if (c->plain_graph) cudaGraphExecDestroy(c->plain_graph);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->f32_fork.side) cudaStreamDestroy(c->f32_fork.side);
    if (c->f32_fork.fork) cudaEventDestroy(c->f32_fork.fork);
    if (c->f32_fork.join) cudaEventDestroy(c->f32_fork.join);
    free_fp32_launch(c->fs, c->fs_owned);
    c->arena.release();
    if (c->h_status) cudaFreeHost(c->h_status);
    if (c->h_mac) cudaFreeHost(c->h_mac);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

int meso_init_macros(meso_ctx *c, const double *rho, const double *u, const double *T, const double *q, int32_t mode) {
    CTX_CHECK(c);
    return init_common(c, rho, u, T, q, mode);
}

int meso_initial(meso_ctx *c) {
    CTX_CHECK(c);
    if (!c->kase) return fail(MESO_ERR_INVALID, "meso_initial needs a context made from a case file");
    const int C = c->C;
    auto &k = *c->kase;
    try {
        if (k.read_np_data) {
            std::vector<double> rho, u, T, q;
            if (c->params.solver == MESO_SOLVER_DUGKS) {
                // dugks.cpp:57-59
                rho = read_scalar_file(k.case_name + "/np-data/Rho.np.dat", C);
                u = read_vector_file(k.case_name + "/np-data/vel.np.dat", C);
            } else {
                rho = read_scalar_file(k.case_name + "/latest/Rho", C);
                u = read_vector_file(k.case_name + "/latest/U", C);
                if (c->params.solver == MESO_SOLVER_CDUGKS_SHAKHOV) {
                    T = read_scalar_file(k.case_name + "/latest/T", C);
                    q = read_vector_file(k.case_name + "/latest/q", C);
                }
            }
            return init_common(c, rho.data(), u.data(), T.empty() ? nullptr : T.data(),
                               q.empty() ? nullptr : q.data(), 1);
        }
        std::vector<double> rho(C), u(3 * (size_t)C), T(C);
        k.initial_fields(rho.data(), u.data(), T.data(), nullptr);
        return init_common(c, rho.data(), u.data(), T.data(), nullptr, 0);
    } catch (const std::exception &e) {
        return fail(MESO_ERR_IO, e.what());
    }
}

// One step of an FP32 context with defect correction: the FP64 step from the current state (its
// step counter and flags put back afterwards), the corrected FP32 step from the same state, then
// the corrections take the difference and the state continues from the FP64 result.
static int refine_step(meso_ctx *c) {
    const auto &I = c->f32;
    auto &s = c->ps64;
    s.kp = c->ps.kp;  // the current step settings
    if (meso::fp32_to_plain(I, c->fs.d_inst, s.f0, s.f1, s.rho, c->num_sms, c->stream))
        return fail(MESO_ERR_CUDA, std::string("refine: ") + cudaGetErrorString(cudaGetLastError()));
    CUDA_TRY(cudaMemcpyAsync(c->d_status_save, c->d_status, sizeof(meso::DStatus), cudaMemcpyDeviceToDevice, c->stream));
    if (meso::plain_step(s, c->stream, &c->last_launches))
        return fail(MESO_ERR_CUDA, std::string("refine: FP64 step: ") + cudaGetErrorString(cudaGetLastError()));
    CUDA_TRY(cudaMemcpyAsync(c->d_status, c->d_status_save, sizeof(meso::DStatus), cudaMemcpyDeviceToDevice, c->stream));
    c->fs.corr = 2;  // the measuring step, launched directly (the captured step is the corrected one)
    const int rc = meso::fp32_step(c->fs, c->stream, &c->last_launches);
    c->fs.corr = 1;
    if (rc) return fail(MESO_ERR_CUDA, std::string("refine: FP32 step: ") + cudaGetErrorString(cudaGetLastError()));
    if (meso::fp32_refine(I, c->fs.d_inst, s.f0, s.f1, s.rho, c->num_sms, c->stream))
        return fail(MESO_ERR_CUDA, std::string("refine: ") + cudaGetErrorString(cudaGetLastError()));
    return MESO_OK;
}

int meso_fp32_refine(meso_ctx *c, int32_t interval) {
    CTX_CHECK(c);
    if (interval < 0) return fail(MESO_ERR_INVALID, "interval must be >= 0");
    if (c->params.precision != MESO_FP32 || c->params.solver != MESO_SOLVER_CDUGKS_SHAKHOV || c->dim != 2)
        return fail(MESO_ERR_UNSUPPORTED, "defect correction applies to 2-D Shakhov FP32 contexts");
    if (c->batch) return fail(MESO_ERR_INVALID, "a batch member steps with its batch: leave the batch first");
    auto &I = c->f32;
    const size_t C = (size_t)c->C;
    if (interval > 0 && !c->corrS_mem) {  // first use: the corrections and the FP64 step's buffers
        auto &A = c->arena;
        auto &s = c->ps64;
        s.solver = c->params.solver;
        s.num_sms = c->num_sms;
        s.mesh = c->dm;
        s.status = c->d_status;
        const size_t cv = C * (size_t)c->NV, fv = (size_t)c->F * (size_t)c->NV;
        const size_t bv = (size_t)std::max(c->nb, 1) * (size_t)c->NV;
        try {
            c->corrS_mem = A.alloc<float2>(C * (size_t)I.NVp);
            c->corrW_mem = A.alloc<double>(4 * C);
            c->corrq_mem = A.alloc<double>(2 * C);
            c->corrR_mem = A.alloc<float2>(C * (size_t)I.NVp);
            s.f0 = A.alloc<double>(cv);
            s.f1 = A.alloc<double>(cv);
            s.face0 = A.alloc<double>(fv);
            s.face1 = A.alloc<double>(fv);
            s.grad0 = A.alloc<double>(cv * 2);
            s.grad1 = A.alloc<double>(cv * 2);
            s.flux0 = A.alloc<double>(cv);
            s.flux1 = A.alloc<double>(cv);
            s.snap0 = A.alloc<double>(bv);
            s.snap1 = A.alloc<double>(bv);
            s.rho = A.alloc<double>(8 * C);
            s.u = s.rho + C;
            s.T = s.rho + 4 * C;
            s.q = s.rho + 5 * C;
            s.fm0 = A.alloc<double>(C);
            s.fm1 = A.alloc<double>(3 * C);
            s.fm2 = A.alloc<double>(C);
            s.repair_list = A.alloc<int>(C);
            c->d_status_save = A.alloc<meso::DStatus>(1);
        } catch (const std::bad_alloc &) {
            cudaGetLastError();
            c->corrS_mem = nullptr;
            return fail(MESO_ERR_OOM, "device allocation for the defect correction failed");
        }
    }
    if (interval > 0 && !I.corrS) {  // switched on: the corrections start from zero
        CUDA_TRY(cudaMemsetAsync(c->corrS_mem, 0, sizeof(float2) * C * (size_t)I.NVp, c->stream));
        CUDA_TRY(cudaMemsetAsync(c->corrW_mem, 0, sizeof(double) * 4 * C, c->stream));
        CUDA_TRY(cudaMemsetAsync(c->corrq_mem, 0, sizeof(double) * 2 * C, c->stream));
    }
    I.corrS = interval > 0 ? c->corrS_mem : nullptr;
    I.corrW = interval > 0 ? c->corrW_mem : nullptr;
    I.corrq = interval > 0 ? c->corrq_mem : nullptr;
    I.corrR = interval > 0 ? c->corrR_mem : nullptr;
    c->refine_interval = interval;
    c->fs.corr = interval > 0 ? 1 : 0;
    CUDA_TRY(cudaMemcpyAsync(c->fs.d_inst, &I, sizeof(I), cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->f32_version++;
    return MESO_OK;
}

int meso_step(meso_ctx *c, int32_t nsteps, int32_t *steps_done) {
    CTX_CHECK(c);
    if (steps_done) *steps_done = 0;
    if (!c->initialized) return fail(MESO_ERR_INVALID, "meso_step before initial()");
    if (nsteps < 0) return fail(MESO_ERR_INVALID, "nsteps must be >= 0");
    if (c->batch) return fail(MESO_ERR_INVALID, "this context is stepped by its batch (meso_batch_step)");
    const int start = c->step;
    std::vector<double> dts;
    dts.reserve(nsteps);
    c->last_launches = 0;
    CUDA_TRY(cudaEventRecord(c->ev0, c->stream));
    int issued = 0;
    bool stopped = false;
    for (int i = 0; i < nsteps && c->run_state; ++i) {
        maybe_reload(c);
        const int ki = c->refine_interval;
        int rc = ki > 0 && c->params.precision == MESO_FP32 && (start + issued) % ki == 0 ? refine_step(c)
                                                                                       : launch_step(c);
        if (rc) return rc;
        dts.push_back(c->params.dt);
        ++issued;
        const int s = start + issued;
        const int ri = c->params.residual_interval;
        if (ri > 0 && s % ri == 0 && c->params.precision != MESO_FP32) {  // FP32: on the device
            rc = read_status(c);
            if (rc) return rc;
            if (c->h_status->stop_step != INT_MAX) {
                stopped = true;
                break;
            }
            rc = residual_check(c);
            if (rc) return rc;
        }
    }
    CUDA_TRY(cudaEventRecord(c->ev1, c->stream));
    int rc = read_status(c);
    if (rc) return rc;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    c->last_ms = ms;
    const int done = c->h_status->step - start;
    for (int i = 0; i < done && i < (int)dts.size(); ++i) c->solution_time += dts[i];
    c->step = c->h_status->step;
    const int ri = c->params.residual_interval;
    if (c->params.precision == MESO_FP32 && ri > 0 && c->step / ri > start / ri &&
        (rc = meso_host::ctx_read_resid(c)))
        return rc;
    if (steps_done) *steps_done = done;
    if (c->h_status->timeout) {
        c->run_state = 0;
        return fail(MESO_ERR_TIMEOUT, "a bounded device wait gave up: the last step's results are invalid");
    }
    if (stopped || c->h_status->stop_step != INT_MAX) {
        c->run_state = 0;
        return fail(MESO_ERR_NAN, "cell " + std::to_string(c->rn.cell_new2old[std::min(c->h_status->first_bad, c->C - 1)]) +
                                      " caught rho = NaN or T < 0 (no mask)");
    }
    return MESO_OK;
}

int meso_get_macros(meso_ctx *c, double *rho, double *u, double *T, double *q) {
    CTX_CHECK(c);
    return fetch_macros(c, rho, u, T, q);
}

int meso_get_flux_moments(meso_ctx *c, double *m0, double *m1, double *m2) {
    CTX_CHECK(c);
    const int C = c->C;
    std::vector<double> a(C), b(3 * (size_t)C), d(C);
    CUDA_TRY(cudaMemcpyAsync(a.data(), c->ps.fm0, sizeof(double) * C, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaMemcpyAsync(b.data(), c->ps.fm1, sizeof(double) * 3 * C, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaMemcpyAsync(d.data(), c->ps.fm2, sizeof(double) * C, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (m0) to_orig(c, a, m0, 1);
    if (m1) to_orig(c, b, m1, 3);
    if (m2) to_orig(c, d, m2, 1);
    return MESO_OK;
}

int meso_get_status(meso_ctx *c, meso_status *st) {
    CTX_CHECK(c);
    if (!st) return fail(MESO_ERR_INVALID, "null status");
    int rc = read_status(c);
    if (rc) return rc;
    std::memset(st, 0, sizeof(*st));
    st->step = c->step;
    st->run_state = c->run_state;
    st->converged = c->converged;
    st->bad_cells = c->h_status->bad_count;
    st->first_bad_cell = c->h_status->first_bad == INT_MAX ? -1 : c->rn.cell_new2old[c->h_status->first_bad];
    st->masked_repairs = c->h_status->repairs_total;
    st->solution_time = c->solution_time;
    st->nresidual = c->nres;
    for (int i = 0; i < c->nres; ++i) st->residual[i] = c->last_res[i];
    return MESO_OK;
}

int meso_set_params(meso_ctx *c, const meso_params *p) {
    CTX_CHECK(c);
    if (!p) return fail(MESO_ERR_INVALID, "null params");
    if (p->solver != c->params.solver || p->precision != c->params.precision)
        return fail(MESO_ERR_INVALID, "solver and precision are fixed for a context");
    std::string why;
    if (!valid_params(*p, why)) return fail(MESO_ERR_INVALID, why);
    if (c->params.precision == MESO_FP32 && fp32_fixed_changed(c->params, *p))
        return fail(MESO_ERR_UNSUPPORTED, "the FP32 form fixes R, T0, rho0, K, the limiter switch and the kernel shape at creation");
    c->params = *p;
    derive_kparams(c->params, c->dim, c->ps.kp);
    return refresh_f32(c);
}

int meso_get_params(meso_ctx *c, meso_params *p) {
    if (!c || !p) return fail(MESO_ERR_INVALID, "null argument");
    *p = c->params;
    return MESO_OK;
}

int meso_output(meso_ctx *c) {
    CTX_CHECK(c);
    if (!c->kase) return fail(MESO_ERR_INVALID, "meso_output needs a context made from a case file");
    std::vector<double> rho, u, T, q, m0(c->C), m1(3 * (size_t)c->C), m2(c->C);
    int rc = download_macros(c, rho, u, T, q);
    if (rc) return rc;
    if (c->params.solver == MESO_SOLVER_CDUGKS_SHAKHOV) {
        rc = meso_get_flux_moments(c, m0.data(), m1.data(), m2.data());
        if (rc) return rc;
    }
    try {
        write_solver_output(*c->kase, c->step, c->solution_time, rho, u, T, q, m0, m1, m2);
    } catch (const std::exception &e) {
        return fail(MESO_ERR_IO, e.what());
    }
    return MESO_OK;
}

// Bytes of the distribution state as stored on the device.
static size_t state_bytes(const meso_ctx *c) {
    if (c->params.precision == MESO_FP32) return sizeof(float2) * (size_t)c->C * c->f32.NVp;
    const size_t nd = c->params.solver == MESO_SOLVER_CDUGKS_SHAKHOV ? 2 : 1;
    return sizeof(double) * nd * (size_t)c->C * c->NV;
}

size_t meso_snapshot_size(meso_ctx *c) {
    if (!c) return 0;
    return 64 + state_bytes(c) + sizeof(double) * 8 * (size_t)c->C + sizeof(meso::DStatus);
}

struct SnapHeader {
    uint32_t magic, C, NV, solver;
    int32_t step, run_state, converged, converge_state;
    double solution_time;
    uint8_t pad[24];
};

int meso_snapshot(meso_ctx *c, void *host, size_t bytes) {
    CTX_CHECK(c);
    if (!host || bytes < meso_snapshot_size(c)) return fail(MESO_ERR_INVALID, "snapshot buffer too small");
    static_assert(sizeof(SnapHeader) == 64, "header size");
    SnapHeader h{};
    h.magic = 0x4D534E50u;
    h.C = c->C;
    h.NV = c->NV;
    h.solver = c->params.solver;
    h.step = c->step;
    h.run_state = c->run_state;
    h.converged = c->converged;
    h.converge_state = c->converge_state;
    h.solution_time = c->solution_time;
    char *p = static_cast<char *>(host);
    std::memcpy(p, &h, sizeof(h));
    p += sizeof(h);
    const size_t cv = (size_t)c->C * c->NV;
    auto d2h = [&](const double *src, size_t n) {
        cudaMemcpyAsync(p, src, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
        p += n * sizeof(double);
    };
    if (c->params.precision == MESO_FP32) {
        int rc = read_status(c);  // the current FP32 buffer is S[device step parity]
        if (rc) return rc;
        cudaMemcpyAsync(p, c->f32.S[c->h_status->step & 1], state_bytes(c), cudaMemcpyDeviceToHost, c->stream);
        p += state_bytes(c);
    } else {
        d2h(c->ps.f0, cv);
        if (c->params.solver == MESO_SOLVER_CDUGKS_SHAKHOV) d2h(c->ps.f1, cv);
    }
    d2h(c->ps.rho, c->C);
    d2h(c->ps.u, 3 * (size_t)c->C);
    d2h(c->ps.T, c->C);
    d2h(c->ps.q, 3 * (size_t)c->C);
    CUDA_TRY(cudaMemcpyAsync(p, c->d_status, sizeof(meso::DStatus), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    return MESO_OK;
}

int meso_restore(meso_ctx *c, const void *host, size_t bytes) {
    CTX_CHECK(c);
    if (!host || bytes < meso_snapshot_size(c)) return fail(MESO_ERR_INVALID, "snapshot buffer too small");
    SnapHeader h;
    std::memcpy(&h, host, sizeof(h));
    if (h.magic != 0x4D534E50u || (int)h.C != c->C || (int)h.NV != c->NV || (int)h.solver != c->params.solver)
        return fail(MESO_ERR_INVALID, "snapshot does not match this context");
    const char *p = static_cast<const char *>(host) + sizeof(h);
    const size_t cv = (size_t)c->C * c->NV;
    auto h2d = [&](double *dst, size_t n) {
        cudaMemcpyAsync(dst, p, n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
        p += n * sizeof(double);
    };
    if (c->params.precision == MESO_FP32) {
        meso::DStatus ds;
        std::memcpy(&ds, p + state_bytes(c) + sizeof(double) * 8 * (size_t)c->C, sizeof(ds));
        cudaMemcpyAsync(c->f32.S[ds.step & 1], p, state_bytes(c), cudaMemcpyHostToDevice, c->stream);
        p += state_bytes(c);
    } else {
        h2d(c->ps.f0, cv);
        if (c->params.solver == MESO_SOLVER_CDUGKS_SHAKHOV) h2d(c->ps.f1, cv);
    }
    h2d(c->ps.rho, c->C);
    h2d(c->ps.u, 3 * (size_t)c->C);
    h2d(c->ps.T, c->C);
    h2d(c->ps.q, 3 * (size_t)c->C);
    CUDA_TRY(cudaMemcpyAsync(c->d_status, p, sizeof(meso::DStatus), cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (c->params.precision == MESO_FP32) {
        std::vector<double> uu(3 * (size_t)c->C);
        std::vector<float2> u32(c->C);
        cudaMemcpyAsync(uu.data(), c->ps.u, sizeof(double) * 3 * c->C, cudaMemcpyDeviceToHost, c->stream);
        cudaStreamSynchronize(c->stream);
        for (int i = 0; i < c->C; ++i) u32[i] = make_float2((float)uu[3 * i], (float)uu[3 * i + 1]);
        cudaMemcpyAsync(c->f32.u32, u32.data(), sizeof(float2) * c->C, cudaMemcpyHostToDevice, c->stream);
    }
    c->step = h.step;
    c->run_state = h.run_state;
    c->converged = h.converged;
    c->converge_state = h.converge_state;
    c->solution_time = h.solution_time;
    c->initialized = true;
    if (c->params.precision == MESO_FP32) {  // the device residual check resumes from the snapshot
        const meso::F32Inst &I = c->f32;
        const size_t C = (size_t)c->C;
        meso::F32Resid r{};
        r.converge_state = h.converge_state;
        r.converged = h.converged;
        r.checks = c->params.residual_interval > 0 ? h.step / c->params.residual_interval : 0;
        r.nres = c->nres;
        for (int i = 0; i < 8; ++i) r.res[i] = c->last_res[i];
        CUDA_TRY(cudaMemcpyAsync(I.resid, &r, sizeof(r), cudaMemcpyHostToDevice, c->stream));
        CUDA_TRY(cudaMemcpyAsync(I.rho_old, I.rho, sizeof(double) * C, cudaMemcpyDeviceToDevice, c->stream));
        CUDA_TRY(cudaMemcpyAsync(I.u_old, I.u, sizeof(double) * 3 * C, cudaMemcpyDeviceToDevice, c->stream));
        CUDA_TRY(cudaMemcpyAsync(I.T_old, I.T, sizeof(double) * C, cudaMemcpyDeviceToDevice, c->stream));
        CUDA_TRY(cudaMemcpyAsync(I.q_old, I.q, sizeof(double) * 3 * C, cudaMemcpyDeviceToDevice, c->stream));
    }
    std::vector<double> T2, q2;
    int rc = download_macros(c, c->rho_res, c->u_res, T2, q2);
    c->T_res = T2;
    c->q_res = q2;
    return rc;
}

size_t meso_ctx_device_bytes(meso_ctx *c) { return c ? c->arena.bytes : 0; }

int meso_phase_times(meso_ctx *c, int32_t nsteps, double *ms, int32_t max_phases, int32_t *nphases) {
    CTX_CHECK(c);
    if (!c->initialized) return fail(MESO_ERR_INVALID, "meso_phase_times before initial()");
    if (nsteps <= 0 || !ms) return fail(MESO_ERR_INVALID, "nsteps must be > 0 and ms non-null");
    const bool f32 = c->params.precision == MESO_FP32;
    const int np = f32 ? meso::F32_NPHASE : meso::PLAIN_NPHASE;
    if (nphases) *nphases = np;
    std::vector<cudaEvent_t> ev((size_t)np + 1);
    for (auto &e : ev) CUDA_TRY(cudaEventCreate(&e));
    std::vector<double> acc(np, 0.0);
    int rc = MESO_OK;
    for (int s = 0; s < nsteps && c->run_state; ++s) {
        rc = f32 ? meso::fp32_step(c->fs, c->stream, &c->last_launches, ev.data())
                 : meso::plain_step(c->ps, c->stream, &c->last_launches, ev.data());
        if (rc) {
            rc = fail(MESO_ERR_CUDA, "kernel launch failed");
            break;
        }
        if (cudaEventSynchronize(ev[np]) != cudaSuccess) {
            rc = fail(MESO_ERR_CUDA, "phase timing failed");
            break;
        }
        for (int k = 0; k < np; ++k) {
            float t = 0.f;
            cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
            acc[k] += t;
        }
        c->solution_time += c->params.dt;
    }
    for (auto &e : ev) cudaEventDestroy(e);
    if (rc) return rc;
    rc = read_status(c);
    if (rc) return rc;
    c->step = c->h_status->step;
    for (int k = 0; k < np && k < max_phases; ++k) ms[k] = acc[k] / nsteps;
    return MESO_OK;
}

const char *meso_phase_name(meso_ctx *c, int32_t i) {
    if (!c) return "";
    if (c->params.precision == MESO_FP32) return (i >= 0 && i < meso::F32_NPHASE) ? meso::kFp32Phases[i] : "";
    return (i >= 0 && i < meso::PLAIN_NPHASE) ? meso::kPlainPhases[i] : "";
}

double meso_last_step_ms(meso_ctx *c) { return c ? c->last_ms : 0.0; }

int64_t meso_last_step_launches(meso_ctx *c) { return c ? c->last_launches : 0; }

}  // extern "C"
