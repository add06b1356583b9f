// FP32 instance set-up.  See fp32_host.h.
#include "fp32_host.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <queue>
#include <utility>

#include "capi_internal.h"

namespace meso_host {

constexpr double kPI_HOST = 3.14159265358979323846;

bool plan_fp32(const meso_mesh_desc &m, int tile_cells, Renumbering &rn, TilePlan &plan) {
    for (int T = std::min(tile_cells, meso::F32_MAX_CELLS); T >= 4; T = T * 7 / 8) {
        std::vector<int> sizes;
        rn = renumber_tiled(m, T, sizes);
        if (build_tile_plan(m, rn, sizes, meso::F32_MAX_SLOTS, meso::F32_MAX_GSLOTS, meso::F32_MAX_OWNED,
                            meso::F32_MAX_CELLS, plan) &&
            plan.max_gentries <= meso::F32_MAX_GENT && plan.max_cf <= meso::F32_MAX_CF &&
            plan.max_tf <= meso::F32_MAX_TF)
            return true;
    }
    return false;
}

namespace {
// A split over P runs: the first (ntile / P) P tiles go whole, tile t to run t % P, so that the
// runs step through them in rounds of P neighbouring tiles, all at the same velocity chunk (the
// halo cells one tile reads are read by its neighbours' CTAs at the same time, from L2).  The
// chunks of the b = ntile % P tiles left, tile after tile, are cut into P equal runs of q (at
// least two chunks where tiles have two), unless b is nearly P: then they go whole too.
struct SplitShape {
    int full, b;  // tiles of the whole rounds; tiles left
    long q;       // chunks per run of the tiles left (0: they go whole)
};
SplitShape split_shape(int ntile, int chunks, int split) {
    SplitShape sh;
    sh.full = ntile / split * split;
    sh.b = ntile - sh.full;
    sh.q = 0;
    if (sh.b > 0 && (long)sh.b * 10 < (long)split * 9)
        sh.q = std::max(((long)sh.b * chunks + split - 1) / split, (long)std::min(2, chunks));
    return sh;
}
}  // namespace

std::vector<TilePiece> tile_pieces(int ntile, int chunks, int ngroup, int split) {
    std::vector<TilePiece> out;
    if (split <= 0) {  // ngroup groups of ceil(chunks / ngroup) chunks per tile
        const int cpg = (chunks + ngroup - 1) / ngroup;
        for (int t = 0; t < ntile; ++t)
            for (int g = 0; g < ngroup; ++g) {
                const int c0 = std::min(chunks, g * cpg), c1 = std::min(chunks, c0 + cpg);
                out.push_back({t, g, c0, c1, -1});
            }
        return out;
    }
    const SplitShape sh = split_shape(ntile, chunks, split);
    std::vector<int> cnt(ntile, 0);
    auto whole = [&](int t, int r) {
        out.push_back({t, 0, 0, chunks, r});
        cnt[t] = 1;
    };
    for (int t = 0; t < sh.full; ++t) whole(t, t % split);
    if (sh.q == 0) {
        for (int t = sh.full; t < ntile; ++t) whole(t, t - sh.full);
    } else {  // run r: chunks [r q, (r + 1) q) of the tiles left, cut at tile ends
        const long total = (long)sh.b * chunks;
        for (long r = 0; r * sh.q < total; ++r)
            for (long a = r * sh.q, e = std::min(total, a + sh.q); a < e;) {
                const int t = sh.full + (int)(a / chunks), c0 = (int)(a % chunks);
                const int c1 = (int)std::min<long>(chunks, c0 + (e - a));
                out.push_back({t, cnt[t]++, c0, c1, (int)r});
                a += c1 - c0;
            }
    }
    (void)ngroup;  // rows g >= cnt[t] of a tile are never written: zeroed once, when allocated
    return out;
}

int split_ngroup(int ntile, int chunks, int split) {
    const SplitShape sh = split_shape(ntile, chunks, split);
    int most = 1;
    if (sh.q == 0) return most;
    // the pieces of left tile u are the runs that touch it: floor(u chunks / q) .. floor(((u + 1) chunks - 1) / q)
    for (int u = 0; u < sh.b; ++u) {
        const long r0 = (long)u * chunks / sh.q, r1 = ((long)(u + 1) * chunks - 1) / sh.q;
        most = std::max(most, (int)(r1 - r0 + 1));
    }
    return most;
}

int default_ngroup(int ntile, int chunks, int num_sms) {
    // ~6 (tile, group) items per persistent CTA (one per SM), groups of at least 2 chunks
    int want = (6 * num_sms + ntile - 1) / std::max(ntile, 1);
    want = std::max(want, 1);
    want = std::max(1, std::min(want, std::max(1, chunks / 2)));
    return want;
}

namespace {
template <class T> T *up(DevArena &A, const std::vector<T> &v, cudaStream_t s) {
    T *p = A.alloc<T>(v.size());
    if (!v.empty()) cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s);
    return p;
}
}  // namespace

int build_fp32_instance(meso_ctx *c, const meso_mesh_desc *m, const meso_dvs_desc *d, const TilePlan &P, int ngroup,
                        int vpl_req) {
    auto &A = c->arena;
    auto s = c->stream;
    const int C = m->ncell, F = m->nface, NV = d->nv;
    // small velocity sets keep one velocity per lane unless asked otherwise
    const int vpl = vpl_req == 1 || vpl_req == 2 ? vpl_req : (NV >= 256 ? 2 : 1);
    const int NVp = (NV + 32 * vpl - 1) / (32 * vpl) * (32 * vpl);
    const auto &rn = c->rn;
    meso::F32Inst I;
    std::memset(&I, 0, sizeof(I));
    I.C = C;
    I.F = F;
    I.NV = NV;
    I.NVp = NVp;
    I.ntile = P.ntile;
    I.vpl = vpl;
    I.chunks = NVp / (32 * vpl);
    if (I.chunks > 0xffff) return fail(MESO_ERR_UNSUPPORTED, "FP32 form: more than 65535 velocity chunks");
    if (ngroup > 0) {  // groups take ceil(chunks / ngroup) chunks each: drop groups that would be left empty
        I.split = 0;
        I.ngroup = std::min(ngroup, I.chunks);
        const int cpg = (I.chunks + I.ngroup - 1) / I.ngroup;
        I.ngroup = (I.chunks + cpg - 1) / cpg;
    } else {  // equal runs of chunks, one per SM
        I.split = std::max(1, c->num_sms);
        I.ngroup = split_ngroup(P.ntile, I.chunks, I.split);
    }
    const meso_params &p = c->params;
    I.dt = p.dt;
    I.hdt = p.dt * 0.5;
    I.hdt32 = (float)I.hdt;
    I.R = p.R;
    I.Pr = p.Pr;
    I.mu0 = p.mu0;
    I.vhs = p.vhs_index;
    I.T0 = p.T0;
    I.Kd = (double)p.K;
    I.k3_32 = (float)(I.Kd + 1.0);
    I.twoK32 = (float)(2.0 * I.Kd);
    I.Cv = (p.K + 3.0) * p.R * 0.5;
    I.gamma = (p.K + 5.0) / (p.K + 3.0);
    I.rho0 = p.rho0 > 0.0 ? p.rho0 : 1.0;
    I.iR = 1.0 / I.R;
    I.iT0 = 1.0 / I.T0;
    I.iCv = 1.0 / I.Cv;
    I.iRT0 = 1.0 / (I.R * I.T0);
    I.irho0 = 1.0 / I.rho0;
    I.hm0 = (p.K + 1.0) * p.R * p.T0;
    I.gradient = p.gradient_switch;
    I.res_interval = p.residual_interval;
    I.res_fields = p.residual_fields;
    I.res_limit = p.residual_limit;
    I.total_volume = m->total_volume;
    // renumbered face geometry and boundary index
    std::vector<int> fown(F), fnei(F), fbnd(F, -1), bface, fmark(F);
    std::vector<float2> fn32(F), fdo(F), fdn(F);
    std::vector<double2> fn64(F);
    std::vector<float> farea(F);
    std::vector<double> farea64(F);
    for (int f = 0; f < F; ++f) {
        int o = rn.face_new2old[f];
        int ow = m->face_cell[2 * o], ne = m->face_cell[2 * o + 1];
        fown[f] = rn.cell_old2new[ow];
        fnei[f] = rn.cell_old2new[ne];
        fmark[f] = m->face_mark[o];
        const double *n = m->face_normal + 3 * (size_t)o, *fp = m->face_pos + 3 * (size_t)o;
        fn64[f] = make_double2(n[0], n[1]);
        fn32[f] = make_float2((float)n[0], (float)n[1]);
        const double *po = m->cell_pos + 3 * (size_t)ow, *pn = m->cell_pos + 3 * (size_t)ne;
        fdo[f] = make_float2((float)(fp[0] - po[0]), (float)(fp[1] - po[1]));
        fdn[f] = make_float2((float)(fp[0] - pn[0]), (float)(fp[1] - pn[1]));
        farea[f] = (float)m->face_area[o];
        farea64[f] = m->face_area[o];
        if (c->marks[fmark[f]].type != MESO_BC_FLUID_INTERIOR) {
            fbnd[f] = (int)bface.size();
            bface.push_back(f);
        }
    }
    I.nb = (int)bface.size();
    std::vector<float> xx(NVp, 0.f), xy(NVp, 0.f), w(NVp, 0.f);
    std::vector<double> xx64(NVp, 0.0), xy64(NVp, 0.0), w64(NVp, 0.0);
    for (int q = 0; q < NV; ++q) {
        xx64[q] = d->xi[3 * q];
        xy64[q] = d->xi[3 * q + 1];
        w64[q] = d->w[q];
        xx[q] = (float)xx64[q];
        xy[q] = (float)xy64[q];
        w[q] = (float)w64[q];
    }
    // reference Maxwellian g0 = rho0 / (2 pi R T0) exp(-|xi|^2 / (2 R T0)) and its discrete moments
    std::vector<double> g064(NVp, 0.0);
    std::vector<float> g032(NVp, 0.f);
    {
        const double over = 0.5 / (p.R * p.T0);
        double sum[10] = {0}, cmp[10] = {0};
        for (int q = 0; q < NV; ++q) {
            const double x = xx64[q], y = xy64[q];
            g064[q] = I.rho0 * over / kPI_HOST * std::exp(-(x * x + y * y) * over);
            g032[q] = (float)g064[q];
            const double wg = w64[q] * g064[q];
            const double mono[10] = {1.0, x, y, x * x, x * y, y * y, x * x * x, x * x * y, x * y * y, y * y * y};
            for (int k = 0; k < 10; ++k) {  // compensated (Neumaier) sums
                const double v = wg * mono[k], t = sum[k] + v;
                cmp[k] += std::fabs(sum[k]) >= std::fabs(v) ? (sum[k] - t) + v : (v - t) + sum[k];
                sum[k] = t;
            }
        }
        for (int k = 0; k < 10; ++k) I.gmom[k] = sum[k] + cmp[k];
    }
    std::vector<int> sym(3 * (size_t)NV, 0);
    if (d->sym)
        for (int q = 0; q < 3 * NV; ++q) sym[q] = d->sym[q];
    try {
        I.tile_cstart = up(A, P.tile_cstart, s);
        I.tile_ncell = up(A, P.tile_ncell, s);
        I.tile_slot_ptr = up(A, P.tile_slot_ptr, s);
        I.slot_cell = up(A, P.slot_cell, s);
        I.tile_gslots = up(A, P.tile_gslots, s);
        I.tile_gsp_off = up(A, P.tile_gsp_off, s);
        I.gs_ptr = up(A, P.gs_ptr, s);
        I.gs_nbr = up(A, P.gs_nbr, s);
        I.gs_ax = up(A, P.gs_ax, s);
        I.gs_ay = up(A, P.gs_ay, s);
        I.tile_fstart = up(A, P.tile_fstart, s);
        I.face_own_slot = up(A, P.face_own_slot, s);
        I.face_nei_slot = up(A, P.face_nei_slot, s);
        I.tile_tf_ptr = up(A, P.tile_tf_ptr, s);
        I.tf_face = up(A, P.tf_face, s);
        I.cf_tf = up(A, P.cf_tf, s);
        I.cf_ptr = c->dm.cf_ptr;
        I.cf_face = c->dm.cf_face;
        I.fown = up(A, fown, s);
        I.fnei = up(A, fnei, s);
        I.fbnd = up(A, fbnd, s);
        I.bface = up(A, bface, s);
        I.fmark = up(A, fmark, s);
        I.fn32 = up(A, fn32, s);
        I.fdo = up(A, fdo, s);
        I.fdn = up(A, fdn, s);
        I.fn64 = up(A, fn64, s);
        I.farea = up(A, farea, s);
        I.farea64 = up(A, farea64, s);
        I.vol = c->dm.vol;
        I.marks = c->dm.marks;
        I.mask = c->dm.mask;
        I.cn_ptr = c->dm.cn_ptr;
        I.cn_cell = c->dm.cn_cell;
        I.lsq_dr = c->dm.lsq_dr;
        I.xi32x = up(A, xx, s);
        I.xi32y = up(A, xy, s);
        I.w32 = up(A, w, s);
        I.xi64x = up(A, xx64, s);
        I.xi64y = up(A, xy64, s);
        I.w64 = up(A, w64, s);
        I.g0_32 = up(A, g032, s);
        std::vector<float4> vt(NVp);
        for (int q = 0; q < NVp; ++q) vt[q] = make_float4(xx[q], xy[q], w[q], g032[q]);
        I.vt32 = up(A, vt, s);
        I.g0_64 = up(A, g064, s);
        I.sym = up(A, sym, s);
        const size_t cv = (size_t)C * NVp;
        I.S[0] = A.alloc<float2>(cv);
        I.S[1] = A.alloc<float2>(cv);
        I.u32 = A.alloc<float2>(C);
        I.fk = A.alloc<meso::FaceK>(F);
        I.fmom = A.alloc<float2>((size_t)F * meso::F32_NMOM);
        I.fmac = A.alloc<double>((size_t)F * 8);
        I.fgbar = A.alloc<double>((size_t)F * 4);
        I.fsum = A.alloc<double>((size_t)F * 4);
        I.g0flux = A.alloc<double>((size_t)F * 4);
        I.fcls = A.alloc<uint2>((size_t)F * (NVp / 32));
        I.bnd_in = A.alloc<float2>((size_t)std::max(I.nb, 1) * NVp);
        I.bnd_out = A.alloc<float2>((size_t)std::max(I.nb, 1) * NVp);
        I.bnd_g0 = A.alloc<double>(2 * (size_t)std::max(I.nb, 1));
        I.fbar = A.alloc<float2>((size_t)F * NVp);
        I.ck = A.alloc<meso::CellK>(C);
        I.qpart = A.alloc<float4>((size_t)I.ngroup * C);
        I.rho = A.alloc<double>(8 * (size_t)C);  // rho, u, T, q contiguous: one copy to the host
        I.u = I.rho + C;
        I.T = I.rho + 4 * (size_t)C;
        I.q = I.rho + 5 * (size_t)C;
        I.fm0 = A.alloc<double>(C);
        I.fm1 = A.alloc<double>(3 * (size_t)C);
        I.fm2 = A.alloc<double>(C);
        I.repair_list = A.alloc<int>(C);
        I.resid = A.alloc<meso::F32Resid>(1);
        I.rho_old = A.alloc<double>(C);
        I.u_old = A.alloc<double>(3 * (size_t)C);
        I.T_old = A.alloc<double>(C);
        I.q_old = A.alloc<double>(3 * (size_t)C);
        cudaMemsetAsync(I.resid, 0, sizeof(meso::F32Resid), s);
        // heat-flux partial rows that no piece of a tile writes (a split tile's fewer groups) stay zero
        cudaMemsetAsync(I.qpart, 0, sizeof(float4) * (size_t)I.ngroup * C, s);
        I.status = c->d_status;
        cudaMemsetAsync(I.S[0], 0, cv * sizeof(float2), s);
        cudaMemsetAsync(I.S[1], 0, cv * sizeof(float2), s);
        cudaMemsetAsync(I.fm0, 0, sizeof(double) * C, s);
        cudaMemsetAsync(I.fm1, 0, sizeof(double) * 3 * C, s);
        cudaMemsetAsync(I.fm2, 0, sizeof(double) * C, s);
    } catch (const std::bad_alloc &) {
        cudaGetLastError();
        return fail(MESO_ERR_OOM, "device allocation failed for the FP32 state");
    }
    c->f32 = I;
    // the plain-state macro pointers alias the FP32 instance so the shared read-back paths work
    c->ps.rho = I.rho;
    c->ps.u = I.u;
    c->ps.T = I.T;
    c->ps.q = I.q;
    c->ps.fm0 = I.fm0;
    c->ps.fm1 = I.fm1;
    c->ps.fm2 = I.fm2;
    std::vector<meso::F32Inst> one(1, I);
    if (build_fp32_launch(one, c->num_sms, c->fs, c->fs_owned)) return fail(MESO_ERR_OOM, "launch state allocation failed");
    if (meso::fp32_prepare(c->fs, s)) return fail(MESO_ERR_CUDA, "FP32 set-up kernel failed");
    cudaStreamSynchronize(s);
    return MESO_OK;
}

int build_fp32_launch(const std::vector<meso::F32Inst> &insts, int num_sms, meso::Fp32State &s,
                      std::vector<void *> &owned) {
    const int n = (int)insts.size();
    std::vector<int> foff(1, 0), coff(1, 0), boff(1, 0);
    for (int i = 0; i < n; ++i) {
        const auto &I = insts[i];
        foff.push_back(foff.back() + I.F);
        coff.push_back(coff.back() + I.C);
        boff.push_back(boff.back() + I.nb);
    }
    // Work items: the instances' tile pieces, one launch for instances with two velocities per
    // lane and one for those with one.  A launch of a single split instance gives each CTA the
    // pieces of its run; otherwise the pieces go, most chunks first, to the least-loaded CTA.  The
    // results depend only on the pieces (each writes its own heat-flux partial row), not on the
    // CTA that runs them.
    std::vector<int4> items;
    std::vector<int> off;
    int grids[2] = {0, 0};
    for (int k = 0; k < 2; ++k) {
        const int vpl = 2 - k;
        std::vector<std::pair<int, TilePiece>> ps;
        int ninst_k = 0, only = -1;
        for (int i = 0; i < n; ++i) {
            const auto &I = insts[i];
            if (I.vpl != vpl) continue;
            ++ninst_k;
            only = i;
            for (const TilePiece &p : tile_pieces(I.ntile, I.chunks, I.ngroup, I.split)) ps.push_back({i, p});
        }
        std::vector<std::vector<int>> lists;
        if (ninst_k == 1 && insts[only].split > 0 && insts[only].split <= num_sms) {
            for (int j = 0; j < (int)ps.size(); ++j) {
                const int r = ps[j].second.run;
                if (r >= (int)lists.size()) lists.resize(r + 1);
                lists[r].push_back(j);
            }
        } else if (!ps.empty()) {
            std::vector<int> order(ps.size());
            for (int j = 0; j < (int)ps.size(); ++j) order[j] = j;
            auto cost = [&](int j) { return ps[j].second.ch1 - ps[j].second.ch0; };
            std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost(a) > cost(b); });
            lists.resize(std::min((int)ps.size(), std::max(1, num_sms)));
            std::priority_queue<std::pair<long, int>, std::vector<std::pair<long, int>>, std::greater<>> load;
            for (int cta = 0; cta < (int)lists.size(); ++cta) load.push({0, cta});
            for (int j : order) {
                auto [l, cta] = load.top();
                load.pop();
                lists[cta].push_back(j);
                load.push({l + cost(j), cta});
            }
        }
        for (const auto &L : lists) {
            off.push_back((int)items.size());
            for (int j : L) {
                const TilePiece &p = ps[j].second;
                items.push_back(make_int4(ps[j].first, p.tile, p.grp, p.ch0 | (p.ch1 << 16)));
            }
        }
        off.push_back((int)items.size());
        grids[k] = (int)lists.size();
    }
    // boundary faces: one block per face for large velocity sets, eight faces (a warp each) per
    // block for small ones
    std::vector<int2> bblocks, bblk;
    for (int i = 0; i < n; ++i) {
        const auto &I = insts[i];
        if (I.NVp <= meso::F32_SMALL_NVP) s.has_small = 1;
        else s.has_large = 1;
        if (I.NVp <= meso::F32_SMALL_NVP)
            for (int b = 0; b < I.nb; b += meso::F32_BND_FACES_PER_BLOCK) bblocks.push_back(make_int2(i, -b - 1));
        else
            for (int b = 0; b < I.nb; ++b) bblk.push_back(make_int2(i, b));
    }
    const int nbw = (int)bblocks.size();
    bblocks.insert(bblocks.end(), bblk.begin(), bblk.end());
    auto put = [&](const void *src, size_t bytes) -> void * {
        void *p = nullptr;
        if (cudaMalloc(&p, bytes ? bytes : 1) != cudaSuccess) return nullptr;
        owned.push_back(p);
        cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice);
        return p;
    };
    s.d_inst = (meso::F32Inst *)put(insts.data(), sizeof(meso::F32Inst) * n);
    s.d_items = (int4 *)put(items.data(), sizeof(int4) * items.size());
    s.d_item_off = (int *)put(off.data(), sizeof(int) * off.size());
    s.d_face_items = (int *)put(foff.data(), sizeof(int) * foff.size());
    s.d_cell_items = (int *)put(coff.data(), sizeof(int) * coff.size());
    s.d_bnd_items = (int *)put(boff.data(), sizeof(int) * boff.size());
    s.d_bnd_blocks = (int2 *)put(bblocks.data(), sizeof(int2) * bblocks.size());
    if (!s.d_inst || !s.d_items || !s.d_item_off || !s.d_face_items || !s.d_cell_items || !s.d_bnd_items || !s.d_bnd_blocks)
        return -1;
    s.nbnd_blocks = (int)bblocks.size();
    s.nbnd_warp = nbw;
    s.ninst = n;
    s.nitems = (int)items.size();
    s.grid2 = grids[0];
    s.grid1 = grids[1];
    s.total_faces = foff.back();
    s.total_cells = coff.back();
    s.total_bnd = boff.back();
    s.num_sms = num_sms;
    s.enabled = 1;
    return 0;
}

void free_fp32_launch(meso::Fp32State &s, std::vector<void *> &owned) {
    for (void *p : owned) cudaFree(p);
    owned.clear();
    s = meso::Fp32State();
}

}  // namespace meso_host
