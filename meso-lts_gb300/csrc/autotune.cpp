// Kernel-shape autotuner for the FP32 step (include/meso_gpu.h, meso_autotune*).
//
// The FP32 tile kernels have three shape parameters: cells per tile (which
// sets the halo overhead, the shared-memory footprint and how evenly a tile's
// cells split over the 24 warps), velocities per lane (1 or 2: registers and
// shared memory against per-chunk overhead) and velocity groups per tile (how
// many CTAs share one tile's velocity range).  The best choice depends on the
// mesh and the velocity set, so it is measured: each candidate shape builds a
// context for the solve, runs a few steps from a uniform equilibrium and is
// timed with CUDA events; the fastest shape is returned and remembered for
// solves of the same size (cells, faces, velocities), which later contexts
// created with shape 0 then use.
//
// No counterpart in the reference (which has no GPU kernels to shape).
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "capi_internal.h"
#include "host/fp32_host.h"

using meso_host::fail;

namespace {

struct Shape {
    int tile_cells, vpl, ngroup;
};

std::mutex g_mu;
std::map<std::tuple<int, int, int>, Shape> g_cache;  // (cells, faces, velocities) -> best shape

std::vector<Shape> candidates(int nv, int ncell, int num_sms) {
    std::vector<Shape> out;
    const int vmax = nv >= 64 ? 2 : 1;
    for (int T : {24, 32, 40, 48})
        for (int v = 1; v <= vmax; ++v) {
            out.push_back({T, v, 0});  // the tiles' velocity chunks in equal runs, one per SM
            // equal velocity groups per tile instead, when the mesh has few tiles for the SM count
            const int tiles = (ncell + T - 1) / T;
            if (tiles < 2 * num_sms && nv >= 256) {
                const int chunks = (nv + 32 * v - 1) / (32 * v);
                out.push_back({T, v, meso_host::default_ngroup(tiles, chunks, num_sms)});
            }
        }
    return out;
}

}  // namespace

namespace meso_host {
// Shape remembered for a solve of this size, if the autotuner measured one.
bool tuned_shape(int ncell, int nface, int nv, int &tile_cells, int &vpl, int &ngroup) {
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_cache.find(std::make_tuple(ncell, nface, nv));
    if (it == g_cache.end()) return false;
    tile_cells = it->second.tile_cells;
    vpl = it->second.vpl;
    ngroup = it->second.ngroup;
    return true;
}
}  // namespace meso_host

extern "C" {

int meso_autotune(const meso_mesh_desc *mesh, const meso_dvs_desc *dvs, const meso_mark_desc *marks, int32_t nmarks,
                  const meso_params *params, int32_t steps, meso_params *best, double *best_ms) {
    if (!mesh || !dvs || !params || !best) return fail(MESO_ERR_INVALID, "null argument");
    if (steps <= 0) return fail(MESO_ERR_INVALID, "steps must be > 0");
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev))
        return fail(MESO_ERR_CUDA, "no CUDA device");
    const int C = mesh->ncell;
    std::vector<double> rho(C, params->rho0 > 0.0 ? params->rho0 : 1.0), u(3 * (size_t)C, 0.0), T(C, params->T0);
    double best_t = 0.0;
    meso_params bp = *params;
    bool found = false;
    for (const Shape &sh : candidates(dvs->nv, C, sms)) {
        meso_params p = *params;
        p.precision = MESO_FP32;
        p.tile_cells = sh.tile_cells;
        p.vpl = sh.vpl;
        p.ngroup = sh.ngroup;
        p.residual_interval = 0;
        meso_ctx *c = nullptr;
        int rc = meso_ctx_create(mesh, dvs, marks, nmarks, &p, nullptr, &c);
        if (rc == MESO_ERR_UNSUPPORTED) continue;  // the mesh does not fit this tile size
        if (rc) return rc;
        int32_t done = 0;
        rc = meso_init_macros(c, rho.data(), u.data(), T.data(), nullptr, 0);
        if (!rc) rc = meso_step(c, 2, &done);
        if (!rc) rc = meso_step(c, steps, &done);
        const double ms = meso_last_step_ms(c) / steps;
        meso_ctx_destroy(c);
        if (rc) return rc;
        if (!found || ms < best_t) {
            best_t = ms;
            bp = p;
            found = true;
        }
    }
    if (!found) return fail(MESO_ERR_UNSUPPORTED, "no FP32 kernel shape fits this mesh");
    bp.precision = params->precision;
    bp.residual_interval = params->residual_interval;
    *best = bp;
    if (best_ms) *best_ms = best_t;
    std::lock_guard<std::mutex> lock(g_mu);
    g_cache[std::make_tuple(mesh->ncell, mesh->nface, dvs->nv)] = {bp.tile_cells, bp.vpl, bp.ngroup};
    return MESO_OK;
}

int meso_autotune_case(const char *case_file, int32_t steps, meso_params *best, double *best_ms) {
    meso_case *k = nullptr;
    int rc = meso_case_load(case_file, &k);
    if (rc) return rc;
    meso_mesh_desc m;
    meso_dvs_desc d;
    const meso_mark_desc *marks = nullptr;
    int32_t nmarks = 0;
    meso_params p;
    meso_case_mesh(k, &m);
    meso_case_dvs(k, &d);
    meso_case_marks(k, &marks, &nmarks);
    meso_case_params(k, &p);
    rc = meso_autotune(&m, &d, marks, nmarks, &p, steps, best, best_ms);
    meso_case_free(k);
    return rc;
}

void meso_autotune_forget(void) {
    std::lock_guard<std::mutex> lock(g_mu);
    g_cache.clear();
}

}  // extern "C"
