// Host-visible interface of the FP32-storage Shakhov step (fp32_step.cu).
//
// One solve is an F32Inst: device pointers to its tile plan, geometry,
// velocity set and state.  The phase kernels take an array of instances and
// a work list of (instance, tile, velocity group) items, so one launch
// serves one solve or a whole batch of solves of different sizes.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "device_common.cuh"

namespace meso {

// Kernel limits (the tile planner shrinks tiles until every tile fits).
constexpr int F32_MAX_VPL = 2;      // velocities per lane (a chunk is 32 x VPL velocities)
constexpr int F32_MAX_SLOTS = 104;  // tile + 1-ring + (part of the) 2-ring halo cells
constexpr int F32_MAX_GSLOTS = 72;  // slots with a gradient (tile + 1-ring cells owned faces reconstruct from)
constexpr int F32_MAX_GENT = 400;   // gradient stencil entries per tile
constexpr int F32_MAX_OWNED = 112;  // faces owned by a tile
constexpr int F32_MAX_CELLS = 48;   // cells per tile
constexpr int F32_DEFAULT_CELLS = 48;  // tile size without an autotuned shape (three cells per warp)
constexpr int F32_MAX_CF = 200;     // cell-face entries per tile (tile cells x faces per cell)
constexpr int F32_MAX_TF = 120;     // faces touching a tile cell (< 128: indices fit 7 bits)
constexpr int F32_NMOM = 11;        // raw face moments about the reference velocity (2-D)
constexpr int F32_SMALL_NVP = 2048;  // velocity sets up to this size: a warp per boundary face, float-float face sums

// Scalars of one Shakhov equilibrium (rho, u, T, q) for FP32 evaluation of its
// deviation from the instance's reference Maxwellian g0 (see F32Inst::g0_32):
//   g_M / g0 = exp(E),  E = ea |xi|^2 + ebx xi_x + eby xi_y + ec,
//   ea = 1/(2 R T0) - 1/(2 R T),  eb = u / (R T),  ec = ln(rho T0 / (rho0 T)) - |u|^2 / (2 R T),
// so that E, and with it g_M - g0 = g0 expm1(E), carries the rounding of the
// deviation only.
struct EqP {
    float ux, uy;
    float qgx, qgy;  // q (1 - Pr) / (5 p R T): the Shakhov factor of g folded into q
    float ea, ebx, eby, ec;
    float RT;     // R T: the h factor over the g factor
    float iRT;    // 1 / (R T)
    float iRTk3;  // (K + 1) / (R T)
    float hm;     // (K + 3 - D) R T
    float dhm;    // (K + 3 - D) R (T - T0)
};

// Residual check state of one instance (the reference's Res[...] print list and converge counter,
// cdugks_shakhov.cpp:729-757), kept on the device.
struct F32Resid {
    double res[8];        // last residuals: rho, T, u (D components), q (D components)
    int nres;
    int converge_state;   // consecutive checks at or below the limit
    int converged;        // 1 once converge_state reached 10 (the instance is then halted)
    int checks;
};

// Face equilibrium and blend weights.
struct FaceK {
    EqP e;
    float Cs, oCs, pad0;
};

// Per-cell evolution constants: equilibria at states n and n+1 (the latter with q at n,
// cdugks_shakhov.cpp:684) and the evolution coefficients.
struct CellK {
    EqP en, e1;
    float cm, C, Cs, hdt_tau, hdt_taun, dt_v;
};

struct F32Inst {
    int C, F, NV, NVp, nb, ntile, ngroup, chunks;  // chunks = NVp / (32 vpl)
    int vpl;                                       // velocities per lane: 1 or 2
    int split;  // > 0: the tiles' velocity chunks, tile after tile, cut into `split` equal runs (one
                // per persistent CTA); 0: each tile's chunks in ngroup equal groups
    // physics
    double dt, hdt, R, Pr, mu0, vhs, T0, Kd, Cv, gamma, rho0;
    float hdt32, k3_32, twoK32;  // FP32 copies of dt/2, K + 1 and 2K for the velocity loops
    double iR, iT0, iCv, iRT0, irho0;  // reciprocals of R, T0, Cv, R T0, rho0 (FP64 divisions are slow)
    // reference Maxwellian g0 (rho0, u = 0, T0) and h0 = hm0 g0: the state holds g - g0, h - h0
    double hm0;
    double gmom[10];  // sum w g0 xi^a over the velocity set: 1, x, y, xx, xy, yy, xxx, xxy, xyy, yyy
    int gradient;
    // residual check and convergence counter of do_step, on the device (k32_residual)
    int res_interval, res_fields;
    double res_limit, total_volume;
    // tile plan
    const int *tile_cstart, *tile_ncell, *tile_slot_ptr, *slot_cell, *tile_gslots, *tile_gsp_off, *gs_ptr;
    const uint16_t *gs_nbr;
    const float *gs_ax, *gs_ay;
    const int *tile_fstart;
    const uint16_t *face_own_slot, *face_nei_slot;
    const int *tile_tf_ptr, *tf_face;
    const uint8_t *cf_tf;
    // mesh (renumbered)
    const int *cf_ptr, *cf_face, *fown, *fnei, *fbnd, *bface, *fmark;
    const float2 *fn32, *fdo, *fdn;
    const double2 *fn64;
    const float *farea;
    const double *vol, *farea64, *fn64raw;
    const meso_mark_desc *marks;
    const uint8_t *mask;
    const int *cn_ptr, *cn_cell;
    const double *lsq_dr;
    // velocities (padded to NVp with zero weight)
    const float *xi32x, *xi32y, *w32;
    const double *xi64x, *xi64y, *w64;
    const float *g0_32;    // [NVp] reference Maxwellian (0 on padding)
    const float4 *vt32;    // [NVp] (xi_x, xi_y, w, g0) packed for one 16-byte load
    const double *g0_64;
    const int *sym;
    uint2 *fcls;           // [chunks][F][vpl] upwind masks of each face (fp32_prepare)
    // state and work buffers
    float2 *S[2];          // [C][NVp] (g - g0, h - h0) ping-pong; S[status->step & 1] is current
    float2 *u32;           // [C] cell velocity (FP32) = reference velocity of the face moments
    FaceK *fk;             // [F]
    float2 *fmom;          // [F][11] raw face moments of the reconstruction (deviation part), float pairs
    double *fmac;          // [F][8] rho, ux, uy, T, qx, qy, Cs, tau
    double *fgbar;         // [F][4] fluxes of the reconstructed values (mass, mom x, mom y, energy) per unit area along n0
    double *fsum;          // [F][4] same for the face equilibrium (interior) or the final boundary values
    double *g0flux;        // [F][4] fluxes of the reference pair along n0 (static, fp32_prepare)
    float2 *bnd_in, *bnd_out;  // [nb][NVp]
    float2 *fbar;              // [F][NVp] reconstructed interior face values (moments -> update kernel)
    double *bnd_g0;            // [nb][2] half-range sums of g0 (fp32_prepare)
    CellK *ck;             // [C]
    float4 *qpart;         // [ngroup][C] heat-flux partials (qx, qy) as float pairs
    double *rho, *u, *T, *q;   // [C], [3C], [C], [3C]
    double *fm0, *fm1, *fm2;   // flux moments
    int *repair_list;
    DStatus *status;
    F32Resid *resid;           // residual state (device)
    double *rho_old, *u_old, *T_old, *q_old;  // macros at the last residual check
    // defect correction (null when off): added to each step's FP32 results so that the step
    // reproduces the FP64 step at the state it was last measured on (fp32_refine)
    float2 *corrS;         // [C][NVp] stored state (g - g0, h - h0)
    double *corrW;         // [C][4] rho, rho ux, rho uy, rho E after the conservative update
    double *corrq;         // [C][2] heat flux
    float2 *corrR;         // [C][NVp] on a measuring step: the rounding residual of each stored value
};

// Boundary faces of small velocity sets per boundary-kernel block (a warp each).
constexpr int F32_BND_FACES_PER_BLOCK = 8;

// Host-side handle of one or more instances sharing the phase launches.
struct Fp32State {
    int enabled = 0;
    int ninst = 0;
    F32Inst *d_inst = nullptr;   // device copy of the instance array
    int4 *d_items = nullptr;     // (inst, tile, group, ch0 | ch1 << 16) work items, grouped by CTA
    int *d_item_off = nullptr;   // CTA c of the vpl == 2 launch runs items [off[c], off[c + 1]),
                                 // CTA c of the vpl == 1 launch items [off[grid2 + 1 + c], ...)
    int nitems = 0;
    int grid2 = 0, grid1 = 0;    // CTAs of the two tile launches (instances with vpl 2 / 1)
    int *d_face_items = nullptr; // prefix sums of faces / cells / boundary faces over instances
    int *d_cell_items = nullptr;
    int *d_bnd_items = nullptr;
    int2 *d_bnd_blocks = nullptr; // boundary-kernel blocks: (inst, -(first of 8 faces) - 1), then (inst, face b)
    int nbnd_blocks = 0, nbnd_warp = 0;  // the first nbnd_warp items are warp-per-face items
    int has_small = 0, has_large = 0;  // instances with NVp <= / > F32_SMALL_NVP
    int total_faces = 0, total_cells = 0, total_bnd = 0;
    int num_sms = 0;
    int corr = 0;                // 1: the single instance carries defect corrections (corrS non-null);
                                 // 2: this step measures them (the state rounded to nearest, residuals kept)
};

int fp32_configure(int device);
constexpr int F32_NPHASE = 7;
extern const char *const kFp32Phases[F32_NPHASE];
// A second stream and two events with which the boundary kernel runs beside the face-equilibrium
// kernel (they depend on the same face macros and write disjoint faces).  Used when the step is
// captured as a graph, where the fork and join become graph edges.
struct StepFork {
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};
// One step of every instance; ev (may be null) receives F32_NPHASE + 1 events around the phases
// (the phases then run in order on `stream`); fork (may be null) runs the boundary kernel beside
// the face-equilibrium kernel.
int fp32_step(Fp32State &s, cudaStream_t stream, int64_t *launches, cudaEvent_t *ev = nullptr,
              const StepFork *fork = nullptr);
// Once per instance set-up, after the instances are on the device.
int fp32_prepare(const Fp32State &s, cudaStream_t stream);
int fp32_init(const Fp32State &s, int mode, cudaStream_t stream);

// Defect correction of a single 2-D Shakhov instance (I: its host copy; d_inst: the device copy).
// fp32_to_plain writes the current state and macros in the FP64 step's layout (f0 = g, f1 = h
// [C][NV], the 8C macro block rho); fp32_refine, called after one FP32 step from that state and
// one FP64 step from its copy, adds the FP64 step's results minus the FP32 step's to the
// corrections and replaces the FP32 step's results with the FP64 ones.
int fp32_to_plain(const F32Inst &I, const F32Inst *d_inst, double *f0, double *f1, double *mac, int sms,
                  cudaStream_t stream);
int fp32_refine(const F32Inst &I, const F32Inst *d_inst, const double *f0, const double *f1, const double *mac,
                int sms, cudaStream_t stream);

}  // namespace meso
