// FP32-storage Shakhov CDUGKS step (2-D), tiled and fused.
//
// Storage: g - g0, h - h0 (deviations from a reference Maxwellian) interleaved
// as float2, velocity-contiguous per cell ([cell][NVp], NVp = NV rounded up to
// 32 VPL), two buffers (state n, n+1).  VPL (velocities per lane) is 2 for
// velocity sets of 256 and more, 1 below: a chunk is 32 VPL velocities, lane l
// of a warp handles velocities chunk*32*VPL + v*32 + l, v < VPL.  Velocity sets
// up to NVp = 2048 are "small": their face kernels take 8 lanes per face and
// their boundary faces a warp each.
// A step is eleven launches (one more per face kernel when a batch mixes
// small and large velocity sets), each over all instances of a batch,
// replayed as one CUDA graph:
//
//   P1  k32_reconstruct  persistent CTAs of 24 warps (one per SM) over their own
//                        list of pieces (a tile and a range of its velocity
//                        chunks; whole tiles in rounds of one per CTA, the
//                        chunks of the tiles left cut into equal runs): the tile
//                        and its two-ring halo of one chunk of 32 VPL velocities
//                        double-buffered in shared memory (16-byte cp.async
//                        copies by all threads) with the owned faces' upwind
//                        masks, least-squares gradients of the tile and 1-ring
//                        cells once per chunk, and the half-step upwind
//                        reconstruction of each face the tile owns
//                        (cdugks_shakhov.cpp:223-276) stored to HBM (fbar, or
//                        bnd_in for boundary faces)
//   FMa k32_face_moments a warp (large sets) or 8 lanes (small sets) per face:
//                        11 raw moments about a reference velocity of the
//                        stored reconstruction (FP32 terms, compensated; FP64 or
//                        float-float cross-lane sums)
//       k32_face_macros  one thread per face, FP64: face rho, u, T, tau, q
//                        (cdugks_shakhov.cpp:341-349) and the moment fluxes of
//                        the reconstruction, by exact algebra on the moments
//   FMb k32_face_eqflux  a warp (large sets) or 8 lanes (small sets) per
//                        interior face: discrete moment fluxes of the face
//                        Shakhov equilibrium, and the face's flux value
//                        (n0.xi) A (blend of the reconstruction and the
//                        equilibrium) stored in place
//   BND k32_boundary     a block (large sets) or a warp (small sets) per
//                        boundary face: blend, diffuse-wall balance, inlets /
//                        outlets, symmetry, slip (cdugks_shakhov.cpp:364-607),
//                        moment fluxes, flux values
//   CM  k32_cell_macros  one thread per cell, FP64: flux moments from the face
//                        fluxes, conservative update, tau, evolution constants
//                        (cdugks_shakhov.cpp:636-668), NaN / T<0 monitor
//   P2  k32_update       the same CTAs and pieces: the tile's cells and
//                        the flux values of every face touching them, one chunk
//                        at a time; per cell and velocity the signed sum of its
//                        faces' flux values, evolution to f-bar-plus, heat-flux
//                        partials, one row per piece of the tile
//                        (cdugks_shakhov.cpp:616-696)
//   QR  k32_heat_flux    q = sum of the heat-flux partials (FP64); then the mask
//                        repair, the end-of-step counter and the residual check
//                        with the convergence counter (k32_residual)
//
// The state is read twice and written once per step; each face's values are
// written once (reconstruction), read and rewritten once (flux value) and read
// by the one or two tiles whose cells it bounds.  Upwind classification is
// exact: static per-face masks record the class of every velocity from n.xi in
// FP64 in the reference's order (k32_cls_setup).  Per-face and per-cell scalar
// work runs one thread per face / cell in FP64, sharing reciprocals: FP64 runs
// at a small fraction of the FP32 rate on this GPU, so the velocity loops and
// the cross-lane sums stay in FP32 (compensated, float-float where needed).
#include <cfloat>
#include <cstddef>
#include <climits>

#include "fp32_step.h"

namespace meso {
namespace {

constexpr int kRW = 24;       // warps of the reconstruction kernel
constexpr int kT = kRW * 32;
// Both tile kernels run 24 warps in their one CTA per SM (the register budget is then 85 per
// thread); the update kernel's warps take two cells of a 48-cell tile each.
constexpr int kUW = 24, kUT = kUW * 32;
constexpr int kSmallFaceLanes = 8;  // lanes per face in the moments of small velocity sets
constexpr double kLOG2E = 1.4426950408889634;

__device__ __forceinline__ float fast_ex2(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Upwind class of velocity p at face f from the static masks (k32_cls_setup): 0 from the owner
// (n0.xi >= VSMALL), 1 from the neighbour (< -VSMALL), 2 between (cdugks_shakhov.cpp:223-276).
__device__ __forceinline__ int cls_bits(uint2 m, int lane) {
    return ((m.x >> lane) & 1u) ? 0 : (((m.y >> lane) & 1u) ? 1 : 2);
}
__device__ __forceinline__ int cls_of(const F32Inst &I, int f, int p) {
    const int w = p >> 5;
    const int ch = I.vpl == 2 ? w >> 1 : w, v = w - ch * I.vpl;
    return cls_bits(I.fcls[((size_t)ch * I.F + f) * I.vpl + v], p & 31);
}

// exp(x) - 1 in FP32 with a small relative error near 0: the Taylor series of
// exp through x^8 for |x| < 1/2 (truncation below 1.1e-8 relative), exp(x) - 1
// from ex2.approx beyond (|exp(x) - 1| > 0.39 there).  Branch-free.
__device__ __forceinline__ float expm1_dev(float x) {
    float p = fmaf(x, 1.f / 40320.f, 1.f / 5040.f);
    p = fmaf(x, p, 1.f / 720.f);
    p = fmaf(x, p, 1.f / 120.f);
    p = fmaf(x, p, 1.f / 24.f);
    p = fmaf(x, p, 1.f / 6.f);
    p = fmaf(x, p, 0.5f);
    p = fmaf(x, p, 1.f);
    const float series = x * p;
    const float direct = fast_ex2(x * (float)kLOG2E) - 1.f;
    return fabsf(x) < 0.5f ? series : direct;
}

// 32 random bits from three keys (a multiply-xorshift mix): the draws of stochastic rounding.
__device__ __forceinline__ unsigned mix3(unsigned a, unsigned b, unsigned c) {
    unsigned h = a ^ b ^ c;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    h *= 0x297A2D39u;
    h ^= h >> 15;
    return h;
}
// x + r stochastically rounded to FP32 (x the value rounded to nearest, r its residual, |r| at
// most half a unit in the last place): x + r plus a dither uniform over one unit in the last place
// of x, rounded to nearest, rounds up with probability equal to the distance from the float below
// (16 random bits).  Zero, subnormal and non-finite x come back unchanged.
__device__ __forceinline__ float sr_round(float x, float r, unsigned bits16) {
    const unsigned e = __float_as_uint(x) & 0x7f800000u;
    if (e == 0u || e == 0x7f800000u) return x;
    const float ulp = __uint_as_float(e) * 1.1920928955078125e-7f;  // 2^(exponent - 23)
    const float u = __uint_as_float(0x3f800000u | (bits16 << 7)) - 1.5f;  // [-1/2, 1/2)
    return x + fmaf(u, ulp, r);
}

// Deviation of the Shakhov g, h (2-D, cdugks_shakhov.cpp:185-211) at one velocity
// from the reference pair (g0, hm0 g0):
//   g_M = g0 + dg_M,  dg_M = g0 expm1(E)
//   g_S - g0 = dg_M + g_M (1 - Pr) (c.q) / (5 p R T) (c^2 / RT - 4)
//   h_S - h0 = hm dg_M + dhm g0 + g_M (1 - Pr) (c.q) / (5 p) ((c^2 / RT - 2)(K + 1) - 2K)
// dshakhov_c takes the peculiar velocity c = xi - u (cx, cy, cc = |c|^2); dshakhov forms it.
__device__ __forceinline__ float2 dshakhov_c(const EqP &e, float xx, float xy, float xi2, float g0, float cx, float cy,
                                             float cc, float k3, float twoK) {
    const float E = fmaf(e.ea, xi2, fmaf(e.ebx, xx, fmaf(e.eby, xy, e.ec)));
    const float dgm = g0 * expm1_dev(E);
    const float gm = g0 + dgm;
    const float a = gm * fmaf(cx, e.qgx, cy * e.qgy);  // g_M (1 - Pr) (c.q) / (5 p R T)
    const float dg = fmaf(a, fmaf(cc, e.iRT, -4.0f), dgm);
    // (c^2 / RT - 2)(K + 1) - 2K = c^2 (K + 1) / RT - 2 (K + 1) - 2K
    const float dh = fmaf(a * e.RT, fmaf(cc, e.iRTk3, fmaf(-2.0f, k3, -twoK)), fmaf(e.hm, dgm, e.dhm * g0));
    return make_float2(dg, dh);
}
__device__ __forceinline__ float2 dshakhov(const EqP &e, float xx, float xy, float xi2, float g0, float k3,
                                           float twoK) {
    const float cx = xx - e.ux, cy = xy - e.uy;
    return dshakhov_c(e, xx, xy, xi2, g0, cx, cy, fmaf(cx, cx, cy * cy), k3, twoK);
}

// EqP of (rho, u, T, q), from FP64 macros, given irho = 1 / rho and iRT = 1 / (R T): FP64 runs at
// a small fraction of the FP32 rate here, so the per-face and per-cell scalar work shares its
// reciprocals instead of dividing again.
__device__ __forceinline__ EqP make_eqp_r(const F32Inst &I, double rho, double irho, double ux, double uy, double T,
                                          double iRT, double qx, double qy) {
    const double RT = I.R * T, ip = irho * iRT, c1 = (1.0 - I.Pr) * 0.2;
    EqP e;
    e.ux = (float)ux;
    e.uy = (float)uy;
    const double sg = c1 * ip * iRT;  // (1 - Pr) / (5 p R T)
    e.qgx = (float)(sg * qx);
    e.qgy = (float)(sg * qy);
    e.ea = (float)(0.5 * (I.iRT0 - iRT));
    e.ebx = (float)(ux * iRT);
    e.eby = (float)(uy * iRT);
    // ln(rho T0 / (rho0 T)) from its argument's offset from 1 (formed in FP64) by the FP32 log1p:
    // its error is within the FP32 rounding the FP64 logarithm's result would get here
    e.ec = log1pf((float)(rho * I.irho0 * (I.T0 * I.R * iRT) - 1.0)) - (float)(0.5 * (ux * ux + uy * uy) * iRT);
    e.RT = (float)RT;
    e.iRT = (float)iRT;
    e.iRTk3 = (float)((I.Kd + 1.0) * iRT);
    e.hm = (float)((I.Kd + 1.0) * RT);
    e.dhm = (float)((I.Kd + 1.0) * I.R * (T - I.T0));
    return e;
}

__device__ __forceinline__ EqP make_eqp(const F32Inst &I, double rho, double ux, double uy, double T, double qx,
                                        double qy) {
    return make_eqp_r(I, rho, 1.0 / rho, ux, uy, T, 1.0 / (I.R * T), qx, qy);
}

// (T / T0)^omega: the square root for the common omega = 1/2.
__device__ __forceinline__ double vhs_pow(const F32Inst &I, double t_ratio) {
    return I.vhs == 0.5 ? sqrt(t_ratio) : pow(t_ratio, I.vhs);
}

// tau = mu0 (T / T0)^omega / (rho R T) (cdugks_shakhov.cpp:181-183) from the reciprocals of rho and T.
__device__ __forceinline__ double tau_r(const F32Inst &I, double irho, double T, double iT) {
    return I.mu0 * vhs_pow(I, T * I.iT0) * irho * iT * I.iR;
}

// The 11 raw moments of the reference pair about velocity (a, b), from the discrete
// moments of g0 (same order as the moments k32_face_macros accumulates).
__device__ __forceinline__ void g0_raw_moments(const F32Inst &I, double a, double b, double (&M)[F32_NMOM]) {
    const double *G = I.gmom;  // 1, x, y, xx, xy, yy, xxx, xxy, xyy, yyy
    const double g1 = G[0], gx = G[1], gy = G[2], gxx = G[3], gxy = G[4], gyy = G[5];
    const double gxxx = G[6], gxxy = G[7], gxyy = G[8], gyyy = G[9];
    M[0] = g1;
    M[1] = gx - a * g1;
    M[2] = gy - b * g1;
    M[3] = gxx - 2.0 * a * gx + a * a * g1;
    M[4] = gxy - a * gy - b * gx + a * b * g1;
    M[5] = gyy - 2.0 * b * gy + b * b * g1;
    const double cxxx = gxxx - 3.0 * a * gxx + 3.0 * a * a * gx - a * a * a * g1;
    const double cxyy = gxyy - a * gyy - 2.0 * b * gxy + 2.0 * a * b * gy + b * b * gx - a * b * b * g1;
    const double cyyy = gyyy - 3.0 * b * gyy + 3.0 * b * b * gy - b * b * b * g1;
    const double cxxy = gxxy - b * gxx - 2.0 * a * gxy + 2.0 * a * b * gx + a * a * gy - a * a * b * g1;
    M[6] = cxxx + cxyy;
    M[7] = cyyy + cxxy;
    M[8] = I.hm0 * g1;
    M[9] = I.hm0 * (gx - a * g1);
    M[10] = I.hm0 * (gy - b * g1);
}

// Fluxes of the reference pair along n (mass, momentum x, y, energy), full velocity set.
__device__ __forceinline__ void g0_fluxes(const F32Inst &I, double nx, double ny, double (&o)[4]) {
    const double *G = I.gmom;
    o[0] = nx * G[1] + ny * G[2];
    o[1] = nx * G[3] + ny * G[4];
    o[2] = nx * G[4] + ny * G[5];
    o[3] = nx * (G[6] + G[8]) + ny * (G[7] + G[9]) + I.hm0 * (nx * G[1] + ny * G[2]);
}

// Packed FP32 pairs (sm_100 and later): each is the two scalar operations, rounded alike, in one
// instruction; the (g, h) pairs of the step map onto them.
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }

__device__ __forceinline__ void kahan(float &s, float &c, float v) {
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
}

template <int N> __device__ __forceinline__ void warp_sum(float (&v)[N]) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int k = 0; k < N; ++k) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
}

// Sum over aligned groups of W lanes (W = 32: the warp) of per-lane values hi + lo (a compensated
// FP32 partial: hi = Kahan sum, lo = minus its compensation) as an unevaluated float pair: each xor
// level adds the partner's pair with Knuth's two-sum (exact rounding error of hi + hi') and
// renormalises, so the result carries about 44 significant bits (the pair's precision) at FP32
// instruction rates.  Every lane of a group receives the same, order-independent-of-lane value;
// the FP64 result is hi + lo.  All 32 lanes of the warp must call it.
template <int W = 32> __device__ __forceinline__ float2 warp_sum_ff2(float hi, float lo) {
#pragma unroll
    for (int o = W / 2; o > 0; o >>= 1) {
        const float bh = __shfl_xor_sync(0xffffffffu, hi, o), bl = __shfl_xor_sync(0xffffffffu, lo, o);
        const float sum = __fadd_rn(hi, bh);
        const float bv = __fsub_rn(sum, hi);
        const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(sum, bv)), __fsub_rn(bh, bv));
        const float l = __fadd_rn(__fadd_rn(lo, bl), err);
        hi = __fadd_rn(sum, l);
        lo = __fsub_rn(l, __fsub_rn(hi, sum));
    }
    return make_float2(hi, lo);
}
template <int W = 32> __device__ __forceinline__ double warp_sum_ff(float hi, float lo) {
    const float2 r = warp_sum_ff2<W>(hi, lo);
    return (double)r.x + (double)r.y;
}

// A double as an unevaluated float pair (hi + lo, about 48 significant bits), and back: FP64
// results that a warp holds in every lane are stored as pairs and combined by the one thread per
// face or cell that uses them.
__device__ __forceinline__ float2 split_ff(double v) {
    const float hi = (float)v;
    return make_float2(hi, (float)(v - (double)hi));
}
__device__ __forceinline__ double join_ff(float2 v) { return (double)v.x + (double)v.y; }

template <int N> __device__ __forceinline__ float pick(const float (&v)[N], int lane) {
    float r = 0.f;
#pragma unroll
    for (int k = 0; k < N; ++k) r = (lane == k) ? v[k] : r;
    return r;
}

// instance owning global index g, given prefix offsets off[0..n]
__device__ __forceinline__ int find_inst(const int *off, int n, int g) {
    int lo = 0, hi = n;
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (off[mid] <= g) lo = mid;
        else hi = mid;
    }
    return lo;
}

// ---- asynchronous global -> shared copies (cp.async, sm_80 and later) -------------
__device__ __forceinline__ unsigned smem_u32(const void *p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
// 16 bytes from global to shared, completing with the thread's current commit group.
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
// 8 bytes from global to shared (both 8-byte aligned).
__device__ __forceinline__ void cp_async8(void *dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// Waits until at most N of the thread's commit groups are still in flight.
template <int N> __device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

struct OwnedFace {     // P1: one face owned by the tile
    float2 fdo, fdn;   // face centre minus owner / neighbour centre
    int bnd, face;
    unsigned short os, ns;
    int pad;
};

template <int VPL> struct __align__(128) TileSmem {
    static constexpr int SEG = 32 * VPL;         // velocities of one slot in a chunk
    float2 phi[2][F32_MAX_SLOTS * SEG];         // double-buffered chunk of the tile + halo (cp.async target)
    float4 G[F32_MAX_GSLOTS * SEG];             // gradients (g_x, h_x, g_y, h_y) of tile + 1-ring cells
    float2 ga[F32_MAX_GENT];                    // gradient stencil coefficients
    int4 g4o[F32_MAX_GSLOTS];                   // slots with four stencil entries: neighbour offsets into phi
    float4 g4x[F32_MAX_GSLOTS], g4y[F32_MAX_GSLOTS];  // and their coefficients
    uint2 cls[2][F32_MAX_OWNED * VPL];          // upwind masks of the owned faces for the chunk (cp.async target)
    const uint2 *cls_src;                       // masks of chunk 0 of the tile's first owned face
    size_t cls_stride;                          // F * VPL: from one chunk's masks to the next
    int slot_cell[F32_MAX_SLOTS];
    unsigned short gnbr[F32_MAX_GENT];
    unsigned short gptr[F32_MAX_GSLOTS + 1];
    int nS, nG, nX, ncls;
    union {
        struct {
            OwnedFace of[F32_MAX_OWNED];
        } p1;

    } u;
};

template <int VPL> constexpr size_t tile_smem() { return sizeof(TileSmem<VPL>); }

// Shared memory of the update kernel: the tile's cells and the face values of every face touching
// them, one chunk at a time (no halo, no gradients: the moments kernel stored each face's
// reconstruction).
template <int VPL> struct __align__(128) UpdSmem {
    static constexpr int SEG = 32 * VPL;
    float2 phi[2][F32_MAX_CELLS * SEG];         // tile cells (cp.async target)
    float2 fv[2][F32_MAX_TF * SEG];             // (n0.xi) A f_face of each tile face (cp.async target)
    const float2 *src[F32_MAX_TF];              // where each tile face's flux values are, [NVp]
    CellK ck[F32_MAX_CELLS];
    int4 c4o[F32_MAX_CELLS];                    // cells with four faces: their faces' offsets into fv
    float4 c4s[F32_MAX_CELLS];                  // and signs (-1 where the cell is the face's neighbour)
    int cf_off[F32_MAX_CELLS + 1];
    unsigned char cft[F32_MAX_CF];              // per cell-face entry: tile face | 0x80 if the cell is its neighbour
    int nc, ntf, cs;
};
template <int VPL> constexpr size_t upd_smem() { return sizeof(UpdSmem<VPL>); }
static_assert(offsetof(UpdSmem<1>, fv) % 16 == 0 && offsetof(UpdSmem<2>, fv) % 16 == 0, "fv alignment");
static_assert(sizeof(UpdSmem<F32_MAX_VPL>) <= 227 * 1024, "update staging exceeds the shared memory of one CTA");
// cp.async destinations must be 16-byte aligned
static_assert(offsetof(TileSmem<1>, phi) % 16 == 0 && offsetof(TileSmem<2>, phi) % 16 == 0, "phi alignment");
static_assert(sizeof(TileSmem<F32_MAX_VPL>) <= 227 * 1024, "tile staging exceeds the shared memory of one CTA");

// Per-item staging of the slot list and the gradient stencil.
template <int VPL> __device__ __forceinline__ void stage_common(const F32Inst &I, int tile, TileSmem<VPL> &sm) {
    const int sbase = I.tile_slot_ptr[tile];
    const int nS = I.tile_slot_ptr[tile + 1] - sbase;
    const int nG = I.tile_gslots[tile];
    const int *gp = I.gs_ptr + I.tile_gsp_off[tile];
    const int e0 = gp[0];
    for (int s = threadIdx.x; s < nS; s += kT) sm.slot_cell[s] = I.slot_cell[sbase + s];
    for (int s = threadIdx.x; s <= nG; s += kT) sm.gptr[s] = (unsigned short)(gp[s] - e0);
    const int ne = gp[nG] - e0;
    for (int j = threadIdx.x; j < ne; j += kT) {
        sm.gnbr[j] = I.gs_nbr[e0 + j];
        sm.ga[j] = make_float2(I.gs_ax[e0 + j], I.gs_ay[e0 + j]);
    }
    constexpr int SEG = TileSmem<VPL>::SEG;
    for (int s = threadIdx.x; s < nG; s += kT) {  // four-entry stencils decoded once per item
        const int j = gp[s];
        if (gp[s + 1] - gp[s] != 4) continue;
        sm.g4o[s] = make_int4(I.gs_nbr[j] * SEG, I.gs_nbr[j + 1] * SEG, I.gs_nbr[j + 2] * SEG, I.gs_nbr[j + 3] * SEG);
        sm.g4x[s] = make_float4(I.gs_ax[j], I.gs_ax[j + 1], I.gs_ax[j + 2], I.gs_ax[j + 3]);
        sm.g4y[s] = make_float4(I.gs_ay[j], I.gs_ay[j + 1], I.gs_ay[j + 2], I.gs_ay[j + 3]);
    }
    if (threadIdx.x == 0) {
        sm.nS = nS;
        sm.nG = nG;
    }
}

// Every thread issues 16-byte asynchronous copies of chunk `ch` (32 VPL velocities of every slot)
// into phi[buf]; a warp instruction covers 512 contiguous bytes of one or two slots.  One commit
// group per chunk.  Spreading the copies over all threads keeps any one warp from stalling on them.
template <int VPL>
__device__ __forceinline__ void load_chunk(const float2 *S, int NVp, int ch, int buf, TileSmem<VPL> &sm) {
    constexpr int SEG = TileSmem<VPL>::SEG;
    constexpr int PER = SEG / 2;  // 16-byte pieces of one slot's segment
    const int n = sm.nS * PER;
    for (int i = threadIdx.x; i < n; i += kT) {
        const int s = i / PER, k = i - s * PER;
        cp_async16(&sm.phi[buf][s * SEG + 2 * k], S + (size_t)sm.slot_cell[s] * NVp + (size_t)ch * SEG + 2 * k);
    }
    const uint2 *cs = sm.cls_src + (size_t)ch * sm.cls_stride;
    for (int i = threadIdx.x; i < sm.ncls; i += kT) cp_async8(&sm.cls[buf][i], cs + i);
    cp_async_commit();
}

// Makes chunk `ch` (issued one iteration earlier) visible to the CTA; the barrier also certifies
// that every warp has finished the previous iteration, which read the other buffer and the
// gradients, so the copies of chunk ch + 1 go into that buffer right after it.
template <int VPL>
__device__ __forceinline__ void next_chunk(const float2 *S, int NVp, int ch, int ch1, int buf, TileSmem<VPL> &sm) {
    cp_async_wait<0>();
    __syncthreads();
    if (ch + 1 < ch1) load_chunk<VPL>(S, NVp, ch + 1, buf ^ 1, sm);
}

// Gradients of the first nG slots from phi[buf].
// Gradients of the first nG slots from phi[buf], stored as (dg/dx, dh/dx, dg/dy, dh/dy).
template <int VPL> __device__ __forceinline__ void gradients(TileSmem<VPL> &sm, int buf, int gradient_on) {
    constexpr int SEG = TileSmem<VPL>::SEG;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nG = sm.nG;
    const float2 *phi = sm.phi[buf];
    for (int s = warp; s < nG; s += kRW) {
        float2 gx[VPL], gy[VPL], c[VPL];  // (g, h) pairs
#pragma unroll
        for (int v = 0; v < VPL; ++v) {
            gx[v] = gy[v] = make_float2(0.f, 0.f);
            c[v] = phi[s * SEG + v * 32 + lane];
        }
        if (gradient_on && sm.gptr[s + 1] - sm.gptr[s] == 4) {  // the same sums, entries in order
            const int4 o = sm.g4o[s];
            const float4 ax = sm.g4x[s], ay = sm.g4y[s];
            const int oo[4] = {o.x, o.y, o.z, o.w};
            const float aa[4][2] = {{ax.x, ay.x}, {ax.y, ay.y}, {ax.z, ay.z}, {ax.w, ay.w}};
            float2 x[4][VPL];
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int v = 0; v < VPL; ++v) x[q][v] = phi[oo[q] + lane + v * 32];
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int v = 0; v < VPL; ++v) {
                    const float2 d = sub2(x[q][v], c[v]);
                    gx[v] = fma2(f2(aa[q][0]), d, gx[v]);
                    gy[v] = fma2(f2(aa[q][1]), d, gy[v]);
                }
        } else if (gradient_on) {
            const int j0 = sm.gptr[s], j1 = sm.gptr[s + 1];
            int j = j0;
            for (; j + 4 <= j1; j += 4) {  // four stencil entries: all loads, then the sums in entry order
                float2 a[4], x[4][VPL];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int nb = sm.gnbr[j + q] * SEG + lane;
                    a[q] = sm.ga[j + q];
#pragma unroll
                    for (int v = 0; v < VPL; ++v) x[q][v] = phi[nb + v * 32];
                }
#pragma unroll
                for (int q = 0; q < 4; ++q)
#pragma unroll
                    for (int v = 0; v < VPL; ++v) {
                        const float2 d = sub2(x[q][v], c[v]);
                        gx[v] = fma2(f2(a[q].x), d, gx[v]);
                        gy[v] = fma2(f2(a[q].y), d, gy[v]);
                    }
            }
            for (; j < j1; ++j) {
                const int nb = sm.gnbr[j] * SEG + lane;
                const float2 a = sm.ga[j];
#pragma unroll
                for (int v = 0; v < VPL; ++v) {
                    const float2 d = sub2(phi[nb + v * 32], c[v]);
                    gx[v] = fma2(f2(a.x), d, gx[v]);
                    gy[v] = fma2(f2(a.y), d, gy[v]);
                }
            }
        }
#pragma unroll
        for (int v = 0; v < VPL; ++v) sm.G[s * SEG + v * 32 + lane] = make_float4(gx[v].x, gx[v].y, gy[v].x, gy[v].y);
    }
}

// Half-step reconstruction from slot s, velocity v of the lane: phi + (d - xi dt/2) . grad  (g and h)
template <int VPL>
__device__ __forceinline__ float2 recon(const TileSmem<VPL> &sm, int buf, int s, int v, float2 d, float hx, float hy) {
    constexpr int SEG = TileSmem<VPL>::SEG;
    const int k = s * SEG + v * 32 + (threadIdx.x & 31);
    const float2 x = sm.phi[buf][k];
    const float4 g = sm.G[k];  // (dg/dx, dh/dx, dg/dy, dh/dy)
    const float ax = d.x - hx, ay = d.y - hy;
    return fma2(f2(ax), make_float2(g.x, g.y), fma2(f2(ay), make_float2(g.z, g.w), x));
}

// The upwind side is selected per lane (slot and offset), so lanes of one warp that upwind from
// different sides of the face share one reconstruction; only the rare between-sides case (|n.xi|
// below VSMALL) evaluates the second side.
template <int VPL>
__device__ __forceinline__ float2 face_bar(const TileSmem<VPL> &sm, int buf, int v, int cls, int os, int ns,
                                           float2 fdo, float2 fdn, float hx, float hy) {
    const bool nb = cls == 1;
    const int s = nb ? ns : os;
    const float2 d = make_float2(nb ? fdn.x : fdo.x, nb ? fdn.y : fdo.y);
    float2 a = recon(sm, buf, s, v, d, hx, hy);
    if (cls == 2) {
        const float2 b = recon(sm, buf, ns, v, fdn, hx, hy);
        a = make_float2(0.5f * (a.x + b.x), 0.5f * (a.y + b.y));
    }
    return a;
}


// =============================================================================
// P1: upwind half-step reconstruction of every face (owned by a tile) into HBM
// =============================================================================
template <int VPL>
__global__ void __launch_bounds__(kT, 1) k32_reconstruct(const F32Inst *__restrict__ insts, const int4 *__restrict__ items,
                                                    const int *__restrict__ item_off) {
    constexpr int SEG = TileSmem<VPL>::SEG;
    extern __shared__ float4 smem_raw[];
    TileSmem<VPL> &sm = *reinterpret_cast<TileSmem<VPL> *>(smem_raw);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int it = item_off[blockIdx.x]; it < item_off[blockIdx.x + 1]; ++it) {
        const int4 item = items[it];  // (instance, tile, group, ch0 | ch1 << 16)
        const F32Inst &I = insts[item.x];
        if (step_stopped(I.status)) continue;
        const int cur = I.status->step & 1;  // S[step parity] holds the current state
        const int tile = item.y;
        const int fs = I.tile_fstart[tile], nOF = I.tile_fstart[tile + 1] - fs;
        const int ch0 = item.w & 0xffff, ch1 = item.w >> 16;
        if (ch0 >= ch1) continue;
        const float2 *__restrict__ S = I.S[cur];
        const int NVp = I.NVp;
        const float hdt = I.hdt32;
        const int grad_on = I.gradient;
        const float4 *__restrict__ vt32 = I.vt32;
        float2 *__restrict__ bnd_in = I.bnd_in;
        float2 *__restrict__ fbar = I.fbar;
        stage_common(I, tile, sm);
        if (threadIdx.x == 0) {
            sm.cls_src = I.fcls + (size_t)fs * VPL;
            sm.cls_stride = (size_t)I.F * VPL;
            sm.ncls = nOF * VPL;
        }
        for (int f = threadIdx.x; f < nOF; f += kT) {
            const int g = fs + f;
            OwnedFace o;
            o.fdo = I.fdo[g];
            o.fdn = I.fdn[g];
            o.bnd = I.fbnd[g];
            o.face = g;
            o.os = I.face_own_slot[g];
            o.ns = I.face_nei_slot[g];
            o.pad = 0;
            sm.u.p1.of[f] = o;
        }
        __syncthreads();
        load_chunk<VPL>(S, NVp, ch0, 0, sm);
        for (int ch = ch0; ch < ch1; ++ch) {
            const int buf = (ch - ch0) & 1;
            // the chunk's velocities first: their loads overlap the wait, the gradients and the barriers
            float2 xv[VPL];
            int p[VPL];
#pragma unroll
            for (int v = 0; v < VPL; ++v) {
                p[v] = ch * SEG + v * 32 + lane;
                xv[v] = *reinterpret_cast<const float2 *>(&vt32[p[v]]);
            }
            next_chunk<VPL>(S, NVp, ch, ch1, buf, sm);
            gradients(sm, buf, grad_on);
            __syncthreads();
            float hx[VPL], hy[VPL];
#pragma unroll
            for (int v = 0; v < VPL; ++v) {
                hx[v] = hdt * xv[v].x;
                hy[v] = hdt * xv[v].y;
            }
#pragma unroll 2
            for (int fl = warp; fl < nOF; fl += kRW) {
                const OwnedFace o = sm.u.p1.of[fl];
                if (o.bnd >= 0) {  // own = neighbour: every upwind choice gives the owner's reconstruction
                    float2 *dst = bnd_in + (size_t)o.bnd * NVp;
#pragma unroll
                    for (int v = 0; v < VPL; ++v) dst[p[v]] = recon(sm, buf, o.os, v, o.fdo, hx[v], hy[v]);
                } else {
                    float2 *dst = fbar + (size_t)o.face * NVp;
#pragma unroll
                    for (int v = 0; v < VPL; ++v) {
                        const int cls = cls_bits(sm.cls[buf][fl * VPL + v], lane);
                        dst[p[v]] = face_bar(sm, buf, v, cls, o.os, o.ns, o.fdo, o.fdn, hx[v], hy[v]);
                    }
                }
            }
        }
        __syncthreads();  // the next item restages the tile tables
    }
}

// =============================================================================
// P2: face values, flux, evolution, heat-flux partials
// =============================================================================
// Copies of chunk `ch` of the tile's cells and of its faces' values into buffer `buf`, 16 bytes per
// thread, one commit group.
template <int VPL>
__device__ __forceinline__ void load_upd_chunk(const float2 *S, int NVp, int ch, int buf, UpdSmem<VPL> &sm) {
    constexpr int SEG = UpdSmem<VPL>::SEG, PER = SEG / 2;
    const int nc = sm.nc, ntf = sm.ntf;
    for (int i = threadIdx.x; i < (nc + ntf) * PER; i += kUT) {
        const int s = i / PER, k = i - s * PER;
        if (s < nc)
            cp_async16(&sm.phi[buf][s * SEG + 2 * k], S + (size_t)(sm.cs + s) * NVp + (size_t)ch * SEG + 2 * k);
        else
            cp_async16(&sm.fv[buf][(s - nc) * SEG + 2 * k], sm.src[s - nc] + (size_t)ch * SEG + 2 * k);
    }
    cp_async_commit();
}

// MODE 0: plain.  MODE 1: the instance carries defect corrections; each stored value is the FP32
// result plus its correction, rounded stochastically (round to nearest would return the same value
// every step at a steady state and the corrected iteration would stall short of it).  MODE 2: a
// measuring step of the correction: the value rounded to nearest, its rounding residual kept in
// corrR, so that the correction is measured against the unrounded result.
template <int VPL, int MODE>
__global__ void __launch_bounds__(kUT, 1) k32_update(const F32Inst *__restrict__ insts, const int4 *__restrict__ items,
                                                   const int *__restrict__ item_off) {
    constexpr int SEG = UpdSmem<VPL>::SEG;
    extern __shared__ float4 smem_raw[];
    UpdSmem<VPL> &sm = *reinterpret_cast<UpdSmem<VPL> *>(smem_raw);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int it = item_off[blockIdx.x]; it < item_off[blockIdx.x + 1]; ++it) {
        const int4 item = items[it];  // (instance, tile, group, ch0 | ch1 << 16)
        const F32Inst &I = insts[item.x];
        if (step_stopped(I.status)) continue;
        const int cur = I.status->step & 1;  // S[step parity] holds the current state
        const int tile = item.y, grp = item.z;
        const int cs = I.tile_cstart[tile], nc = I.tile_ncell[tile];
        const int ch0 = item.w & 0xffff, ch1 = item.w >> 16;
        if (ch0 >= ch1) {  // a piece without chunks (a tile cut into fewer pieces than ngroup) adds nothing
            for (int c = threadIdx.x; c < nc; c += kUT) I.qpart[(size_t)grp * I.C + cs + c] = make_float4(0.f, 0.f, 0.f, 0.f);
            continue;
        }
        const float2 *__restrict__ S = I.S[cur];
        float2 *__restrict__ Sn = I.S[cur ^ 1];
        const int NVp = I.NVp;
        const float k3 = I.k3_32, twoK = I.twoK32;
        const float4 *__restrict__ vt32 = I.vt32;
        const int j0 = I.cf_ptr[cs];
        for (int c = threadIdx.x; c < nc; c += kUT) sm.ck[c] = I.ck[cs + c];
        for (int c = threadIdx.x; c <= nc; c += kUT) sm.cf_off[c] = I.cf_ptr[cs + c] - j0;
        const int ncf = I.cf_ptr[cs + nc] - j0;
        for (int e = threadIdx.x; e < ncf; e += kUT) sm.cft[e] = I.cf_tf[j0 + e];
        for (int c = threadIdx.x; c < nc; c += kUT) {  // four-face cells decoded once per item
            const int e0 = I.cf_ptr[cs + c] - j0;
            if (I.cf_ptr[cs + c + 1] - j0 - e0 != 4) continue;
            int o[4];
            float g[4];
            for (int q = 0; q < 4; ++q) {
                const unsigned char t = I.cf_tf[j0 + e0 + q];
                o[q] = (t & 0x7f) * SEG;
                g[q] = (t & 0x80) ? -1.f : 1.f;
            }
            sm.c4o[c] = make_int4(o[0], o[1], o[2], o[3]);
            sm.c4s[c] = make_float4(g[0], g[1], g[2], g[3]);
        }
        const int q0 = I.tile_tf_ptr[tile], ntf = I.tile_tf_ptr[tile + 1] - q0;
        for (int q = threadIdx.x; q < ntf; q += kUT) {
            const int f = I.tf_face[q0 + q], b = I.fbnd[f];
            sm.src[q] = b >= 0 ? I.bnd_out + (size_t)b * NVp : I.fbar + (size_t)f * NVp;
        }
        if (threadIdx.x == 0) {
            sm.nc = nc;
            sm.ntf = ntf;
            sm.cs = cs;
        }
        __syncthreads();
        // heat-flux partials of this warp's cells (cl = warp + 16 r): per lane, compensated, across chunks
        constexpr int RC = (F32_MAX_CELLS + kUW - 1) / kUW;
        float qs[RC][2], qc[RC][2];
#pragma unroll
        for (int r = 0; r < RC; ++r) qs[r][0] = qs[r][1] = qc[r][0] = qc[r][1] = 0.f;
        load_upd_chunk<VPL>(S, NVp, ch0, 0, sm);
        for (int ch = ch0; ch < ch1; ++ch) {
            const int buf = (ch - ch0) & 1;
            // the chunk's velocity table first: its loads overlap the wait and the barrier below
            float xx[VPL], xy[VPL], w[VPL], g0[VPL], x2[VPL];
            int p[VPL];
#pragma unroll
            for (int v = 0; v < VPL; ++v) {
                p[v] = ch * SEG + v * 32 + lane;
                const float4 t = vt32[p[v]];
                xx[v] = t.x;
                xy[v] = t.y;
                w[v] = t.z;
                g0[v] = t.w;
            }
            // chunk ch visible; every warp has finished chunk ch - 1, so its buffer takes chunk ch + 1
            cp_async_wait<0>();
            __syncthreads();
            if (ch + 1 < ch1) load_upd_chunk<VPL>(S, NVp, ch + 1, buf ^ 1, sm);
#pragma unroll
            for (int v = 0; v < VPL; ++v) x2[v] = fmaf(xx[v], xx[v], xy[v] * xy[v]);
#pragma unroll
            for (int r = 0; r < RC; ++r) {
                const int cl = warp + kUW * r;
                if (cl >= nc) break;
                float2 fl[VPL];  // (g, h) outward flux sums
#pragma unroll
                for (int v = 0; v < VPL; ++v) fl[v] = make_float2(0.f, 0.f);
                const int e0 = sm.cf_off[cl], e1 = sm.cf_off[cl + 1];
                if (e1 - e0 == 4) {  // outward flux of the cell (:616-629), the four faces in entry order
                    const int4 o = sm.c4o[cl];
                    const float4 g = sm.c4s[cl];
                    const float2 *ff = sm.fv[buf] + lane;
#pragma unroll
                    for (int v = 0; v < VPL; ++v) {
                        const float2 a = ff[o.x + v * 32], b = ff[o.y + v * 32], c = ff[o.z + v * 32],
                                     d = ff[o.w + v * 32];
                        fl[v] = fma2(f2(g.w), d, fma2(f2(g.z), c, fma2(f2(g.y), b, fma2(f2(g.x), a, fl[v]))));
                    }
                } else {
#pragma unroll 4
                    for (int e = e0; e < e1; ++e) {
                        const unsigned char t = sm.cft[e];
                        const float2 *ff = sm.fv[buf] + (t & 0x7f) * SEG + lane;
                        const float sgn = (t & 0x80) ? -1.f : 1.f;
#pragma unroll
                        for (int v = 0; v < VPL; ++v) fl[v] = fma2(f2(sgn), ff[v * 32], fl[v]);
                    }
                }
                const CellK k = sm.ck[cl];
                float qv[2] = {0.f, 0.f};
#pragma unroll
                for (int v = 0; v < VPL; ++v) {
                    const float2 old = sm.phi[buf][cl * SEG + v * 32 + lane];
                    // state n (cdugks_shakhov.cpp:673-680)
                    const float2 sn = dshakhov(k.en, xx[v], xy[v], x2[v], g0[v], k3, twoK);
                    const float2 gn = fma2(f2(k.cm), sub2(sn, old), old);
                    // state n+1 with q at n (:682-687)
                    const float cx = xx[v] - k.e1.ux, cy = xy[v] - k.e1.uy, cc = fmaf(cx, cx, cy * cy);
                    const float2 s1 = dshakhov_c(k.e1, xx[v], xy[v], x2[v], g0[v], cx, cy, cc, k3, twoK);
                    // evolution (:689-690): C (g^n + dt/2 g_S / tau + dt/2 (g_S^n - g^n) / tau^n - dt/V flux)
                    float2 e = fma2(f2(k.hdt_tau), s1, gn);
                    e = fma2(f2(k.hdt_taun), sub2(sn, gn), e);
                    e = fma2(f2(-k.dt_v), fl[v], e);
                    const float2 gh = mul2(f2(k.C), e);
                    const size_t at = (size_t)(cs + cl) * NVp + p[v];
                    if (MODE != 0) {
                        // C (...) + Cs (g_S - C (...)) + correction: the fused result, the residual of
                        // its rounding, the correction added with its error (|correction| is small)
                        const float2 d1 = sub2(s1, gh);
                        const float2 xs = fma2(f2(k.Cs), d1, gh);
                        const float2 rs = fma2(f2(k.Cs), d1, sub2(gh, xs));
                        const float2 cS = I.corrS[at];
                        const float2 y = add2(xs, cS);
                        const float2 r = add2(rs, sub2(cS, sub2(y, xs)));
                        if (MODE == 2) {
                            Sn[at] = y;
                            I.corrR[at] = r;
                        } else {
                            const unsigned hb = mix3((unsigned)(cs + cl) * 0x9E3779B1u,
                                                     (unsigned)p[v] * 0x85EBCA77u,
                                                     (unsigned)I.status->step * 0xC2B2AE3Du);
                            Sn[at] = make_float2(sr_round(y.x, r.x, hb & 0xffffu), sr_round(y.y, r.y, hb >> 16));
                        }
                    } else {
                        Sn[at] = fma2(f2(k.Cs), sub2(s1, gh), gh);
                    }
                    // heat-flux partial (:692)
                    const float hw = 0.5f * w[v] * fmaf(cc, gh.x, gh.y);
                    qv[0] = fmaf(hw, cx, qv[0]);
                    qv[1] = fmaf(hw, cy, qv[1]);
                }
                kahan(qs[r][0], qc[r][0], qv[0]);
                kahan(qs[r][1], qc[r][1], qv[1]);
            }
        }
#pragma unroll
        for (int r = 0; r < RC; ++r) {  // one float-float warp reduction per cell and item
            const int cl = warp + kUW * r;
            if (cl >= nc) break;
            const float2 q0 = warp_sum_ff2(qs[r][0], -qc[r][0]), q1 = warp_sum_ff2(qs[r][1], -qc[r][1]);
            if (lane == 0) I.qpart[(size_t)grp * I.C + cs + cl] = make_float4(q0.x, q0.y, q1.x, q1.y);
        }
        __syncthreads();
    }
}

// =============================================================================
// FMa: face moments from the stored reconstructions (one warp per face), face macros in FP64
// =============================================================================
// Two kernels, each launched over the faces of the instances of its class: large velocity sets
// (NVp > F32_SMALL_NVP: a warp per face, long streaming loops, blocks of NB velocities per lane,
// FP64 warp sums) and small ones (k32_face_moments_small: a group of L lanes per face, so the
// cross-lane sums, which dominate short faces, are shorter and shared by 32 / L faces).
template <int NB>
__global__ void __launch_bounds__(256) k32_face_moments(const F32Inst *__restrict__ insts, const int *__restrict__ foff,
                                                       int ninst, int total) {
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    for (int g = blockIdx.x * wpb + (threadIdx.x >> 5); g < total; g += gridDim.x * wpb) {
        const int i = find_inst(foff, ninst, g);
        const F32Inst &I = insts[i];
        if (step_stopped(I.status) || I.NVp <= F32_SMALL_NVP) continue;
        const int f = g - foff[i];
        const float2 uo = I.u32[I.fown[f]], un = I.u32[I.fnei[f]];
        const float u0xf = 0.5f * (uo.x + un.x), u0yf = 0.5f * (uo.y + un.y);
        // 11 raw moments about u0 of the face's reconstructed deviations (cdugks_shakhov.cpp:305-349):
        // FP32 terms summed over blocks of NB velocities per lane, compensated across blocks
        const int b = I.fbnd[f];
        const float2 *__restrict__ src = b >= 0 ? I.bnd_in + (size_t)b * I.NVp : I.fbar + (size_t)f * I.NVp;
        const float4 *__restrict__ vt32 = I.vt32;
        float s[F32_NMOM], c[F32_NMOM];
#pragma unroll
        for (int k = 0; k < F32_NMOM; ++k) s[k] = c[k] = 0.f;
        for (int p0 = 0; p0 < I.NVp; p0 += 32 * NB) {
            float4 tv[NB];
            float2 gv[NB];
#pragma unroll
            for (int j = 0; j < NB; ++j) {
                const int p = p0 + 32 * j + lane;
                tv[j] = p < I.NVp ? vt32[p] : make_float4(0.f, 0.f, 0.f, 0.f);
                gv[j] = p < I.NVp ? __ldcs(&src[p]) : make_float2(0.f, 0.f);  // read once: evict first
            }
            float m[F32_NMOM];
#pragma unroll
            for (int k = 0; k < F32_NMOM; ++k) m[k] = 0.f;
#pragma unroll
            for (int j = 0; j < NB; ++j) {
                const float c0x = tv[j].x - u0xf, c0y = tv[j].y - u0yf;
                const float wg = tv[j].z * gv[j].x, wh = tv[j].z * gv[j].y;
                const float cc = fmaf(c0x, c0x, c0y * c0y);
                const float a = c0x * wg, bb = c0y * wg;
                m[0] += wg;
                m[1] += a;
                m[2] += bb;
                m[3] = fmaf(c0x, a, m[3]);
                m[4] = fmaf(c0x, bb, m[4]);
                m[5] = fmaf(c0y, bb, m[5]);
                m[6] = fmaf(cc, a, m[6]);
                m[7] = fmaf(cc, bb, m[7]);
                m[8] += wh;
                m[9] = fmaf(c0x, wh, m[9]);
                m[10] = fmaf(c0y, wh, m[10]);
            }
#pragma unroll
            for (int k = 0; k < F32_NMOM; ++k) kahan(s[k], c[k], m[k]);
        }
        double M[F32_NMOM];
#pragma unroll
        for (int k = 0; k < F32_NMOM; ++k) {
            double v = (double)s[k] - (double)c[k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            M[k] = v;
        }
        if (lane < F32_NMOM) {
            double mine = M[0];
#pragma unroll
            for (int k = 1; k < F32_NMOM; ++k)
                if (lane == k) mine = M[k];
            I.fmom[(size_t)f * F32_NMOM + lane] = split_ff(mine);
        }
    }
}

// The moments of faces of small velocity sets: L lanes per face, 32 / L faces per warp, blocks of
// NB velocities per lane, float-float sums over the L lanes.  Lanes of a group whose face is past
// the end, stopped or of the other class accumulate nothing but still take part in the sums.
template <int NB, int L>
__global__ void __launch_bounds__(256) k32_face_moments_small(const F32Inst *__restrict__ insts,
                                                             const int *__restrict__ foff, int ninst, int total) {
    constexpr int FPW = 32 / L;
    const int lane = threadIdx.x & 31, sl = lane % L;
    const int wpb = blockDim.x >> 5;
    for (int g0 = (blockIdx.x * wpb + (threadIdx.x >> 5)) * FPW; g0 < total; g0 += gridDim.x * wpb * FPW) {
        const int g = g0 + lane / L;
        int i = 0, f = 0;
        bool on = g < total;
        if (on) {
            i = find_inst(foff, ninst, g);
            on = !step_stopped(insts[i].status) && insts[i].NVp <= F32_SMALL_NVP;
            f = g - foff[i];
        }
        float s[F32_NMOM], c[F32_NMOM];
#pragma unroll
        for (int k = 0; k < F32_NMOM; ++k) s[k] = c[k] = 0.f;
        if (on) {
            const F32Inst &I = insts[i];
            const float2 uo = I.u32[I.fown[f]], un = I.u32[I.fnei[f]];
            const float u0xf = 0.5f * (uo.x + un.x), u0yf = 0.5f * (uo.y + un.y);
            const int b = I.fbnd[f];
            const float2 *__restrict__ src = b >= 0 ? I.bnd_in + (size_t)b * I.NVp : I.fbar + (size_t)f * I.NVp;
            const float4 *__restrict__ vt32 = I.vt32;
            for (int p0 = 0; p0 < I.NVp; p0 += L * NB) {
                float4 tv[NB];
                float2 gv[NB];
#pragma unroll
                for (int j = 0; j < NB; ++j) {
                    const int p = p0 + L * j + sl;
                    tv[j] = p < I.NVp ? vt32[p] : make_float4(0.f, 0.f, 0.f, 0.f);
                    gv[j] = p < I.NVp ? __ldcs(&src[p]) : make_float2(0.f, 0.f);  // read once: evict first
                }
                float m[F32_NMOM];
#pragma unroll
                for (int k = 0; k < F32_NMOM; ++k) m[k] = 0.f;
#pragma unroll
                for (int j = 0; j < NB; ++j) {
                    const float c0x = tv[j].x - u0xf, c0y = tv[j].y - u0yf;
                    const float wg = tv[j].z * gv[j].x, wh = tv[j].z * gv[j].y;
                    const float cc = fmaf(c0x, c0x, c0y * c0y);
                    const float a = c0x * wg, bb = c0y * wg;
                    m[0] += wg;
                    m[1] += a;
                    m[2] += bb;
                    m[3] = fmaf(c0x, a, m[3]);
                    m[4] = fmaf(c0x, bb, m[4]);
                    m[5] = fmaf(c0y, bb, m[5]);
                    m[6] = fmaf(cc, a, m[6]);
                    m[7] = fmaf(cc, bb, m[7]);
                    m[8] += wh;
                    m[9] = fmaf(c0x, wh, m[9]);
                    m[10] = fmaf(c0y, wh, m[10]);
                }
#pragma unroll
                for (int k = 0; k < F32_NMOM; ++k) kahan(s[k], c[k], m[k]);
            }
        }
        float2 M[F32_NMOM];
#pragma unroll
        for (int k = 0; k < F32_NMOM; ++k) M[k] = warp_sum_ff2<L>(s[k], -c[k]);
        if (on) {
#pragma unroll
            for (int k0 = 0; k0 < F32_NMOM; k0 += L) {
                const int k = k0 + sl;
                float2 mine = make_float2(0.f, 0.f);
#pragma unroll
                for (int q = 0; q < F32_NMOM; ++q)
                    if (q == k) mine = M[q];
                if (k < F32_NMOM) insts[i].fmom[(size_t)f * F32_NMOM + k] = mine;
            }
        }
    }
}

// FP64 face macros from the moments (one thread per face)
__global__ void k32_face_macros(const F32Inst *__restrict__ insts, const int *__restrict__ foff, int ninst,
                                int total) {
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
        const int i = find_inst(foff, ninst, g);
        const F32Inst &I = insts[i];
        if (step_stopped(I.status)) continue;
        const int f = g - foff[i];
        const float2 uo = I.u32[I.fown[f]], un = I.u32[I.fnei[f]];
        const double u0x = (double)(0.5f * (uo.x + un.x)), u0y = (double)(0.5f * (uo.y + un.y));
        double M[F32_NMOM];
        for (int k = 0; k < F32_NMOM; ++k) M[k] = join_ff(I.fmom[(size_t)f * F32_NMOM + k]);
        {  // the reference pair's part of the moments, exactly in FP64
            double M0[F32_NMOM];
            g0_raw_moments(I, u0x, u0y, M0);
            for (int k = 0; k < F32_NMOM; ++k) M[k] += M0[k];
        }
        const double rho = M[0], irho = 1.0 / rho;
        const double dx = M[1] * irho, dy = M[2] * irho;
        const double ux = u0x + dx, uy = u0y + dy;
        const double trM = M[3] + M[5];
        const double dd = dx * dx + dy * dy;
        const double e2 = trM - rho * dd + M[8];  // sum w (|xi-u|^2 g + h)
        const double T = 0.5 * e2 * irho * I.iCv, iT = 1.0 / T;
        const double tau = tau_r(I, irho, T, iT);
        const double m3x = M[6] - 2.0 * (M[3] * dx + M[4] * dy) - dx * trM + 2.0 * dd * rho * dx + M[9] - dx * M[8];
        const double m3y = M[7] - 2.0 * (M[4] * dx + M[5] * dy) - dy * trM + 2.0 * dd * rho * dy + M[10] - dy * M[8];
        const double qs = tau / (2.0 * tau + I.hdt * I.Pr);
        const double qx = qs * m3x, qy = qs * m3y;
        const double Cs = I.hdt / (2.0 * tau + I.hdt);
        double *fm = I.fmac + (size_t)f * 8;
        fm[0] = rho;
        fm[1] = ux;
        fm[2] = uy;
        fm[3] = T;
        fm[4] = qx;
        fm[5] = qy;
        fm[6] = Cs;
        fm[7] = tau;
        FaceK k;
        k.e = make_eqp_r(I, rho, irho, ux, uy, T, iT * I.iR, qx, qy);
        k.Cs = (float)Cs;
        k.oCs = (float)(1.0 - Cs);
        k.pad0 = 0.f;
        I.fk[f] = k;
        // moment fluxes of the reconstructed values along n0 (per unit area)
        const double2 n = I.fn64[f];
        const double un0 = u0x * n.x + u0y * n.y;
        const double M1n = M[1] * n.x + M[2] * n.y;
        const double M2nx = M[3] * n.x + M[4] * n.y, M2ny = M[4] * n.x + M[5] * n.y;
        const double uu0 = u0x * u0x + u0y * u0y;
        double *fb = I.fgbar + (size_t)f * 4;
        fb[0] = un0 * M[0] + M1n;
        fb[1] = u0x * un0 * M[0] + u0x * M1n + un0 * M[1] + M2nx;
        fb[2] = u0y * un0 * M[0] + u0y * M1n + un0 * M[2] + M2ny;
        fb[3] = un0 * (uu0 * M[0] + 2.0 * (u0x * M[1] + u0y * M[2]) + trM) + uu0 * M1n +
                2.0 * (u0x * M2nx + u0y * M2ny) + (M[6] * n.x + M[7] * n.y) + un0 * M[8] + (M[9] * n.x + M[10] * n.y);
    }
}

// =============================================================================
// FMb: discrete moment fluxes of the face equilibrium (one warp per interior face)
// =============================================================================
// One block of 8 velocities per lane of one interior face (velocities p0 + L j + sl): the face's
// flux values (n0.xi) A (blend of the reconstruction and the equilibrium, cdugks_shakhov.cpp:350-361)
// written in place of the reconstruction for the update kernel, and the moment fluxes of the face
// equilibrium added to the lane's compensated partials.  The block's table entries and stored
// reconstructions are loaded before any is used.
template <int L>
__device__ __forceinline__ void eqflux_block(const FaceK &k, float2 n, float area, float k3, float twoK,
                                             const float4 *__restrict__ vt32, float2 *__restrict__ fb, int NVp,
                                             int p0, int sl, float (&s)[4], float (&c)[4]) {
    float b[4] = {0.f, 0.f, 0.f, 0.f};
    float4 tv[8];
    float2 gv[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int p = p0 + L * i + sl;
        if (p < NVp) {
            tv[i] = vt32[p];
            gv[i] = fb[p];
        }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int p = p0 + L * i + sl;
        if (p >= NVp) continue;
        const float4 t = tv[i];
        const float xx = t.x, xy = t.y, w = t.z;
        const float x2 = fmaf(xx, xx, xy * xy);
        const float2 gs = dshakhov(k.e, xx, xy, x2, t.w, k3, twoK);
        const float2 gb = gv[i];
        const float d = fmaf(n.x, xx, n.y * xy), knA = d * area;
        fb[p] = mul2(f2(knA), fma2(f2(k.oCs), gb, mul2(f2(k.Cs), gs)));
        const float wkn = w * d;
        const float a = wkn * gs.x;
        b[0] += a;
        b[1] = fmaf(a, xx, b[1]);
        b[2] = fmaf(a, xy, b[2]);
        b[3] = fmaf(wkn, fmaf(x2, gs.x, gs.y), b[3]);
    }
    for (int q = 0; q < 4; ++q) kahan(s[q], c[q], b[q]);
}

// Large velocity sets: a warp per interior face, plain FP32 sums over blocks of 8 velocities per
// lane, compensated across blocks, one FP32 warp sum per face.
__global__ void __launch_bounds__(256) k32_face_eqflux(const F32Inst *__restrict__ insts, const int *__restrict__ foff,
                                                      int ninst, int total) {
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    for (int g = blockIdx.x * wpb + (threadIdx.x >> 5); g < total; g += gridDim.x * wpb) {
        const int i = find_inst(foff, ninst, g);
        const F32Inst &I = insts[i];
        if (step_stopped(I.status) || I.NVp <= F32_SMALL_NVP) continue;
        const int f = g - foff[i];
        if (I.fbnd[f] >= 0) continue;
        const FaceK k = I.fk[f];
        float s[4] = {0.f, 0.f, 0.f, 0.f}, c[4] = {0.f, 0.f, 0.f, 0.f};
        float2 *__restrict__ fb = I.fbar + (size_t)f * I.NVp;
        for (int p0 = 0; p0 < I.NVp; p0 += 32 * 8)
            eqflux_block<32>(k, I.fn32[f], I.farea[f], I.k3_32, I.twoK32, I.vt32, fb, I.NVp, p0, lane, s, c);
        float v[4] = {s[0] - c[0], s[1] - c[1], s[2] - c[2], s[3] - c[3]};
        warp_sum(v);
        if (lane < 4) {
            const double *g0f = I.g0flux + (size_t)f * 4;
            I.fsum[(size_t)f * 4 + lane] = g0f[lane] + (double)pick(v, lane);
        }
    }
}

// Small velocity sets: L lanes per interior face, 32 / L faces per warp, sums over the L lanes.
// Lanes of a group without a face to do accumulate nothing but take part in the sums.
template <int L>
__global__ void __launch_bounds__(256) k32_face_eqflux_small(const F32Inst *__restrict__ insts,
                                                            const int *__restrict__ foff, int ninst, int total) {
    constexpr int FPW = 32 / L;
    const int lane = threadIdx.x & 31, sl = lane % L;
    const int wpb = blockDim.x >> 5;
    for (int g0 = (blockIdx.x * wpb + (threadIdx.x >> 5)) * FPW; g0 < total; g0 += gridDim.x * wpb * FPW) {
        const int g = g0 + lane / L;
        int i = 0, f = 0;
        bool on = g < total;
        if (on) {
            i = find_inst(foff, ninst, g);
            f = g - foff[i];
            on = !step_stopped(insts[i].status) && insts[i].NVp <= F32_SMALL_NVP && insts[i].fbnd[f] < 0;
        }
        float s[4] = {0.f, 0.f, 0.f, 0.f}, c[4] = {0.f, 0.f, 0.f, 0.f};
        if (on) {
            const F32Inst &I = insts[i];
            const FaceK k = I.fk[f];
            float2 *__restrict__ fb = I.fbar + (size_t)f * I.NVp;
            for (int p0 = 0; p0 < I.NVp; p0 += L * 8)
                eqflux_block<L>(k, I.fn32[f], I.farea[f], I.k3_32, I.twoK32, I.vt32, fb, I.NVp, p0, sl, s, c);
        }
        float v[4] = {s[0] - c[0], s[1] - c[1], s[2] - c[2], s[3] - c[3]};
#pragma unroll
        for (int o = L / 2; o > 0; o >>= 1)
#pragma unroll
            for (int q = 0; q < 4; ++q) v[q] += __shfl_xor_sync(0xffffffffu, v[q], o);
        if (on && sl < 4) {
            const double *g0f = insts[i].g0flux + (size_t)f * 4;
            insts[i].fsum[(size_t)f * 4 + sl] = g0f[sl] + (double)pick(v, sl);
        }
    }
}

// =============================================================================
// BND: boundary faces; cdugks_shakhov.cpp:364-607.  A group of TPF threads per face: the block
// (TPF = 256) for large velocity sets, one warp (TPF = 32, eight faces per block) for small ones.
// =============================================================================
__device__ __forceinline__ double block_sum(double v, double *sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double s = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += sh[k];
    __syncthreads();
    return s;
}

__device__ __forceinline__ double solve_pressure(double P0, double R, double T, double ux, double uy, double gamma) {
    const double Ma = sqrt(ux * ux + uy * uy) / sqrt(gamma * R * T);
    return P0 / pow(1.0 + (gamma - 1.0) / 2.0 * (Ma * Ma), gamma / (gamma - 1.0));
}

// Threads of a boundary block: one face (large velocity sets) or F32_BND_FACES_PER_BLOCK faces, a warp
// each (small sets; the host plans the blocks' first faces with the same constant).
constexpr int kBndThreads = 32 * F32_BND_FACES_PER_BLOCK;

// Per-face scalars the group shares (written by its first warp).
struct BndShared {
    EqP ew, ein;
    double red[kBndThreads / 32][4];
    double tot[4];
    double rr, TT, uux, uuy;
    int mode;
};

template <int TPF> struct BndGroup;
template <> struct BndGroup<32> {  // one warp per face
    static __device__ __forceinline__ int rank() { return threadIdx.x & 31; }
    static __device__ __forceinline__ bool leader() { return true; }
    static __device__ __forceinline__ void sync() { __syncwarp(); }
};
template <> struct BndGroup<kBndThreads> {  // the block per face
    static __device__ __forceinline__ int rank() { return threadIdx.x; }
    static __device__ __forceinline__ bool leader() { return threadIdx.x < 32; }
    static __device__ __forceinline__ void sync() { __syncthreads(); }
};

// Group sums of N compensated FP32 partials (sum s, compensation c) in float-float, then FP64
// across the block's warps in warp order; every thread of the group receives the totals.
template <int TPF, int N>
__device__ __forceinline__ void group_sum(const float (&s)[N], const float (&c)[N], double (&out)[N], BndShared &S) {
#pragma unroll
    for (int k = 0; k < N; ++k) out[k] = warp_sum_ff(s[k], -c[k]);
    if (TPF == 32) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < N; ++k) S.red[warp][k] = out[k];
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < N; ++k) {
            double v = lane < kBndThreads / 32 ? S.red[lane][k] : 0.0;
#pragma unroll
            for (int o = kBndThreads / 64; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) S.tot[k] = v;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < N; ++k) out[k] = S.tot[k];
}

template <int TPF> __device__ __forceinline__ void bnd_face(const F32Inst &I, int b, BndShared &S) {
    using G = BndGroup<TPF>;
    const int r = G::rank();
    const int f = I.bface[b];
    const meso_mark_desc &mk = I.marks[I.fmark[f]];
    const int nb = I.fown[f];
    const float k3 = I.k3_32, twoK = I.twoK32;
    float2 *bin = I.bnd_in + (size_t)b * I.NVp;
    float2 *bout = I.bnd_out + (size_t)b * I.NVp;
    const float2 n = I.fn32[f];
    const double2 n64 = I.fn64[f];
    {  // blend with the face equilibrium (cdugks_shakhov.cpp:350-361), deviations from (g0, h0)
        const FaceK k = I.fk[f];
        for (int p = r; p < I.NVp; p += TPF) {
            const float4 t = I.vt32[p];
            const float2 gs = dshakhov(k.e, t.x, t.y, fmaf(t.x, t.x, t.y * t.y), t.w, k3, twoK);
            const float2 gb = bin[p];
            bin[p] = make_float2(fmaf(k.oCs, gb.x, k.Cs * gs.x), fmaf(k.oCs, gb.y, k.Cs * gs.y));
        }
    }
    // incoming set for this face type; kn = xi . n_in = -(xi . n0): class 1 = incoming, 2 = grazing
    if (G::leader()) {
        const int type = mk.type;
        double rr = 0.0, TT = 0.0, uux = 0.0, uuy = 0.0;
        int mode = 0;  // 0 keep, 1 Maxwell incoming, 2 wall, 3 slip wall, 4 symmetry
        if (type == MESO_BC_PRESSURE_INLET) {
            const double T_m = I.T[nb], umx = I.u[3 * nb], umy = I.u[3 * nb + 1];
            const double nx = -n64.x, ny = -n64.y;
            const double sn = umx * nx + umy * ny;
            uux = nx * sn;
            uuy = ny * sn;
            TT = mk.temperature;
            rr = solve_pressure(mk.pressure, I.R, T_m, uux, uuy, I.gamma) / (I.R * TT);
            mode = 1;
        } else if (type == MESO_BC_FARFIELD_INLET) {
            rr = mk.density;
            uux = mk.velocity[0];
            uuy = mk.velocity[1];
            TT = mk.temperature;
            mode = 1;
        } else if (type == MESO_BC_FREESTREAM_INLET) {
            TT = mk.temperature;
            rr = mk.pressure / (I.R * TT);
            uux = mk.velocity[0];
            uuy = mk.velocity[1];
            mode = 1;
        } else if (type == MESO_BC_PRESSURE_OUTLET) {
            const double umx = I.u[3 * nb], umy = I.u[3 * nb + 1], T_m = I.T[nb];
            rr = solve_pressure(mk.pressure, I.R, T_m, umx, umy, I.gamma) / (I.R * T_m);
            const double nx = n64.x, ny = n64.y;  // nv_e = -nv = n0
            const double sn = umx * nx + umy * ny;
            uux = nx * sn;
            uuy = ny * sn;
            TT = mk.temperature;
            mode = 1;
        } else if (type == MESO_BC_FARFIELD_OUTLET) {
            rr = I.rho[nb];
            TT = I.T[nb];
            uux = I.u[3 * nb];
            uuy = I.u[3 * nb + 1];
            mode = 1;
        } else if (type == MESO_BC_WALL) {
            mode = 2;
        } else if (type == MESO_BC_SLIP_WALL) {
            mode = 3;
        } else if (type == MESO_BC_SYMMETRY) {
            mode = 4;
        }
        if (mode == 2 || mode == 3) {
            // the balance's wall Maxwellian: zeroGradient walls balance with the cell's temperature
            double T_w = 0.0;
            if (mk.temperature_type == MESO_PATCH_ZERO_GRADIENT) T_w = I.T[nb];
            else if (mk.temperature_type == MESO_PATCH_FIXED_VALUE) T_w = mk.temperature;
            const EqP ew = make_eqp(I, 1.0, mk.velocity[0], mk.velocity[1], T_w, 0.0, 0.0);
            if ((threadIdx.x & 31) == 0) S.ew = ew;
        }
        if ((threadIdx.x & 31) == 0) {
            S.mode = mode;
            S.rr = rr;
            S.TT = TT;
            S.uux = uux;
            S.uuy = uuy;
        }
    }
    G::sync();  // blended values and the face scalars are visible to the whole group
    const int mode = S.mode;
    double rr = S.rr, TT = S.TT, uux = S.uux, uuy = S.uuy;
    double rho_w = 0.0, den_w = 0.0;
    if (mode == 2 || mode == 3) {
        // diffuse-wall density balance (cdugks_shakhov.cpp:468-497): outgoing mass of the
        // blended face values over the incoming mass of a unit-density wall Maxwellian
        // g0 (1 + expm1(E_w)); the g0 parts are the precomputed half-range sums
        const EqP ew = S.ew;
        float s2[2] = {0.f, 0.f}, c2[2] = {0.f, 0.f};
        for (int p = r; p < I.NVp; p += TPF) {
            const float4 t = I.vt32[p];
            const float xx = t.x, xy = t.y, w = t.z;
            const float d = fmaf(n.x, xx, n.y * xy);
            const int cls = cls_of(I, f, p);
            if (cls == 1) {  // kn = -d >= VSMALL
                const float E = fmaf(ew.ea, fmaf(xx, xx, xy * xy), fmaf(ew.ebx, xx, fmaf(ew.eby, xy, ew.ec)));
                kahan(s2[1], c2[1], -d * w * t.w * expm1_dev(E));
            } else {
                kahan(s2[0], c2[0], d * w * bin[p].x);
            }
        }
        double tot2[2];
        group_sum<TPF, 2>(s2, c2, tot2, S);
        const double num = I.bnd_g0[2 * b] + tot2[0];
        const double den = I.bnd_g0[2 * b + 1] + tot2[1];
        rho_w = num / den;
        den_w = den;
        rr = rho_w;
        TT = mk.temperature;
        uux = mk.velocity[0];
        uuy = mk.velocity[1];
    }
    // incoming Maxwellian (rr, uu, TT) as a deviation from (g0, h0)
    if (G::leader()) {
        const EqP ein = make_eqp(I, rr > 0.0 ? rr : 1.0, uux, uuy, TT > 0.0 ? TT : I.T0, 0.0, 0.0);
        if ((threadIdx.x & 31) == 0) S.ein = ein;
    }
    G::sync();
    const EqP ein = S.ein;
    const int dir = mk.direction;
    const float au = (float)mk.alpha_u, aT = (float)mk.alpha_T;
    // The balance and the incoming set use the same temperature only for a fixedValue wall
    // (a zeroGradient wall balances with T_cell but sets with the patch scalar, :473-479 vs :533).
    const bool exact_mass = mode == 2 && mk.temperature_type == MESO_PATCH_FIXED_VALUE;
    const float knA0 = I.farea[f];
    float sm4[4] = {0.f, 0.f, 0.f, 0.f}, cm4[4] = {0.f, 0.f, 0.f, 0.f};
    for (int p = r; p < I.NVp; p += TPF) {
        const float4 t = I.vt32[p];
        const float xx = t.x, xy = t.y, w = t.z;
        const float d = fmaf(n.x, xx, n.y * xy);
        float2 v = bin[p];
        int cls = 0;
        if (mode != 0 && p < I.NV) {
            cls = cls_of(I, f, p);
            if (mode == 4) {
                const float2 rv = bin[I.sym[3 * p + dir]];
                if (cls == 1) v = rv;
                else if (cls == 2) v = make_float2(0.5f * (v.x + rv.x), 0.5f * (v.y + rv.y));
            } else if (cls != 0) {
                float2 inc = dshakhov(ein, xx, xy, fmaf(xx, xx, xy * xy), t.w, k3, twoK);
                if (mode == 3) {
                    const float2 rv = bin[I.sym[3 * p + dir]];
                    inc = make_float2((1.f - au) * inc.x + au * rv.x, (1.f - aT) * inc.y + aT * rv.y);
                }
                if (mode == 1) {
                    if (cls == 1) v = inc;
                } else {
                    v = cls == 1 ? inc : make_float2(0.5f * (inc.x + v.x), 0.5f * (inc.y + v.y));
                }
            }
        }
        // the face's flux value (n0.xi) A f for the update kernel
        const float knA = d * knA0;
        bout[p] = make_float2(knA * v.x, knA * v.y);
        // moment fluxes of the deviations along n0 (the g0 parts are added in FP64 below)
        const float wkn = w * d;
        const float a = wkn * v.x;
        // diffuse wall: the incoming mass flux is rho_w * den exactly (added below), so the face
        // carries no net mass in FP32 storage either (cdugks_shakhov.cpp:468-497)
        if (!(exact_mass && cls == 1)) kahan(sm4[0], cm4[0], a);
        kahan(sm4[1], cm4[1], a * xx);
        kahan(sm4[2], cm4[2], a * xy);
        kahan(sm4[3], cm4[3], wkn * fmaf(fmaf(xx, xx, xy * xy), v.x, v.y));
    }
    double tot[4];
    group_sum<TPF, 4>(sm4, cm4, tot, S);
    if (r == 0) {
        const double *g0f = I.g0flux + (size_t)f * 4;
        // exact-mass wall: the g0 mass over the non-incoming set is the balance's numerator part
        tot[0] += exact_mass ? I.bnd_g0[2 * b] - rho_w * den_w : g0f[0];
        for (int q = 1; q < 4; ++q) tot[q] += g0f[q];
        double *o = I.fsum + (size_t)f * 4;
        for (int q = 0; q < 4; ++q) o[q] = tot[q];
    }
    G::sync();  // the group's shared scalars are rewritten by its next face
}

// Work items (instance, first boundary face): for TPF = kBndThreads (large velocity sets) y is
// one face for the whole block; for TPF = 32 (small sets) y = -(first face) - 1 of the eight faces
// the block's warps take, one each.  Two kernels, so that each form gets its own register budget.
template <int TPF>
__global__ void __launch_bounds__(kBndThreads) k32_boundary(const F32Inst *__restrict__ insts,
                                                           const int2 *__restrict__ items, int nitems) {
    __shared__ BndShared sh[TPF == 32 ? kBndThreads / 32 : 1];
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        const int2 item = items[it];
        const F32Inst &I = insts[item.x];
        if (step_stopped(I.status)) continue;
        if (TPF == 32) {
            const int b = -item.y - 1 + (threadIdx.x >> 5);
            if (b < I.nb) bnd_face<32>(I, b, sh[threadIdx.x >> 5]);
        } else {
            bnd_face<kBndThreads>(I, item.y, sh[0]);
        }
    }
}

// Half-range sums of the reference Maxwellian over each boundary face (static: geometry and
// velocity set only): [2b] = sum over non-incoming xi of (xi.n0) w g0, [2b+1] = sum over
// incoming xi of (xi.n_in) w g0, with the step's classification.  One block per face, FP64.
__global__ void __launch_bounds__(256) k32_bnd_setup(const F32Inst *__restrict__ insts, const int *__restrict__ boff,
                                                    int ninst, int total) {
    __shared__ double sh[8];
    for (int g = blockIdx.x; g < total; g += gridDim.x) {
        const int i = find_inst(boff, ninst, g);
        const F32Inst &I = insts[i];
        const int b = g - boff[i];
        const int f = I.bface[b];
        const double2 n64 = I.fn64[f];
        double s0 = 0.0, s1 = 0.0;
        for (int p = threadIdx.x; p < I.NVp; p += blockDim.x) {
            const int cls = cls_of(I, f, p);
            const double d = n64.x * I.xi64x[p] + n64.y * I.xi64y[p];
            const double t = d * I.w64[p] * I.g0_64[p];
            if (cls == 1) s1 -= t;
            else s0 += t;
        }
        const double a = block_sum(s0, sh), c = block_sum(s1, sh);
        if (threadIdx.x == 0) {
            I.bnd_g0[2 * b] = a;
            I.bnd_g0[2 * b + 1] = c;
        }
        __syncthreads();
    }
}

// Upwind masks of every face (static: geometry and velocity set), one warp per face: for each word
// of 32 velocities (chunk ch, slot v of the lane layout) bit l of .x is set when velocity
// 32 (ch VPL + v) + l upwinds from the owner (n0.xi >= VSMALL, in FP64 in the reference's order,
// cdugks_shakhov.cpp:223-276), bit l of .y when it upwinds from the neighbour (< -VSMALL); neither
// bit: between, the average of both sides.  Layout [chunk][face][v].
__global__ void __launch_bounds__(256) k32_cls_setup(const F32Inst *__restrict__ insts, const int *__restrict__ foff,
                                                    int ninst, int total) {
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    for (int g = blockIdx.x * wpb + (threadIdx.x >> 5); g < total; g += gridDim.x * wpb) {
        const int i = find_inst(foff, ninst, g);
        const F32Inst &I = insts[i];
        const int f = g - foff[i];
        const double2 n = I.fn64[f];
        for (int w = 0; w < I.NVp / 32; ++w) {
            const int p = 32 * w + lane;
            const double d = __dadd_rn(__dmul_rn(n.x, I.xi64x[p]), __dmul_rn(n.y, I.xi64y[p]));
            const unsigned own = __ballot_sync(0xffffffffu, d >= kVSMALL);
            const unsigned nei = __ballot_sync(0xffffffffu, d < -kVSMALL);
            if (lane == 0) {
                const int ch = w / I.vpl, v = w - ch * I.vpl;
                I.fcls[((size_t)ch * I.F + f) * I.vpl + v] = make_uint2(own, nei);
            }
        }
    }
}

// Fluxes of the reference pair along each face's n0 (static), one thread per face.
__global__ void k32_face_setup(const F32Inst *__restrict__ insts, const int *__restrict__ foff, int ninst, int total) {
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
        const int i = find_inst(foff, ninst, g);
        const F32Inst &I = insts[i];
        const int f = g - foff[i];
        double o[4];
        g0_fluxes(I, I.fn64[f].x, I.fn64[f].y, o);
        for (int q = 0; q < 4; ++q) I.g0flux[(size_t)f * 4 + q] = o[q];
    }
}

// =============================================================================
// CM: cell macros and evolution constants (one thread per cell, FP64)
// =============================================================================

__global__ void k32_cell_macros(const F32Inst *__restrict__ insts, const int *__restrict__ coff, int ninst, int total) {
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
        const int i = find_inst(coff, ninst, g);
        const F32Inst &I = insts[i];
        if (step_stopped(I.status)) continue;
        const int c = g - coff[i];
        double m0 = 0.0, m1x = 0.0, m1y = 0.0, m2 = 0.0;
        for (int j = I.cf_ptr[c]; j < I.cf_ptr[c + 1]; ++j) {
            const int f = I.cf_face[j];
            const double sA = (I.fown[f] == c ? 1.0 : -1.0) * I.farea64[f];
            const double *fs = I.fsum + (size_t)f * 4;
            double F0, F1, F2, F3;
            if (I.fbnd[f] >= 0) {
                F0 = fs[0];
                F1 = fs[1];
                F2 = fs[2];
                F3 = fs[3];
            } else {
                const double Cs = I.fmac[(size_t)f * 8 + 6], oCs = 1.0 - Cs;
                const double *fb = I.fgbar + (size_t)f * 4;
                F0 = oCs * fb[0] + Cs * fs[0];
                F1 = oCs * fb[1] + Cs * fs[1];
                F2 = oCs * fb[2] + Cs * fs[2];
                F3 = oCs * fb[3] + Cs * fs[3];
            }
            m0 += sA * F0;
            m1x += sA * F1;
            m1y += sA * F2;
            m2 += sA * F3;
        }
        I.fm0[c] = m0;
        I.fm1[3 * c] = m1x;
        I.fm1[3 * c + 1] = m1y;
        I.fm1[3 * c + 2] = 0.0;
        I.fm2[c] = m2;
        // conservative update (cdugks_shakhov.cpp:645-660)
        const double dt_v = I.dt / I.vol[c];
        const double rho_n = I.rho[c], unx = I.u[3 * c], uny = I.u[3 * c + 1], T_n = I.T[c];
        const double qnx = I.q[3 * c], qny = I.q[3 * c + 1];
        const double rhoE_n = rho_n * (0.5 * (unx * unx + uny * uny) + I.Cv * T_n);
        const double irho_n = 1.0 / rho_n, iT_n = 1.0 / T_n;
        const double tau_n = tau_r(I, irho_n, T_n, iT_n);
        double rho = rho_n - dt_v * m0;
        double rux = rho_n * unx - dt_v * m1x, ruy = rho_n * uny - dt_v * m1y;
        double rhoE = rhoE_n - dt_v * 0.5 * m2;
        if (I.corrW) {  // defect correction of the conserved update
            const double *cw = I.corrW + 4 * (size_t)c;
            rho += cw[0];
            rux += cw[1];
            ruy += cw[2];
            rhoE += cw[3];
        }
        const double irho = 1.0 / rho;
        const double ux = rux * irho, uy = ruy * irho;
        const double T = (rhoE * irho - 0.5 * (ux * ux + uy * uy)) * I.iCv, iT = 1.0 / T;
        const double tau = tau_r(I, irho, T, iT);
        I.rho[c] = rho;
        I.u[3 * c] = ux;
        I.u[3 * c + 1] = uy;
        I.u[3 * c + 2] = 0.0;
        I.T[c] = T;
        I.u32[c] = make_float2((float)ux, (float)uy);
        CellK k;
        k.en = make_eqp_r(I, rho_n, irho_n, unx, uny, T_n, iT_n * I.iR, qnx, qny);
        k.e1 = make_eqp_r(I, rho, irho, ux, uy, T, iT * I.iR, qnx, qny);
        const double itau = 1.0 / tau, itau_n = 1.0 / tau_n;
        k.cm = (float)(I.hdt / (I.hdt - 2.0 * tau_n));
        k.C = (float)(tau / (tau + I.hdt));
        k.Cs = (float)(0.5 * I.hdt * itau);
        k.hdt_tau = (float)(I.hdt * itau);
        k.hdt_taun = (float)(I.hdt * itau_n);
        k.dt_v = (float)dt_v;
        I.ck[c] = k;
        // monitor (cdugks_shakhov.cpp:697-719)
        if (isnan(rho) || T < 0.0 || isnan(T)) {
            DStatus *st = I.status;
            atomicAdd(&st->bad_count, 1);
            atomicMin(&st->first_bad, c);
            if (I.mask && I.mask[c]) {
                int slot = atomicAdd(&st->repair_count, 1);
                if (slot < I.C) I.repair_list[slot] = c;
            } else {
                atomicMin(&st->stop_step, st->step);
            }
        }
    }
}

// =============================================================================
// QR: heat flux from the partials; mask repair; end of step
// =============================================================================
__global__ void k32_heat_flux(const F32Inst *__restrict__ insts, const int *__restrict__ coff, int ninst, int total,
                              int count_step) {
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
        const int i = find_inst(coff, ninst, g);
        const F32Inst &I = insts[i];
        if (count_step && step_stopped(I.status)) continue;
        const int c = g - coff[i];
        double qx = 0.0, qy = 0.0;
#pragma unroll 4
        for (int grp = 0; grp < I.ngroup; ++grp) {
            const float4 qp = I.qpart[(size_t)grp * I.C + c];
            qx += (double)qp.x + (double)qp.y;
            qy += (double)qp.z + (double)qp.w;
        }
        {  // the reference pair's part, 1/2 sum w c (c^2 g0 + h0) about the cell velocity
            double M0[F32_NMOM];
            g0_raw_moments(I, I.u[3 * c], I.u[3 * c + 1], M0);
            qx += 0.5 * (M0[6] + M0[9]);
            qy += 0.5 * (M0[7] + M0[10]);
        }
        if (I.corrq) {  // defect correction
            qx += I.corrq[2 * (size_t)c];
            qy += I.corrq[2 * (size_t)c + 1];
        }
        I.q[3 * c] = qx;
        I.q[3 * c + 1] = qy;
        I.q[3 * c + 2] = 0.0;
    }
}

// cell_value_interp (cdugks_shakhov.cpp:766-789) for queued masked cells, writing state n+1
__global__ void k32_mask_repair(const F32Inst *__restrict__ insts, int ninst) {
    for (int i = blockIdx.x; i < ninst; i += gridDim.x) {  // a block per instance: repairs are rare
        const F32Inst &I = insts[i];
        const int n = min(I.status->repair_count, I.C);
        if (n == 0) continue;
        const int nxt = (I.status->step & 1) ^ 1;  // before k32_end_step advances the step
        for (int r = 0; r < n; ++r) {
            const int c = I.repair_list[r];
            double sw = 0.0, sr = 0.0, sT = 0.0, sux = 0.0, suy = 0.0, sqx = 0.0, sqy = 0.0;
            for (int j = I.cn_ptr[c]; j < I.cn_ptr[c + 1]; ++j) {
                const double *dr = I.lsq_dr + 3 * (size_t)j;
                const double wi = 1.0 / (dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2]);
                const int nb = I.cn_cell[j];
                sw += wi;
                sr += wi * I.rho[nb];
                sT += wi * I.T[nb];
                sux += wi * I.u[3 * nb];
                suy += wi * I.u[3 * nb + 1];
                sqx += wi * I.q[3 * nb];
                sqy += wi * I.q[3 * nb + 1];
            }
            const double rho = sr / sw, T = sT / sw, ux = sux / sw, uy = suy / sw, qx = sqx / sw, qy = sqy / sw;
            const double RT = I.R * T, p = rho * RT, over = 0.5 / RT;
            for (int pp = threadIdx.x; pp < I.NVp; pp += blockDim.x) {
                const double cx = I.xi64x[pp] - ux, cy = I.xi64y[pp] - uy, cc = cx * cx + cy * cy;
                const double cq = cx * qx + cy * qy;
                const double gm = rho * over / kPI * exp(-cc * over);
                const double gg = (1.0 - I.Pr) * (cq / (5.0 * p * RT)) * (cc / RT - 4.0) * gm + gm;
                const double hh = (1.0 - I.Pr) * (cq / (5.0 * p)) * ((cc / RT - 2.0) * (I.Kd + 1.0) - 2.0 * I.Kd) * gm +
                                  (I.Kd + 1.0) * RT * gm;
                const double g0 = I.g0_64[pp];
                I.S[nxt][(size_t)c * I.NVp + pp] = make_float2((float)(gg - g0), (float)(hh - I.hm0 * g0));
            }
            if (threadIdx.x == 0) {
                I.rho[c] = rho;
                I.T[c] = T;
                I.u[3 * c] = ux;
                I.u[3 * c + 1] = uy;
                I.u32[c] = make_float2((float)ux, (float)uy);
            }
            __syncthreads();  // the next repair's neighbour sums see this one, in every thread alike
        }
    }
}

__global__ void k32_end_step(const F32Inst *__restrict__ insts, int ninst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ninst) return;
    DStatus *st = insts[i].status;
    if (step_stopped(st)) return;
    st->repairs_total += st->repair_count;
    st->repair_count = 0;
    st->step += 1;
}

// Residual check of do_step (Solver::residual, field.cpp:223-249; counter cdugks_shakhov.cpp:747-756)
// every res_interval completed steps, one block per instance: per field the volume-weighted mean of
// |new - old| / |old| (MESO_RES_L2: the volume-weighted L2-relative change instead), summed per
// thread over cells and reduced in a fixed order in FP64; then the converge counter, the halt of a
// converged instance, and old <- new.
__global__ void __launch_bounds__(512) k32_residual(const F32Inst *__restrict__ insts, int ninst) {
    __shared__ double red[16][12];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = blockIdx.x; i < ninst; i += gridDim.x) {
        const F32Inst &I = insts[i];
        DStatus *st = I.status;
        const int step = st->step;
        if (I.res_interval <= 0 || step <= 0 || step % I.res_interval != 0) continue;
        if (st->stop_step != INT_MAX || st->halt) continue;
        F32Resid *R = I.resid;
        if (R->checks == step / I.res_interval) continue;  // this check already ran
        const bool l2 = (I.res_fields & MESO_RES_L2) != 0;
        double a[12];
#pragma unroll
        for (int k = 0; k < 12; ++k) a[k] = 0.0;
        for (int c = threadIdx.x; c < I.C; c += blockDim.x) {
            const double nw[6] = {I.rho[c], I.T[c], I.u[3 * c], I.u[3 * c + 1], I.q[3 * c], I.q[3 * c + 1]};
            const double od[6] = {I.rho_old[c], I.T_old[c], I.u_old[3 * c], I.u_old[3 * c + 1], I.q_old[3 * c],
                                  I.q_old[3 * c + 1]};
            if (l2) {
#pragma unroll
                for (int k = 0; k < 6; ++k) {
                    const double d = nw[k] - od[k];
                    a[2 * k] += I.vol[c] * d * d;
                    a[2 * k + 1] += I.vol[c] * od[k] * od[k];
                }
            } else {
                const double wv = I.vol[c] / I.total_volume;
#pragma unroll
                for (int k = 0; k < 6; ++k) a[k] += fabs((nw[k] - od[k]) / od[k]) * wv;
            }
        }
#pragma unroll
        for (int k = 0; k < 12; ++k) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) a[k] += __shfl_xor_sync(0xffffffffu, a[k], o);
            if (lane == 0) red[warp][k] = a[k];
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double t[12];
            for (int k = 0; k < 12; ++k) {
                t[k] = 0.0;
                for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t[k] += red[w][k];
            }
            const int field[6] = {MESO_RES_RHO, MESO_RES_T, MESO_RES_U, MESO_RES_U, MESO_RES_Q, MESO_RES_Q};
            const int watch = I.res_fields & (MESO_RES_RHO | MESO_RES_T | MESO_RES_U | MESO_RES_Q);
            bool conv = true;
            for (int k = 0; k < 6; ++k) {
                const double r = l2 ? (t[2 * k + 1] > 0.0 ? sqrt(t[2 * k] / t[2 * k + 1]) : sqrt(t[2 * k])) : t[k];
                R->res[k] = r;
                if (watch == 0 || (watch & field[k])) conv = conv && (r <= I.res_limit);
            }
            R->nres = 6;
            R->checks = step / I.res_interval;
            R->converge_state = conv ? R->converge_state + 1 : 0;
            if (R->converge_state >= 10) {
                R->converged = 1;
                st->halt = 1;  // run_state false: no further steps (the reference's loop breaks here)
            }
        }
        for (int c = threadIdx.x; c < I.C; c += blockDim.x) {
            I.rho_old[c] = I.rho[c];
            I.T_old[c] = I.T[c];
            I.u_old[3 * c] = I.u[3 * c];
            I.u_old[3 * c + 1] = I.u[3 * c + 1];
            I.q_old[3 * c] = I.q[3 * c];
            I.q_old[3 * c + 1] = I.q[3 * c + 1];
        }
        __syncthreads();
    }
}

// =============================================================================
// initial() (cdugks_shakhov.cpp:81-168), one warp per cell: the stored deviations are the cell's
// equilibrium (mode 0: Maxwellian; mode 1: Shakhov with the given q) less the reference pair,
// evaluated like every equilibrium of the step (dshakhov, FP32).  Mode 0 then sets the macros to
// the discrete moments of the stored distribution: the reference pair's part in FP64 from its
// discrete moments, the deviations' part as compensated FP32 lane sums, about the given velocity.
// =============================================================================
__global__ void k32_init(const F32Inst *__restrict__ insts, const int *__restrict__ coff, int ninst, int total,
                         int mode) {
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    for (int g = blockIdx.x * wpb + (threadIdx.x >> 5); g < total; g += gridDim.x * wpb) {
        const int i = find_inst(coff, ninst, g);
        const F32Inst &I = insts[i];
        const int c = g - coff[i];
        const int cur = I.status->step & 1;
        const double r = I.rho[c], ux = I.u[3 * c], uy = I.u[3 * c + 1], T = I.T[c];
        const double qx = mode == 0 ? 0.0 : I.q[3 * c], qy = mode == 0 ? 0.0 : I.q[3 * c + 1];
        const EqP e = make_eqp(I, r, ux, uy, T, qx, qy);
        const float k3 = I.k3_32, twoK = I.twoK32, ux32 = (float)ux, uy32 = (float)uy;
        float sm[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, cm[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        float2 *__restrict__ S = I.S[cur] + (size_t)c * I.NVp;
        for (int pp = lane; pp < I.NVp; pp += 32) {
            const float4 t = I.vt32[pp];  // xi_x, xi_y, w, g0
            const float x2 = fmaf(t.x, t.x, t.y * t.y);
            const float2 d = dshakhov(e, t.x, t.y, x2, t.w, k3, twoK);
            S[pp] = d;
            if (mode == 0) {  // w dg, w c dg, w (c^2 dg + dh), w c (c^2 dg + dh) about the given velocity
                const float cx = t.x - ux32, cy = t.y - uy32, cc = fmaf(cx, cx, cy * cy);
                const float wg = t.z * d.x, ws = t.z * fmaf(cc, d.x, d.y);
                kahan(sm[0], cm[0], wg);
                kahan(sm[1], cm[1], wg * cx);
                kahan(sm[2], cm[2], wg * cy);
                kahan(sm[3], cm[3], ws);
                kahan(sm[4], cm[4], ws * cx);
                kahan(sm[5], cm[5], ws * cy);
            }
        }
        if (mode == 0) {
            double v[6];
#pragma unroll
            for (int k = 0; k < 6; ++k) {
                v[k] = (double)sm[k] - (double)cm[k];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
            }
            if (lane == 0) {
                double M0[F32_NMOM];  // the reference pair's moments about the given velocity
                g0_raw_moments(I, ux, uy, M0);
                const double rho = M0[0] + v[0];
                const double mx = M0[1] + v[1], my = M0[2] + v[2];  // sum w c g
                const double vx = ux + mx / rho, vy = uy + my / rho;
                // sum w (xi^2 g + h) with xi = u + c
                const double e2 = (M0[3] + M0[5] + M0[8] + v[3]) + 2.0 * (ux * mx + uy * my) + (ux * ux + uy * uy) * rho;
                I.rho[c] = rho;
                I.u[3 * c] = vx;
                I.u[3 * c + 1] = vy;
                I.u[3 * c + 2] = 0.0;
                I.T[c] = (0.5 * e2 / rho - 0.5 * (vx * vx + vy * vy)) / I.Cv;
                I.q[3 * c] = 0.5 * (M0[6] + M0[9] + v[4]);
                I.q[3 * c + 1] = 0.5 * (M0[7] + M0[10] + v[5]);
                I.q[3 * c + 2] = 0.0;
            }
        }
        if (lane == 0) I.u32[c] = make_float2((float)I.u[3 * c], (float)I.u[3 * c + 1]);
    }
}

// ---- defect correction (fp32_to_plain, fp32_refine) ------------------------------
// The FP32 state in the FP64 step's layout: f0 = g0 + (g - g0), f1 = hm0 g0 + (h - h0), [C][NV].
__global__ void k32_to_plain(const F32Inst *__restrict__ inst, double *__restrict__ f0, double *__restrict__ f1) {
    const F32Inst &I = *inst;
    const float2 *__restrict__ S = I.S[I.status->step & 1];
    for (int c = blockIdx.x; c < I.C; c += gridDim.x)
        for (int p = threadIdx.x; p < I.NV; p += blockDim.x) {
            const float2 x = S[(size_t)c * I.NVp + p];
            const double g0 = I.g0_64[p];
            f0[(size_t)c * I.NV + p] = g0 + (double)x.x;
            f1[(size_t)c * I.NV + p] = I.hm0 * g0 + (double)x.y;
        }
}

// After one (corrected) FP32 step and one FP64 step from the same state: the state's correction
// takes the FP64 result minus the FP32 one, and the FP32 result is replaced by the FP64 one.
__global__ void k32_refine_state(const F32Inst *__restrict__ inst, const double *__restrict__ f0,
                                 const double *__restrict__ f1) {
    const F32Inst &I = *inst;
    if (step_stopped(I.status)) return;
    float2 *__restrict__ S = I.S[I.status->step & 1];
    for (int c = blockIdx.x; c < I.C; c += gridDim.x)
        for (int p = threadIdx.x; p < I.NV; p += blockDim.x) {
            const size_t at = (size_t)c * I.NVp + p, ip = (size_t)c * I.NV + p;
            const double g0 = I.g0_64[p];
            const double gd = f0[ip] - g0, hd = f1[ip] - I.hm0 * g0;
            // the FP32 step's value before rounding: the stored value and its residual
            const float2 x = S[at], r = I.corrR[at], cs = I.corrS[at];
            const double xg = (double)x.x + (double)r.x, xh = (double)x.y + (double)r.y;
            I.corrS[at] = make_float2((float)((double)cs.x + (gd - xg)), (float)((double)cs.y + (hd - xh)));
            // the FP64 result, rounded stochastically like every corrected step
            const float ng = (float)gd, nh = (float)hd;
            const unsigned hb = mix3((unsigned)c * 0x9E3779B1u, (unsigned)p * 0x85EBCA77u,
                                     (unsigned)I.status->step * 0xC2B2AE3Du ^ 0x5bd1e995u);
            S[at] = make_float2(sr_round(ng, (float)(gd - (double)ng), hb & 0xffffu),
                                sr_round(nh, (float)(hd - (double)nh), hb >> 16));
        }
}

// The same for the macros: the corrections of the conserved update and of the heat flux, then the
// FP64 step's rho, u, T, q (mac: the 8C block rho [C], u [3C], T [C], q [3C]).
__global__ void k32_refine_cells(const F32Inst *__restrict__ inst, const double *__restrict__ mac) {
    const F32Inst &I = *inst;
    if (step_stopped(I.status)) return;
    const int C = I.C;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < C; c += gridDim.x * blockDim.x) {
        const double r64 = mac[c], ux64 = mac[C + 3 * c], uy64 = mac[C + 3 * c + 1], T64 = mac[4 * C + c];
        const double qx64 = mac[5 * C + 3 * c], qy64 = mac[5 * C + 3 * c + 1];
        const double r32 = I.rho[c], ux32 = I.u[3 * c], uy32 = I.u[3 * c + 1], T32 = I.T[c];
        double *cw = I.corrW + 4 * (size_t)c;
        cw[0] += r64 - r32;
        cw[1] += r64 * ux64 - r32 * ux32;
        cw[2] += r64 * uy64 - r32 * uy32;
        cw[3] += r64 * (0.5 * (ux64 * ux64 + uy64 * uy64) + I.Cv * T64) -
                 r32 * (0.5 * (ux32 * ux32 + uy32 * uy32) + I.Cv * T32);
        I.corrq[2 * (size_t)c] += qx64 - I.q[3 * c];
        I.corrq[2 * (size_t)c + 1] += qy64 - I.q[3 * c + 1];
        I.rho[c] = r64;
        I.u[3 * c] = ux64;
        I.u[3 * c + 1] = uy64;
        I.T[c] = T64;
        I.q[3 * c] = qx64;
        I.q[3 * c + 1] = qy64;
        I.u32[c] = make_float2((float)ux64, (float)uy64);
    }
}

int grid_of(int total, int per_block, int cap) {
    int b = (total + per_block - 1) / per_block;
    return b < 1 ? 1 : (b < cap ? b : cap);
}

}  // namespace

int fp32_configure(int device) {
    (void)device;
    const int a1 = (int)tile_smem<1>(), a2 = (int)tile_smem<2>();
    if (cudaFuncSetAttribute(k32_reconstruct<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, a1) != cudaSuccess ||
        cudaFuncSetAttribute(k32_reconstruct<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, a2) != cudaSuccess)
        return -1;
    const int u1 = (int)upd_smem<1>(), u2 = (int)upd_smem<2>();
    const void *fn[6] = {(const void *)k32_update<1, 0>, (const void *)k32_update<1, 1>, (const void *)k32_update<1, 2>,
                         (const void *)k32_update<2, 0>, (const void *)k32_update<2, 1>, (const void *)k32_update<2, 2>};
    for (int k = 0; k < 6; ++k)
        if (cudaFuncSetAttribute(fn[k], cudaFuncAttributeMaxDynamicSharedMemorySize, k < 3 ? u1 : u2) != cudaSuccess)
            return -1;
    return 0;
}

const char *const kFp32Phases[] = {"k32_reconstruct", "k32_face_moments+macros", "k32_face_eqflux", "k32_boundary",
                                   "k32_cell_macros", "k32_update", "k32_heat_flux+repair+end+residual"};

int fp32_step(Fp32State &s, cudaStream_t stream, int64_t *launches, cudaEvent_t *ev, const StepFork *fork) {
    const int sms = s.num_sms;
    const int cap = sms * 32;
    // persistent CTAs (at most one per SM) over their own item lists; items of vpl == 2 instances,
    // then those of vpl == 1, each its own launch
    const int grid2 = s.grid2, grid1 = s.grid1;
    const int *off1 = s.d_item_off + grid2 + 1;
    int n = 0;
    auto tiles = [&](bool update) {
        if (grid2 > 0) {
            if (update && s.corr == 2)
                k32_update<2, 2><<<grid2, kUT, upd_smem<2>(), stream>>>(s.d_inst, s.d_items, s.d_item_off);
            else if (update && s.corr)
                k32_update<2, 1><<<grid2, kUT, upd_smem<2>(), stream>>>(s.d_inst, s.d_items, s.d_item_off);
            else if (update)
                k32_update<2, 0><<<grid2, kUT, upd_smem<2>(), stream>>>(s.d_inst, s.d_items, s.d_item_off);
            else k32_reconstruct<2><<<grid2, kT, tile_smem<2>(), stream>>>(s.d_inst, s.d_items, s.d_item_off);
            ++n;
        }
        if (grid1 > 0) {
            if (update && s.corr == 2) k32_update<1, 2><<<grid1, kUT, upd_smem<1>(), stream>>>(s.d_inst, s.d_items, off1);
            else if (update && s.corr) k32_update<1, 1><<<grid1, kUT, upd_smem<1>(), stream>>>(s.d_inst, s.d_items, off1);
            else if (update) k32_update<1, 0><<<grid1, kUT, upd_smem<1>(), stream>>>(s.d_inst, s.d_items, off1);
            else k32_reconstruct<1><<<grid1, kT, tile_smem<1>(), stream>>>(s.d_inst, s.d_items, off1);
            ++n;
        }
    };
    auto mark = [&](int k) {
        if (ev) cudaEventRecord(ev[k], stream);
    };
    mark(0);
    tiles(false);
    mark(1);
    if (s.has_large)
        k32_face_moments<4><<<grid_of(s.total_faces, 8, cap), 256, 0, stream>>>(s.d_inst, s.d_face_items, s.ninst,
                                                                            s.total_faces);
    if (s.has_small)
        k32_face_moments_small<8, kSmallFaceLanes><<<grid_of(s.total_faces, 8 * 32 / kSmallFaceLanes, cap), 256, 0,
                                                     stream>>>(s.d_inst, s.d_face_items, s.ninst, s.total_faces);
    n += (s.has_large ? 1 : 0) + (s.has_small ? 1 : 0) - 1;
    k32_face_macros<<<grid_of(s.total_faces, 128, cap), 128, 0, stream>>>(s.d_inst, s.d_face_items, s.ninst,
                                                                          s.total_faces);
    mark(2);
    auto boundary = [&](cudaStream_t st) {  // warp-per-face items first, then block-per-face items
        int k = 0;
        if (s.nbnd_warp > 0) {
            k32_boundary<32><<<grid_of(s.nbnd_warp, 1, cap), kBndThreads, 0, st>>>(s.d_inst, s.d_bnd_blocks,
                                                                                   s.nbnd_warp);
            ++k;
        }
        if (s.nbnd_blocks > s.nbnd_warp) {
            k32_boundary<kBndThreads><<<grid_of(s.nbnd_blocks - s.nbnd_warp, 1, cap), kBndThreads, 0, st>>>(
                s.d_inst, s.d_bnd_blocks + s.nbnd_warp, s.nbnd_blocks - s.nbnd_warp);
            ++k;
        }
        return k;
    };
    const bool branch = fork && !ev && s.total_bnd > 0;
    int nbl = 0;
    if (branch) {  // boundary faces on the side stream, interior faces' equilibrium fluxes here
        cudaEventRecord(fork->fork, stream);
        cudaStreamWaitEvent(fork->side, fork->fork, 0);
        nbl = boundary(fork->side);
        cudaEventRecord(fork->join, fork->side);
    }
    if (s.has_large)
        k32_face_eqflux<<<grid_of(s.total_faces, 8, cap), 256, 0, stream>>>(s.d_inst, s.d_face_items, s.ninst,
                                                                            s.total_faces);
    if (s.has_small)
        k32_face_eqflux_small<kSmallFaceLanes><<<grid_of(s.total_faces, 8 * 32 / kSmallFaceLanes, cap), 256, 0,
                                                 stream>>>(s.d_inst, s.d_face_items, s.ninst, s.total_faces);
    n += (s.has_large ? 1 : 0) + (s.has_small ? 1 : 0) - 1;
    mark(3);
    n += 3;
    if (branch) {
        cudaStreamWaitEvent(stream, fork->join, 0);
        n += nbl;
    } else if (s.total_bnd > 0) {
        n += boundary(stream);
    }
    mark(4);
    k32_cell_macros<<<grid_of(s.total_cells, 128, cap), 128, 0, stream>>>(s.d_inst, s.d_cell_items, s.ninst,
                                                                          s.total_cells);
    mark(5);
    tiles(true);
    mark(6);
    k32_heat_flux<<<grid_of(s.total_cells, 256, cap), 256, 0, stream>>>(s.d_inst, s.d_cell_items, s.ninst,
                                                                        s.total_cells, 1);
    k32_mask_repair<<<s.ninst < s.num_sms ? s.ninst : s.num_sms, 256, 0, stream>>>(s.d_inst, s.ninst);
    k32_end_step<<<(s.ninst + 63) / 64, 64, 0, stream>>>(s.d_inst, s.ninst);
    k32_residual<<<s.ninst < s.num_sms ? s.ninst : s.num_sms, 512, 0, stream>>>(s.d_inst, s.ninst);
    mark(7);
    n += 5;
    if (launches) *launches += n;
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int fp32_prepare(const Fp32State &s, cudaStream_t stream) {
    k32_cls_setup<<<grid_of(s.total_faces, 8, s.num_sms * 32), 256, 0, stream>>>(s.d_inst, s.d_face_items, s.ninst,
                                                                               s.total_faces);
    k32_face_setup<<<grid_of(s.total_faces, 256, s.num_sms * 32), 256, 0, stream>>>(s.d_inst, s.d_face_items, s.ninst,
                                                                                  s.total_faces);
    if (s.total_bnd > 0)
        k32_bnd_setup<<<grid_of(s.total_bnd, 1, s.num_sms * 32), 256, 0, stream>>>(s.d_inst, s.d_bnd_items, s.ninst,
                                                                                 s.total_bnd);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int fp32_to_plain(const F32Inst &I, const F32Inst *d_inst, double *f0, double *f1, double *mac, int sms,
                  cudaStream_t stream) {
    k32_to_plain<<<grid_of(I.C, 1, sms * 8), 256, 0, stream>>>(d_inst, f0, f1);
    if (cudaMemcpyAsync(mac, I.rho, sizeof(double) * 8 * (size_t)I.C, cudaMemcpyDeviceToDevice, stream) != cudaSuccess)
        return -1;
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int fp32_refine(const F32Inst &I, const F32Inst *d_inst, const double *f0, const double *f1, const double *mac,
                int sms, cudaStream_t stream) {
    k32_refine_state<<<grid_of(I.C, 1, sms * 8), 256, 0, stream>>>(d_inst, f0, f1);
    k32_refine_cells<<<grid_of(I.C, 256, sms * 4), 256, 0, stream>>>(d_inst, mac);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int fp32_init(const Fp32State &s, int mode, cudaStream_t stream) {
    k32_init<<<grid_of(s.total_cells, 8, s.num_sms * 32), 256, 0, stream>>>(s.d_inst, s.d_cell_items, s.ninst,
                                                                           s.total_cells, mode);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}


}  // namespace meso
