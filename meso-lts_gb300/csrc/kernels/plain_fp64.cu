// Plain FP64 step kernels: the parity form of the DUGKS / CDUGKS / Shakhov step.
//
// Distribution functions, face values and fluxes are FP64, laid out
// velocity-contiguous per cell ([cell][xi]) so a warp reads consecutive
// velocities of one cell.  The step runs as five phases, one kernel each,
// in the dependency order of the reference (cdugks_shakhov.cpp:213-722):
//   grad      per (cell, xi)  least-squares gradient      mesh_numerical.cpp:24-49
//   recon     per (face, xi)  half-step upwind value      cdugks_shakhov.cpp:223-298
//   face_eq   per face        moments over xi, blend      cdugks_shakhov.cpp:300-363
//   boundary  per bdry face   wall balance, inlets, ...   cdugks_shakhov.cpp:364-607
//   update    per cell        flux, macros, evolution, q  cdugks_shakhov.cpp:610-722
// Reductions over xi are segment reductions (warp shuffles + shared memory)
// over a fixed-width lane group per face or cell: deterministic, FP64.
//
// Every arithmetic expression follows the reference's operation order and
// this file is compiled with -fmad=false, so results differ from the CPU
// reference only through exp/pow rounding and the order of the xi sums.
#include <cfloat>
#include <climits>

#include "device_common.cuh"
#include "plain_fp64.h"

namespace meso {
namespace {

constexpr int kBlock = 256;

struct V3 {
    double x, y, z;
};
__device__ __forceinline__ V3 v3(double x, double y, double z) { return {x, y, z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ V3 scl(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }  // Vector*double
// Dot product in the reference's order; DIM == 2 drops the z term, which is an
// exact +0 there (z components of xi, normals and velocities are 0).
template <int DIM> __device__ __forceinline__ double dot(V3 a, V3 b) {
    if (DIM == 2) return a.x * b.x + a.y * b.y;
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
__device__ __forceinline__ V3 ld3(const double *p, int i) { return {p[3 * i], p[3 * i + 1], p[3 * i + 2]}; }
__device__ __forceinline__ void st3(double *p, int i, V3 v) {
    p[3 * i] = v.x;
    p[3 * i + 1] = v.y;
    p[3 * i + 2] = v.z;
}
__device__ __forceinline__ V3 xi_of(const DMesh &m, int p) { return {m.xix[p], m.xiy[p], m.xiz[p]}; }

// ---- equilibria (cdugks_shakhov.cpp:181-211, cdugks.cpp:116-121) -------------
template <int DIM> __device__ __forceinline__ double g_maxwell(const KParams &k, double rho, double t, double cc) {
    if (DIM == 2) {
        double over_RT2 = 0.5 / (k.R * t);
        return rho * over_RT2 / kPI * exp(-cc * over_RT2);
    }
    double RT = k.R * t;
    return rho / pow(2.0 * kPI * RT, 1.5) * exp(-cc * 0.5 / RT);
}
__device__ __forceinline__ double h_maxwell(const KParams &k, double t, double gm) {
    return (k.Kd + 3.0 - k.Dd) * (k.R * t) * gm;
}
__device__ __forceinline__ double g_shakhov(const KParams &k, double rho, double t, double cc, double cq, double gm) {
    double RT = k.R * t;
    double p = rho * RT;
    return (1.0 - k.Pr) * (cq / (5.0 * p * RT)) * (cc / RT - k.Dd - 2.0) * gm + gm;
}
__device__ __forceinline__ double h_shakhov(const KParams &k, double rho, double t, double cc, double cq, double gm) {
    double RT = k.R * t;
    double p = rho * RT;
    double h_m = h_maxwell(k, t, gm);
    return (1.0 - k.Pr) * (cq / (5.0 * p)) * ((cc / RT - k.Dd) * (k.Kd + 3.0 - k.Dd) - 2.0 * k.Kd) * gm + h_m;
}
__device__ __forceinline__ double tau_f(const KParams &k, double rho, double t) {
    return k.mu0 * pow(t / k.T0, k.vhs) / (rho * k.R * t);
}

// The Shakhov equilibrium of one (rho, T) with its per-state factors formed once, so that the
// velocity loops evaluate g_maxwell, g_shakhov and h_shakhov (cdugks_shakhov.cpp:185-211) with one
// exp and no division per velocity (FP64 divisions are slow on this GPU).  Same formulas; the
// results differ from the per-velocity divisions in the last bits only.
struct EqK64 {
    double A;     // rho / (2 pi R T)^(D/2)
    double oRT2;  // 1 / (2 R T)
    double iRT;   // 1 / (R T)
    double sg;    // (1 - Pr) / (5 p R T)
    double sh;    // (1 - Pr) / (5 p)
    double hm;    // (K + 3 - D) R T
};
template <int DIM> __device__ __forceinline__ EqK64 make_eqk(const KParams &k, double rho, double t) {
    EqK64 e;
    const double RT = k.R * t;
    e.iRT = 1.0 / RT;
    e.oRT2 = 0.5 * e.iRT;
    e.A = DIM == 2 ? rho * e.oRT2 / kPI : rho / pow(2.0 * kPI * RT, 1.5);
    const double c1 = (1.0 - k.Pr) / 5.0, ip = e.iRT / rho;
    e.sg = c1 * ip * e.iRT;
    e.sh = c1 * ip;
    e.hm = (k.Kd + 3.0 - k.Dd) * RT;
    return e;
}
// g_S and h_S at one velocity (cc = |c|^2, cq = c.q)
__device__ __forceinline__ void shakhov_eq(const KParams &k, const EqK64 &e, double cc, double cq, double &gs,
                                           double &hs) {
    const double gm = e.A * exp(-cc * e.oRT2);
    const double t = cc * e.iRT;
    gs = (e.sg * cq) * (t - k.Dd - 2.0) * gm + gm;
    hs = (e.sh * cq) * ((t - k.Dd) * (k.Kd + 3.0 - k.Dd) - 2.0 * k.Kd) * gm + e.hm * gm;
}
// The same with the Maxwellian g_M given (tensor-product velocity sets: A e^(-cx^2/2RT) e^(-cy^2/2RT)).
__device__ __forceinline__ void shakhov_eq_gm(const KParams &k, const EqK64 &e, double gm, double cc, double cq,
                                              double &gs, double &hs) {
    const double t = cc * e.iRT;
    gs = (e.sg * cq) * (t - k.Dd - 2.0) * gm + gm;
    hs = (e.sh * cq) * ((t - k.Dd) * (k.Kd + 3.0 - k.Dd) - 2.0 * k.Kd) * gm + e.hm * gm;
}
// The segment's factor tables at (u, 1/(2RT)): t[i] = e^(-(tx[i] - ux)^2 / 2RT) for i < ntx, then
// e^(-(ty[j] - uy)^2 / 2RT); every lane of the segment takes part.
__device__ __forceinline__ void exp_tables(const DMesh &m, V3 u, double oRT2, int lane, int L, double *t) {
    for (int i = lane; i < m.ntx + m.nty; i += L) {
        const double c = i < m.ntx ? m.tx[i] - u.x : m.ty[i - m.ntx] - u.y;
        t[i] = exp(-(c * c) * oRT2);
    }
}

template <int DIM> __device__ __forceinline__ double f_maxwell(const KParams &k, double rho, V3 u, V3 xi) {
    double ku_RT = dot<DIM>(u, xi) * k.over_RT;
    double uu_RT = dot<DIM>(u, u) * k.over_RT;
    return rho * (1.0 + ku_RT + (ku_RT * ku_RT - uu_RT) * 0.5);
}
// Boundary::Compressible::solve_pressure (pressure_boundary.cpp:15-18)
__device__ __forceinline__ double solve_pressure(double P0, double R, double T, V3 U, double gamma) {
    double mag = sqrt(U.x * U.x + U.y * U.y + U.z * U.z);
    double Ma = mag / sqrt(gamma * R * T);
    return P0 / pow(1.0 + (gamma - 1.0) / 2.0 * (Ma * Ma), gamma / (gamma - 1.0));
}

// ---- segment reduction of N values over L lanes (L = 32..256) -------------
template <int N>
__device__ __forceinline__ void seg_reduce(double (&v)[N], int L, double *sh) {
#pragma unroll
    for (int k = 0; k < N; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
    if (L <= 32) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < N; ++k) sh[warp * N + k] = v[k];
    __syncthreads();
    const int wps = L >> 5, first = (warp / wps) * wps;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        double s = 0.0;
        for (int q = 0; q < wps; ++q) s += sh[(first + q) * N + k];
        v[k] = s;
    }
    __syncthreads();
}

// ---- venkata_limiter (limiter.cpp:7-31) --------------------------------------
__device__ double venkata(const DMesh &m, const double *f, int p, double dw, int cell, double k, double eps, int dim) {
    if (fabs(dw) <= eps) return 1.0;
    double kh = k * pow(m.vol[cell], 1.0 / (double)dim);
    double omega = kh * kh * kh;
    const size_t NV = (size_t)m.NV;
    double w0 = f[(size_t)cell * NV + p], wmax = w0, wmin = w0;
    for (int j = m.cn_ptr[cell]; j < m.cn_ptr[cell + 1]; ++j) {
        double wn = f[(size_t)m.cn_cell[j] * NV + p];
        if (wn > wmax) wmax = wn;
        if (wn < wmin) wmin = wn;
    }
    double a = dw > 0.0 ? wmax - w0 : wmin - w0;
    double aa = a * a, ab = a * dw, bb = dw * dw;
    return (aa + 2.0 * ab + omega) / (aa + 2.0 * bb + ab + omega);
}

// ============================================================================
// grad: per (cell, xi) weighted least-squares gradient of NDIST distributions.
// ============================================================================
template <int DIM, int NDIST>
__global__ void __launch_bounds__(kBlock) k_grad(DMesh m, const DStatus *st, const double *f0, const double *f1,
                                                 double *g0, double *g1) {
    if (step_stopped(st)) return;
    const size_t NV = (size_t)m.NV;
    const size_t total = (size_t)m.C * NV;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(idx / NV);
        const int p = (int)(idx - (size_t)c * NV);
        const double *fs[2] = {f0, f1};
        double *gs[2] = {g0, g1};
#pragma unroll
        for (int d = 0; d < NDIST; ++d) {
            const double *f = fs[d];
            const double fc = f[idx];
            V3 S = v3(0.0, 0.0, 0.0);
            for (int j = m.cn_ptr[c]; j < m.cn_ptr[c + 1]; ++j) {
                const double wj = m.lsq_w[j];
                const double s = wj * (f[(size_t)m.cn_cell[j] * NV + p] - fc);
                V3 dr = ld3(m.lsq_dr, j);
                S.x = S.x + dr.x * s;
                S.y = S.y + dr.y * s;
                if (DIM == 3) S.z = S.z + dr.z * s;
            }
            const double *Cc = m.lsq_c + 9 * (size_t)c;
            V3 Cx = v3(Cc[0], Cc[1], Cc[2]), Cy = v3(Cc[3], Cc[4], Cc[5]), Cz = v3(Cc[6], Cc[7], Cc[8]);
            double *g = gs[d];
            g[idx * DIM + 0] = dot<DIM>(Cx, S);
            g[idx * DIM + 1] = dot<DIM>(Cy, S);
            if (DIM == 3) g[idx * DIM + 2] = dot<DIM>(Cz, S);
        }
    }
}

// ============================================================================
// recon: per (face, xi) half-step upwind reconstruction (plus optional limiter).
// ============================================================================
template <int DIM>
__device__ __forceinline__ double grad_dot(const double *g, size_t idx, V3 a) {
    V3 gv = v3(g[idx * DIM], g[idx * DIM + 1], DIM == 3 ? g[idx * DIM + 2] : 0.0);
    return dot<DIM>(a, gv);
}

template <int DIM, int NDIST, bool SHAKHOV>
__global__ void __launch_bounds__(kBlock) k_recon(DMesh m, KParams k, const DStatus *st, const double *f0,
                                                  const double *f1, const double *g0, const double *g1, double *face0,
                                                  double *face1) {
    if (step_stopped(st)) return;
    const size_t NV = (size_t)m.NV;
    const size_t total = (size_t)m.F * NV;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
        const int fi = (int)(idx / NV);
        const int p = (int)(idx - (size_t)fi * NV);
        const int own = m.fown[fi], nei = m.fnei[fi];
        const V3 nv = ld3(m.fn, fi);
        const V3 xi = xi_of(m, p);
        const double nv_xi = dot<DIM>(nv, xi);
        const size_t io = (size_t)own * NV + p, in = (size_t)nei * NV + p;
        const double *fs[2] = {f0, f1};
        const double *gs[2] = {g0, g1};
        double *outs[2] = {face0, face1};
        const V3 fpos = ld3(m.fpos, fi);
        const V3 xh = scl(xi, k.hdt);
#pragma unroll
        for (int d = 0; d < NDIST; ++d) {
            const double *f = fs[d];
            double val;
            if (!k.gradient) {
                if (nv_xi >= kVSMALL) val = f[io];
                else if (nv_xi < -kVSMALL) val = f[in];
                else val = 0.5 * (f[io] + f[in]);
            } else if (nv_xi >= kVSMALL) {
                V3 dr = fpos - ld3(m.cpos, own);
                double phi = 1.0;
                if (SHAKHOV && k.limiter)
                    phi = venkata(m, f, p, dot<DIM>(dr, v3(gs[d][io * DIM], gs[d][io * DIM + 1],
                                                           DIM == 3 ? gs[d][io * DIM + 2] : 0.0)),
                                  own, k.venkata_k, 1.0e-10, DIM);
                val = f[io] + phi * grad_dot<DIM>(gs[d], io, dr - xh);
            } else if (nv_xi < -kVSMALL) {
                V3 dr = fpos - ld3(m.cpos, nei);
                double phi = 1.0;
                if (SHAKHOV && k.limiter)
                    phi = venkata(m, f, p, dot<DIM>(dr, v3(gs[d][in * DIM], gs[d][in * DIM + 1],
                                                           DIM == 3 ? gs[d][in * DIM + 2] : 0.0)),
                                  nei, k.venkata_k, kVSMALL, DIM);
                val = f[in] + phi * grad_dot<DIM>(gs[d], in, dr - xh);
            } else {
                V3 dro = fpos - ld3(m.cpos, own), drn = fpos - ld3(m.cpos, nei);
                double po = 1.0, pn = 1.0;
                if (SHAKHOV && k.limiter) {
                    po = venkata(m, f, p, dot<DIM>(dro, v3(gs[d][io * DIM], gs[d][io * DIM + 1],
                                                           DIM == 3 ? gs[d][io * DIM + 2] : 0.0)),
                                 own, k.venkata_k, kVSMALL, DIM);
                    pn = venkata(m, f, p, dot<DIM>(drn, v3(gs[d][in * DIM], gs[d][in * DIM + 1],
                                                           DIM == 3 ? gs[d][in * DIM + 2] : 0.0)),
                                 nei, k.venkata_k, kVSMALL, DIM);
                }
                val = 0.5 * (f[io] + f[in] + po * grad_dot<DIM>(gs[d], io, dro - xh) +
                             pn * grad_dot<DIM>(gs[d], in, drn - xh));
            }
            outs[d][idx] = val;
        }
    }
}

// ============================================================================
// face_eq: per face, moments over xi -> face macros -> blend with the
// equilibrium.  BGK: cdugks.cpp:154-184.  Shakhov: cdugks_shakhov.cpp:300-363.
// ============================================================================
template <int DIM, bool SHAKHOV>
__global__ void __launch_bounds__(kBlock) k_face_eq(DMesh m, KParams k, const DStatus *st, int L, double *face0,
                                                    double *face1) {
    __shared__ double sh[(kBlock / 32) * 5];
    if (step_stopped(st)) return;
    const int spb = kBlock / L;
    const int fi = blockIdx.x * spb + threadIdx.x / L;
    const int lane = threadIdx.x % L;
    const bool active = fi < m.F;
    const size_t NV = (size_t)m.NV;
    const size_t base = (size_t)(active ? fi : 0) * NV;
    if (!SHAKHOV) {
        double v[4] = {0, 0, 0, 0};
        if (active)
            for (int p = lane; p < m.NV; p += L) {
                const double w = m.w[p];
                const double f = face0[base + p];
                const V3 xi = xi_of(m, p);
                v[0] += w * f;
                const double wf = w * f;
                v[1] += xi.x * wf;
                v[2] += xi.y * wf;
                if (DIM == 3) v[3] += xi.z * wf;
            }
        seg_reduce<4>(v, L, sh);
        if (!active) return;
        const double rho = v[0];
        const double r = 1.0 / rho;
        const V3 u = v3(v[1] * r, v[2] * r, v[3] * r);
        const double c_eq = k.c_eq_face;
        for (int p = lane; p < m.NV; p += L) {
            const double f_eq = f_maxwell<DIM>(k, rho, u, xi_of(m, p));
            face0[base + p] = (1.0 - c_eq) * face0[base + p] + c_eq * f_eq;
        }
        return;
    }
    double v[5] = {0, 0, 0, 0, 0};
    if (active)
        for (int p = lane; p < m.NV; p += L) {
            const double w = m.w[p];
            const V3 xi = xi_of(m, p);
            const double kk = dot<DIM>(xi, xi);
            const double g = face0[base + p], h = face1[base + p];
            v[0] += w * g;
            const double wg = w * g;
            v[1] += xi.x * wg;
            v[2] += xi.y * wg;
            if (DIM == 3) v[3] += xi.z * wg;
            v[4] += w * (kk * g + h);
        }
    seg_reduce<5>(v, L, sh);
    const double rho = v[0];
    const double r = 1.0 / rho;
    const V3 u = v3(v[1] * r, v[2] * r, v[3] * r);
    double m3[3] = {0, 0, 0};
    if (active)
        for (int p = lane; p < m.NV; p += L) {
            const double w = m.w[p];
            const V3 c = xi_of(m, p) - u;
            const double cc = dot<DIM>(c, c);
            const double g = face0[base + p], h = face1[base + p];
            const double s = cc * g + h;
            m3[0] += (c.x * w) * s;
            m3[1] += (c.y * w) * s;
            if (DIM == 3) m3[2] += (c.z * w) * s;
        }
    seg_reduce<3>(m3, L, sh);
    const double rhoE = 0.5 * v[4];
    const V3 hu = scl(u, 0.5);
    const double T = (rhoE / rho - dot<DIM>(hu, u)) / k.Cv;
    const double tau = tau_f(k, rho, T);
    const double qs = tau / (2.0 * tau + k.hdt * k.Pr);
    const V3 q = v3(m3[0] * qs, m3[1] * qs, m3[2] * qs);
    const double C_s = k.hdt / (2.0 * tau + k.hdt);
    const EqK64 e = make_eqk<DIM>(k, rho, T);
    if (DIM == 2 && m.ntx > 0) {  // tensor-product set: the exponential from two factor tables
        extern __shared__ double tabs[];
        double *t = tabs + (threadIdx.x / L) * (m.ntx + m.nty);
        exp_tables(m, u, e.oRT2, lane, L, t);
        __syncthreads();  // every thread of the block gets here (inactive segments too)
        if (!active) return;
        for (int p = lane; p < m.NV; p += L) {
            const V3 c = xi_of(m, p) - u;
            const double cc = dot<DIM>(c, c);
            const double cq = dot<DIM>(c, q);
            double g_s, h_s;
            shakhov_eq_gm(k, e, e.A * (t[m.tix[p]] * t[m.ntx + m.tiy[p]]), cc, cq, g_s, h_s);
            face0[base + p] = (1.0 - C_s) * face0[base + p] + C_s * g_s;
            face1[base + p] = (1.0 - C_s) * face1[base + p] + C_s * h_s;
        }
        return;
    }
    if (!active) return;
    for (int p = lane; p < m.NV; p += L) {
        const V3 c = xi_of(m, p) - u;
        const double cc = dot<DIM>(c, c);
        const double cq = dot<DIM>(c, q);
        double g_s, h_s;
        shakhov_eq(k, e, cc, cq, g_s, h_s);
        face0[base + p] = (1.0 - C_s) * face0[base + p] + C_s * g_s;
        face1[base + p] = (1.0 - C_s) * face1[base + p] + C_s * h_s;
    }
}

// ============================================================================
// boundary: one block per non-interior face; pass 1 then pass 2 of the
// reference (cdugks_shakhov.cpp:364-607, cdugks.cpp:185-277).  Faces are
// independent: each pass only reads and writes its own face row, and the
// symmetry / slip-wall mirror reads come from a per-face snapshot.
// ============================================================================
template <int DIM, bool SHAKHOV>
__global__ void __launch_bounds__(kBlock) k_boundary(DMesh m, KParams k, const DStatus *st, const double *rho_c,
                                                     const double *u_c, const double *T_c, double *face0,
                                                     double *face1, double *snap0, double *snap1) {
    __shared__ double sh[(kBlock / 32) * 2];
    if (step_stopped(st)) return;
    const int b = blockIdx.x;
    if (b >= m.nb) return;
    const int fi = m.bface[b];
    const meso_mark_desc mk = m.marks[m.fmark[fi]];
    const int L = blockDim.x;
    const int lane = threadIdx.x;
    const size_t NV = (size_t)m.NV;
    const size_t base = (size_t)fi * NV;
    const V3 nv = -ld3(m.fn, fi);  // normal_vector[1], into the domain
    const int nb = m.fown[fi];
    double *fg = face0 + base;
    double *fh = SHAKHOV ? face1 + base : nullptr;
    double *sg = snap0 + (size_t)b * NV;
    double *sgh = SHAKHOV ? snap1 + (size_t)b * NV : nullptr;
    const V3 u_w = v3(mk.velocity[0], mk.velocity[1], mk.velocity[2]);

    if (!SHAKHOV) {
        if (mk.type == MESO_BC_FARFIELD_INLET || mk.type == MESO_BC_FARFIELD_OUTLET) {
            const double rr = mk.type == MESO_BC_FARFIELD_INLET ? mk.density : rho_c[nb];
            const V3 uu = mk.type == MESO_BC_FARFIELD_INLET ? u_w : ld3(u_c, nb);
            for (int p = lane; p < m.NV; p += L) {
                const V3 xi = xi_of(m, p);
                if (dot<DIM>(xi, nv) >= kVSMALL) fg[p] = f_maxwell<DIM>(k, rr, uu, xi);
            }
        } else if (mk.type == MESO_BC_WALL) {
            double v[2] = {0.0, 0.0};  // rho_w, rho_w0
            for (int p = lane; p < m.NV; p += L) {
                const V3 xi = xi_of(m, p);
                const double kn = dot<DIM>(xi, nv);
                if (kn >= kVSMALL) v[1] += kn * m.w[p] * f_maxwell<DIM>(k, 1.0, u_w, xi);
                else v[0] -= kn * m.w[p] * fg[p];
            }
            seg_reduce<2>(v, L, sh);
            const double rho_w = v[0] / v[1];
            for (int p = lane; p < m.NV; p += L) {
                const V3 xi = xi_of(m, p);
                const double kn = dot<DIM>(xi, nv);
                if (kn >= kVSMALL) fg[p] = f_maxwell<DIM>(k, rho_w, u_w, xi);
                else if (!(kn < -kVSMALL)) fg[p] = 0.5 * (f_maxwell<DIM>(k, rho_w, u_w, xi) + fg[p]);
            }
        }
        return;
    }

    const int type = mk.type;
    if (type == MESO_BC_PRESSURE_INLET || type == MESO_BC_FARFIELD_INLET || type == MESO_BC_FREESTREAM_INLET ||
        type == MESO_BC_PRESSURE_OUTLET || type == MESO_BC_FARFIELD_OUTLET) {
        double rr, TT;
        V3 uu;
        if (type == MESO_BC_PRESSURE_INLET) {
            const double T_m = T_c[nb];
            const V3 u_m = ld3(u_c, nb);
            uu = scl(nv, dot<DIM>(u_m, nv));
            TT = mk.temperature;
            const double p_in = solve_pressure(mk.pressure, k.R, T_m, uu, k.gamma);
            rr = p_in / (k.R * TT);
        } else if (type == MESO_BC_FARFIELD_INLET) {
            rr = mk.density;
            uu = u_w;
            TT = mk.temperature;
        } else if (type == MESO_BC_FREESTREAM_INLET) {
            // intended form of cdugks_shakhov.cpp:419 (the reference divides the loop index)
            TT = mk.temperature;
            rr = mk.pressure / (k.R * TT);
            uu = u_w;
        } else if (type == MESO_BC_PRESSURE_OUTLET) {
            const V3 u_m = ld3(u_c, nb);
            const double T_m = T_c[nb];
            const double p_e = solve_pressure(mk.pressure, k.R, T_m, u_m, k.gamma);
            rr = p_e / (k.R * T_m);
            const V3 nv_e = -nv;
            uu = scl(nv_e, dot<DIM>(u_m, nv_e));
            TT = mk.temperature;
        } else {  // farfield outlet
            rr = rho_c[nb];
            TT = T_c[nb];
            uu = ld3(u_c, nb);
        }
        for (int p = lane; p < m.NV; p += L) {
            const V3 xi = xi_of(m, p);
            if (dot<DIM>(xi, nv) >= kVSMALL) {
                const V3 c = xi - uu;
                const double g_m = g_maxwell<DIM>(k, rr, TT, dot<DIM>(c, c));
                fg[p] = g_m;
                fh[p] = h_maxwell(k, TT, g_m);
            }
        }
        return;
    }
    if (type == MESO_BC_SYMMETRY) {
        const int dir = mk.direction;
        for (int p = lane; p < m.NV; p += L) {
            sg[p] = fg[p];
            sgh[p] = fh[p];
        }
        __syncthreads();
        for (int p = lane; p < m.NV; p += L) {
            const double kn = dot<DIM>(xi_of(m, p), nv);
            const int s = m.sym[3 * p + dir];
            if (kn >= kVSMALL) {
                fg[p] = sg[s];
                fh[p] = sgh[s];
            } else if (!(kn < -kVSMALL)) {
                fg[p] = 0.5 * (fg[p] + sg[s]);
                fh[p] = 0.5 * (fh[p] + sgh[s]);
            }
        }
        return;
    }
    if (type != MESO_BC_WALL && type != MESO_BC_SLIP_WALL) return;
    // pass 1: density balance (cdugks_shakhov.cpp:468-497)
    double T_w = 0.0;
    if (mk.temperature_type == MESO_PATCH_ZERO_GRADIENT) T_w = T_c[nb];
    else if (mk.temperature_type == MESO_PATCH_FIXED_VALUE) T_w = mk.temperature;
    double v[2] = {0.0, 0.0};
    for (int p = lane; p < m.NV; p += L) {
        const V3 xi = xi_of(m, p);
        const double kn = dot<DIM>(xi, nv);
        if (kn >= kVSMALL) {
            const V3 c = xi - u_w;
            const double g_m = g_maxwell<DIM>(k, 1.0, T_w, dot<DIM>(c, c));
            v[1] += kn * m.w[p] * g_m;
        } else {
            v[0] -= kn * m.w[p] * fg[p];
        }
    }
    seg_reduce<2>(v, L, sh);
    const double rho_w = v[0] / v[1];
    const double T_p = mk.temperature;
    // pass 2: incoming set (cdugks_shakhov.cpp:531-602)
    if (type == MESO_BC_WALL) {
        for (int p = lane; p < m.NV; p += L) {
            const V3 xi = xi_of(m, p);
            const double kn = dot<DIM>(xi, nv);
            if (kn >= kVSMALL) {
                const V3 c = xi - u_w;
                const double g_m = g_maxwell<DIM>(k, rho_w, T_p, dot<DIM>(c, c));
                fg[p] = g_m;
                fh[p] = h_maxwell(k, T_p, g_m);
            } else if (!(kn < -kVSMALL)) {
                const V3 c = xi - u_w;
                const double g_m = g_maxwell<DIM>(k, rho_w, T_p, dot<DIM>(c, c));
                const double h_m = h_maxwell(k, T_p, g_m);
                fg[p] = 0.5 * (g_m + fg[p]);
                fh[p] = 0.5 * (h_m + fh[p]);
            }
        }
        return;
    }
    // slip wall
    const int dir = mk.direction;
    const double au = mk.alpha_u, aT = mk.alpha_T;
    for (int p = lane; p < m.NV; p += L) {
        sg[p] = fg[p];
        sgh[p] = fh[p];
    }
    __syncthreads();
    for (int p = lane; p < m.NV; p += L) {
        const V3 xi = xi_of(m, p);
        const double kn = dot<DIM>(xi, nv);
        if (kn < -kVSMALL) continue;
        const V3 c = xi - u_w;
        const double g_m = g_maxwell<DIM>(k, rho_w, T_p, dot<DIM>(c, c));
        const double h_m = h_maxwell(k, T_p, g_m);
        const int s = m.sym[3 * p + dir];
        const double g_r = sg[s], h_r = sgh[s];
        if (kn >= kVSMALL) {
            fg[p] = (1.0 - au) * g_m + au * g_r;
            fh[p] = (1.0 - aT) * h_m + aT * h_r;
        } else {
            fg[p] = 0.5 * ((1.0 - au) * g_m + au * g_r + fg[p]);
            fh[p] = 0.5 * ((1.0 - aT) * h_m + aT * h_r + fh[p]);
        }
    }
}

// ============================================================================
// update: per cell, flux over the cell's faces, flux moments, macroscopic
// update, evolution to the next f-bar-plus, heat flux, NaN / T<0 monitor.
// ============================================================================
template <int DIM>
__device__ __forceinline__ double cell_flux(const DMesh &m, int c, int p, V3 xi, const double *face, double &fh_out,
                                            const double *face_h) {
    double fg = 0.0, fh = 0.0;
    const size_t NV = (size_t)m.NV;
    for (int j = m.cf_ptr[c]; j < m.cf_ptr[c + 1]; ++j) {
        const int fi = m.cf_face[j];
        V3 nv = ld3(m.fn, fi);
        if (m.fown[fi] != c) nv = -nv;
        const double knA = dot<DIM>(xi, nv) * m.farea[fi];
        fg += knA * face[(size_t)fi * NV + p];
        if (face_h) fh += knA * face_h[(size_t)fi * NV + p];
    }
    fh_out = fh;
    return fg;
}

template <int DIM>
__global__ void __launch_bounds__(kBlock) k_update_shakhov(DMesh m, KParams k, DStatus *st, int L, double *g_cell,
                                                           double *h_cell, const double *g_face, const double *h_face,
                                                           double *flux_g, double *flux_h, double *rho_c, double *u_c,
                                                           double *T_c, double *q_c, double *fm0, double *fm1,
                                                           double *fm2, int *repair_list) {
    __shared__ double sh[(kBlock / 32) * 5];
    if (step_stopped(st)) return;
    const int spb = kBlock / L;
    const int c = blockIdx.x * spb + threadIdx.x / L;
    const int lane = threadIdx.x % L;
    const bool active = c < m.C;
    const size_t NV = (size_t)m.NV;
    const size_t base = (size_t)(active ? c : 0) * NV;
    double v[5] = {0, 0, 0, 0, 0};
    if (active)
        for (int p = lane; p < m.NV; p += L) {
            const V3 xi = xi_of(m, p);
            double fh;
            const double fg = cell_flux<DIM>(m, c, p, xi, g_face, fh, h_face);
            flux_g[base + p] = fg;
            flux_h[base + p] = fh;
            const double w = m.w[p];
            v[0] += w * fg;
            const double wf = w * fg;
            v[1] += xi.x * wf;
            v[2] += xi.y * wf;
            if (DIM == 3) v[3] += xi.z * wf;
            v[4] += w * (dot<DIM>(xi, xi) * fg + fh);
        }
    seg_reduce<5>(v, L, sh);
    // macroscopic update (cdugks_shakhov.cpp:644-664)
    const int cc_ = active ? c : 0;
    const double dt_v = k.dt / m.vol[cc_];
    const double rho_n = rho_c[cc_];
    const V3 u_n = ld3(u_c, cc_);
    const double T_n = T_c[cc_];
    const V3 q_n = ld3(q_c, cc_);
    const V3 rhoU_n = scl(u_n, rho_n);
    const double rhoE_n = rho_n * (0.5 * dot<DIM>(u_n, u_n) + k.Cv * T_n);
    const double tau_n = tau_f(k, rho_n, T_n);
    const double rho = rho_n - dt_v * v[0];
    const V3 rhoU = rhoU_n - v3(v[1] * dt_v, v[2] * dt_v, v[3] * dt_v);
    const double rhoE = rhoE_n - dt_v * 0.5 * v[4];
    const double r = 1.0 / rho;
    const V3 u = scl(rhoU, r);
    const double T = (rhoE / rho - dot<DIM>(u, u) * 0.5) / k.Cv;
    const double tau = tau_f(k, rho, T);
    const double cm = k.hdt / (k.hdt - 2.0 * tau_n);
    const double Cc = tau / (tau + k.hdt);
    const double C_s = k.hdt / (2.0 * tau);
    const double itau = 1.0 / tau, itau_n = 1.0 / tau_n;
    const EqK64 e_n = make_eqk<DIM>(k, rho_n, T_n), e1 = make_eqk<DIM>(k, rho, T);
    // tensor-product set: the two equilibria's exponentials from factor tables (state n, then n+1)
    const bool tensor = DIM == 2 && m.ntx > 0;
    extern __shared__ double tabs[];
    const int nt = m.ntx + m.nty;
    double *tn = tabs + (threadIdx.x / L) * 2 * nt, *t1 = tn + nt;
    if (tensor) {
        exp_tables(m, u_n, e_n.oRT2, lane, L, tn);
        exp_tables(m, u, e1.oRT2, lane, L, t1);
        __syncthreads();  // every thread of the block gets here (inactive segments too)
    }
    double m3[3] = {0, 0, 0};
    if (active)
        for (int p = lane; p < m.NV; p += L) {
            const V3 xi = xi_of(m, p);
            const V3 c_n = xi - u_n;
            const double cc_n = dot<DIM>(c_n, c_n);
            const double cq_n = dot<DIM>(c_n, q_n);
            double g_s_n, h_s_n;
            const int ix = tensor ? m.tix[p] : 0, iy = tensor ? m.ntx + m.tiy[p] : 0;
            if (tensor) shakhov_eq_gm(k, e_n, e_n.A * (tn[ix] * tn[iy]), cc_n, cq_n, g_s_n, h_s_n);
            else shakhov_eq(k, e_n, cc_n, cq_n, g_s_n, h_s_n);
            const double g_n = cm * g_s_n + (1.0 - cm) * g_cell[base + p];
            const double h_n = cm * h_s_n + (1.0 - cm) * h_cell[base + p];
            const V3 cv = xi - u;
            const double cc = dot<DIM>(cv, cv);
            const double cq = dot<DIM>(cv, q_n);
            double g_s, h_s;
            if (tensor) shakhov_eq_gm(k, e1, e1.A * (t1[ix] * t1[iy]), cc, cq, g_s, h_s);
            else shakhov_eq(k, e1, cc, cq, g_s, h_s);
            const double g = Cc * (g_n + k.hdt * (g_s * itau + (g_s_n - g_n) * itau_n) - dt_v * flux_g[base + p]);
            const double h = Cc * (h_n + k.hdt * (h_s * itau + (h_s_n - h_n) * itau_n) - dt_v * flux_h[base + p]);
            const double hw = 0.5 * m.w[p];
            const double s = cc * g + h;
            m3[0] += (cv.x * hw) * s;
            m3[1] += (cv.y * hw) * s;
            if (DIM == 3) m3[2] += (cv.z * hw) * s;
            g_cell[base + p] = (1.0 - C_s) * g + C_s * g_s;
            h_cell[base + p] = (1.0 - C_s) * h + C_s * h_s;
        }
    seg_reduce<3>(m3, L, sh);
    if (!active || lane != 0) return;
    rho_c[c] = rho;
    st3(u_c, c, u);
    T_c[c] = T;
    st3(q_c, c, v3(m3[0], m3[1], m3[2]));
    fm0[c] = v[0];
    st3(fm1, c, v3(v[1], v[2], v[3]));
    fm2[c] = v[4];
    // monitor (cdugks_shakhov.cpp:697-719)
    const bool bad_rho = isnan(rho);
    const bool bad_T = (T < 0.0) || isnan(T);
    if (bad_rho || bad_T) {
        atomicAdd(&st->bad_count, 1);
        atomicMin(&st->first_bad, c);
        if (m.mask && m.mask[c]) {
            int slot = atomicAdd(&st->repair_count, 1);
            if (slot < m.C) repair_list[slot] = c;
        } else {
            atomicMin(&st->stop_step, st->step);
        }
    }
}

// BGK CDUGKS update (cdugks.cpp:281-335)
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_update_cdugks(DMesh m, KParams k, const DStatus *st, int L, double *f_cell,
                                                          const double *f_face, double *flux_f, double *rho_c,
                                                          double *u_c) {
    __shared__ double sh[(kBlock / 32) * 4];
    if (step_stopped(st)) return;
    const int spb = kBlock / L;
    const int c = blockIdx.x * spb + threadIdx.x / L;
    const int lane = threadIdx.x % L;
    const bool active = c < m.C;
    const size_t NV = (size_t)m.NV;
    const size_t base = (size_t)(active ? c : 0) * NV;
    double v[4] = {0, 0, 0, 0};
    if (active)
        for (int p = lane; p < m.NV; p += L) {
            const V3 xi = xi_of(m, p);
            double dummy;
            const double fl = cell_flux<DIM>(m, c, p, xi, f_face, dummy, nullptr);
            flux_f[base + p] = fl;
            const double w = m.w[p];
            v[0] += w * fl;
            const double wf = w * fl;
            v[1] += xi.x * wf;
            v[2] += xi.y * wf;
            if (DIM == 3) v[3] += xi.z * wf;
        }
    seg_reduce<4>(v, L, sh);
    const int cc_ = active ? c : 0;
    const double dt_v = k.dt / m.vol[cc_];
    const double rho_n = rho_c[cc_];
    const V3 u_n = ld3(u_c, cc_);
    const double rho = rho_n - dt_v * v[0];
    const double rn = 1.0 / rho_n;
    const V3 u = scl(scl(u_n, rho_n) - v3(v[1] * dt_v, v[2] * dt_v, v[3] * dt_v), rn);
    if (active)
        for (int p = lane; p < m.NV; p += L) {
            const V3 xi = xi_of(m, p);
            const double f_eq_n = f_maxwell<DIM>(k, rho_n, u_n, xi);
            const double f_n = k.cm * f_eq_n + (1.0 - k.cm) * f_cell[base + p];
            const double f_eq = f_maxwell<DIM>(k, rho, u, xi);
            f_cell[base + p] =
                (1.0 - k.c_eq) * (k.Cc * (f_n + k.hdt * (f_eq / k.tau + (f_eq_n - f_n) / k.tau) - dt_v * flux_f[base + p])) +
                k.c_eq * f_eq;
        }
    // all lanes must pass the same barriers before the segment's lane 0 stores
    __syncthreads();
    if (!active || lane != 0) return;
    rho_c[c] = rho;
    st3(u_c, c, u);
}

// Classic DUGKS update (dugks.cpp:282-344)
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_update_dugks(DMesh m, KParams k, const DStatus *st, int L, double *f_cell,
                                                         const double *f_face, double *rho_c, double *u_c) {
    __shared__ double sh[(kBlock / 32) * 4];
    if (step_stopped(st)) return;
    const int spb = kBlock / L;
    const int c = blockIdx.x * spb + threadIdx.x / L;
    const int lane = threadIdx.x % L;
    const bool active = c < m.C;
    const size_t NV = (size_t)m.NV;
    const size_t base = (size_t)(active ? c : 0) * NV;
    const int cc_ = active ? c : 0;
    const double dt_v = k.dt / m.vol[cc_];
    const double rho0 = rho_c[cc_];
    const V3 u0 = ld3(u_c, cc_);
    double v[4] = {0, 0, 0, 0};
    if (active)
        for (int p = lane; p < m.NV; p += L) {
            const V3 xi = xi_of(m, p);
            double dummy;
            const double fl = cell_flux<DIM>(m, c, p, xi, f_face, dummy, nullptr);
            const double f_eq = f_maxwell<DIM>(k, rho0, u0, xi);
            const double f_bp = f_cell[base + p];
            const double f_t = (1.0 - k.C_bp_to_t) * f_bp + k.C_bp_to_t * f_eq;
            const double f = (4.0 * f_bp - f_t) / 3.0 - dt_v * fl;
            f_cell[base + p] = f;
            const double w = m.w[p];
            v[0] += w * f;
            const double wf = w * f;
            v[1] += xi.x * wf;
            v[2] += xi.y * wf;
            if (DIM == 3) v[3] += xi.z * wf;
        }
    seg_reduce<4>(v, L, sh);
    const double rho = v[0];
    const double r = 1.0 / rho;
    const V3 u = v3(v[1] * r, v[2] * r, v[3] * r);
    if (active)
        for (int p = lane; p < m.NV; p += L) {
            const double f_eq = f_maxwell<DIM>(k, rho, u, xi_of(m, p));
            f_cell[base + p] = (1.0 - k.C_t_to_bp) * f_cell[base + p] + k.C_t_to_bp * f_eq;
        }
    __syncthreads();
    if (!active || lane != 0) return;
    rho_c[c] = rho;
    st3(u_c, c, u);
}

// ============================================================================
// initial(): equilibrium from macros; mode 0 recomputes the macros as moments.
// ============================================================================
template <int DIM, int SOLVER>
__global__ void __launch_bounds__(kBlock) k_init(DMesh m, KParams k, int L, int mode, double *f0, double *f1,
                                                 double *rho_c, double *u_c, double *T_c, double *q_c) {
    __shared__ double sh[(kBlock / 32) * 8];
    const int spb = kBlock / L;
    const int c = blockIdx.x * spb + threadIdx.x / L;
    const int lane = threadIdx.x % L;
    const bool active = c < m.C;
    const size_t NV = (size_t)m.NV;
    const int cc_ = active ? c : 0;
    const size_t base = (size_t)cc_ * NV;
    const double rho_p = rho_c[cc_];
    const V3 u_p = ld3(u_c, cc_);
    double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (SOLVER != MESO_SOLVER_CDUGKS_SHAKHOV) {
        if (active)
            for (int p = lane; p < m.NV; p += L) {
                const V3 xi = xi_of(m, p);
                const double f = f_maxwell<DIM>(k, rho_p, u_p, xi);
                f0[base + p] = f;
                const double w = m.w[p];
                v[0] += w * f;
                const double wf = w * f;
                v[1] += xi.x * wf;
                v[2] += xi.y * wf;
                if (DIM == 3) v[3] += xi.z * wf;
            }
        seg_reduce<8>(v, L, sh);
        if (!active || lane != 0 || mode != 0) return;
        const double r = 1.0 / v[0];
        rho_c[c] = v[0];
        st3(u_c, c, v3(v[1] * r, v[2] * r, v[3] * r));
        return;
    }
    const double T_p = T_c[cc_];
    const V3 q_p = ld3(q_c, cc_);
    if (active)
        for (int p = lane; p < m.NV; p += L) {
            const V3 xi = xi_of(m, p);
            const V3 c = xi - u_p;
            const double cc = dot<DIM>(c, c);
            double g, h;
            if (mode == 0) {
                g = g_maxwell<DIM>(k, rho_p, T_p, cc);
                h = h_maxwell(k, T_p, g);
            } else {
                const double cq = dot<DIM>(c, q_p);
                const double g_m = g_maxwell<DIM>(k, rho_p, T_p, cc);
                g = g_shakhov(k, rho_p, T_p, cc, cq, g_m);
                h = h_shakhov(k, rho_p, T_p, cc, cq, g_m);
            }
            f0[base + p] = g;
            f1[base + p] = h;
            const double w = m.w[p];
            const double kk = dot<DIM>(xi, xi);
            v[0] += w * g;
            const double wg = w * g;
            v[1] += xi.x * wg;
            v[2] += xi.y * wg;
            if (DIM == 3) v[3] += xi.z * wg;
            v[4] += w * (kk * g + h);
            const double s = cc * g + h;
            v[5] += (c.x * w) * s;
            v[6] += (c.y * w) * s;
            if (DIM == 3) v[7] += (c.z * w) * s;
        }
    seg_reduce<8>(v, L, sh);
    if (!active || lane != 0 || mode != 0) return;
    const double rho = v[0];
    const double rhoE = 0.5 * v[4];
    const double r = 1.0 / rho;
    const V3 u = v3(v[1] * r, v[2] * r, v[3] * r);
    const V3 hu = scl(u, 0.5);
    const double T = (rhoE / rho - dot<DIM>(hu, u)) / k.Cv;
    rho_c[c] = rho;
    st3(u_c, c, u);
    T_c[c] = T;
    st3(q_c, c, v3(v[5] * 0.5, v[6] * 0.5, v[7] * 0.5));
}

// Mask repair (cell_value_interp, cdugks_shakhov.cpp:766-789 with interp_IDW,
// mesh_numerical.cpp:51-94): inverse-distance macros from the neighbours,
// then Shakhov equilibrium at that cell.  One block per queued cell.
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_mask_repair(DMesh m, KParams k, DStatus *st, const int *repair_list,
                                                        double *g_cell, double *h_cell, double *rho_c, double *u_c,
                                                        double *T_c, double *q_c) {
    const int n = min(st->repair_count, m.C);
    for (int r = blockIdx.x; r < n; r += gridDim.x) {
        const int c = repair_list[r];
        double sw = 0.0, srho = 0.0, sT = 0.0;
        V3 su = v3(0, 0, 0), sq = v3(0, 0, 0);
        for (int j = m.cn_ptr[c]; j < m.cn_ptr[c + 1]; ++j) {
            const V3 dr = ld3(m.lsq_dr, j);
            const double wi = 1.0 / dot<3>(dr, dr);
            const int nb = m.cn_cell[j];
            sw += wi;
            srho += wi * rho_c[nb];
            sT += wi * T_c[nb];
            su = su + scl(ld3(u_c, nb), wi);
            sq = sq + scl(ld3(q_c, nb), wi);
        }
        const double rho = srho / sw, T = sT / sw;
        const double rs = 1.0 / sw;
        const V3 u = scl(su, rs), q = scl(sq, rs);
        const size_t base = (size_t)c * m.NV;
        for (int p = threadIdx.x; p < m.NV; p += blockDim.x) {
            const V3 cv = xi_of(m, p) - u;
            const double cc = dot<DIM>(cv, cv);
            const double cq = dot<DIM>(cv, q);
            const double gm = g_maxwell<DIM>(k, rho, T, cc);
            g_cell[base + p] = g_shakhov(k, rho, T, cc, cq, gm);
            h_cell[base + p] = h_shakhov(k, rho, T, cc, cq, gm);
        }
        if (threadIdx.x == 0) {
            rho_c[c] = rho;
            st3(u_c, c, u);
            T_c[c] = T;
            st3(q_c, c, q);
        }
    }
}

// Cell macros from the renumbered device arrays into one buffer in the caller's (original) cell
// order: rho [C], u [3C], T [C], q [3C], so that one copy brings them to the host.
__global__ void k_gather_macros(const double *__restrict__ rho, const double *__restrict__ u,
                                const double *__restrict__ T, const double *__restrict__ q,
                                const int *__restrict__ new2old, int C, double *__restrict__ out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < C; i += gridDim.x * blockDim.x) {
        const size_t o = (size_t)new2old[i], n = (size_t)C;
        out[o] = rho[i];
        out[4 * n + o] = T[i];
        for (int k = 0; k < 3; ++k) {
            out[n + 3 * o + k] = u[3 * (size_t)i + k];
            out[5 * n + 3 * o + k] = q[3 * (size_t)i + k];
        }
    }
}

// End of step: count the step unless an earlier step stopped the run.
__global__ void k_end_step(DStatus *st) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    if (step_stopped(st)) return;
    st->repairs_total += min(st->repair_count, INT_MAX);
    st->repair_count = 0;
    st->step += 1;
}

int seg_lanes(int nv) {
    if (nv <= 32) return 32;
    if (nv <= 64) return 64;
    if (nv <= 128) return 128;
    return 256;
}

int grid_for(size_t total, int sms) {
    size_t blocks = (total + kBlock - 1) / kBlock;
    size_t cap = (size_t)sms * 16;
    return (int)(blocks < cap ? (blocks > 0 ? blocks : 1) : cap);
}

template <int DIM>
int plain_step_dim(const PlainState &s, cudaStream_t stream, int64_t *launches, cudaEvent_t *ev) {
    auto mark = [&](int k) {
        if (ev) cudaEventRecord(ev[k], stream);
    };
    const DMesh &m = s.mesh;
    const KParams &k = s.kp;
    const int L = seg_lanes(m.NV);
    const int spb = kBlock / L;
    const int sms = s.num_sms;
    const size_t cv = (size_t)m.C * m.NV, fv = (size_t)m.F * m.NV;
    int64_t n = 0;
    mark(0);
    if (s.solver == MESO_SOLVER_CDUGKS_SHAKHOV) {
        if (k.gradient) {
            k_grad<DIM, 2><<<grid_for(cv, sms), kBlock, 0, stream>>>(m, s.status, s.f0, s.f1, s.grad0, s.grad1);
            ++n;
        }
        mark(1);
        k_recon<DIM, 2, true><<<grid_for(fv, sms), kBlock, 0, stream>>>(m, k, s.status, s.f0, s.f1, s.grad0, s.grad1,
                                                                         s.face0, s.face1);
        mark(2);
        const size_t tab = DIM == 2 && m.ntx > 0 ? sizeof(double) * (size_t)spb * (m.ntx + m.nty) : 0;
        k_face_eq<DIM, true><<<(m.F + spb - 1) / spb, kBlock, tab, stream>>>(m, k, s.status, L, s.face0, s.face1);
        mark(3);
        n += 2;
        if (m.nb > 0) {
            k_boundary<DIM, true><<<m.nb, L, 0, stream>>>(m, k, s.status, s.rho, s.u, s.T, s.face0, s.face1, s.snap0,
                                                          s.snap1);
            ++n;
        }
        mark(4);
        k_update_shakhov<DIM><<<(m.C + spb - 1) / spb, kBlock, 2 * tab, stream>>>(
            m, k, s.status, L, s.f0, s.f1, s.face0, s.face1, s.flux0, s.flux1, s.rho, s.u, s.T, s.q, s.fm0, s.fm1,
            s.fm2, s.repair_list);
        k_mask_repair<DIM><<<64, kBlock, 0, stream>>>(m, k, s.status, s.repair_list, s.f0, s.f1, s.rho, s.u, s.T, s.q);
        n += 2;
    } else {
        if (k.gradient) {
            k_grad<DIM, 1><<<grid_for(cv, sms), kBlock, 0, stream>>>(m, s.status, s.f0, nullptr, s.grad0, nullptr);
            ++n;
        }
        mark(1);
        k_recon<DIM, 1, false><<<grid_for(fv, sms), kBlock, 0, stream>>>(m, k, s.status, s.f0, nullptr, s.grad0,
                                                                          nullptr, s.face0, nullptr);
        mark(2);
        k_face_eq<DIM, false><<<(m.F + spb - 1) / spb, kBlock, 0, stream>>>(m, k, s.status, L, s.face0, nullptr);
        mark(3);
        n += 2;
        if (m.nb > 0) {
            k_boundary<DIM, false><<<m.nb, L, 0, stream>>>(m, k, s.status, s.rho, s.u, s.T, s.face0, nullptr, s.snap0,
                                                           nullptr);
            ++n;
        }
        mark(4);
        if (s.solver == MESO_SOLVER_CDUGKS)
            k_update_cdugks<DIM><<<(m.C + spb - 1) / spb, kBlock, 0, stream>>>(m, k, s.status, L, s.f0, s.face0,
                                                                               s.flux0, s.rho, s.u);
        else
            k_update_dugks<DIM><<<(m.C + spb - 1) / spb, kBlock, 0, stream>>>(m, k, s.status, L, s.f0, s.face0, s.rho,
                                                                              s.u);
        ++n;
    }
    mark(5);
    k_end_step<<<1, 32, 0, stream>>>(s.status);
    mark(6);
    ++n;
    if (launches) *launches += n;
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <int DIM>
int plain_init_dim(const PlainState &s, int mode, cudaStream_t stream) {
    const DMesh &m = s.mesh;
    const int L = seg_lanes(m.NV);
    const int spb = kBlock / L;
    const int blocks = (m.C + spb - 1) / spb;
    if (s.solver == MESO_SOLVER_CDUGKS_SHAKHOV)
        k_init<DIM, MESO_SOLVER_CDUGKS_SHAKHOV><<<blocks, kBlock, 0, stream>>>(m, s.kp, L, mode, s.f0, s.f1, s.rho,
                                                                               s.u, s.T, s.q);
    else if (s.solver == MESO_SOLVER_CDUGKS)
        k_init<DIM, MESO_SOLVER_CDUGKS><<<blocks, kBlock, 0, stream>>>(m, s.kp, L, mode, s.f0, nullptr, s.rho, s.u,
                                                                       nullptr, nullptr);
    else
        k_init<DIM, MESO_SOLVER_DUGKS><<<blocks, kBlock, 0, stream>>>(m, s.kp, L, mode, s.f0, nullptr, s.rho, s.u,
                                                                      nullptr, nullptr);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace

// This file is compiled once per dimension (MESO_PLAIN_DIM): the 2-D kernels with multiply-adds
// contracted, the 3-D ones with contraction off (see plain_fp64.h).
#if MESO_PLAIN_DIM == 3
int plain_step_d3(const PlainState &s, cudaStream_t stream, int64_t *launches, cudaEvent_t *ev) {
    return plain_step_dim<3>(s, stream, launches, ev);
}
int plain_init_d3(const PlainState &s, int mode, cudaStream_t stream) { return plain_init_dim<3>(s, mode, stream); }
#elif MESO_PLAIN_DIM == 2
const char *const kPlainPhases[] = {"k_grad", "k_recon", "k_face_eq", "k_boundary", "k_update+repair", "k_end_step"};

int plain_step(const PlainState &s, cudaStream_t stream, int64_t *launches, cudaEvent_t *ev) {
    return s.mesh.dim == 2 ? plain_step_dim<2>(s, stream, launches, ev) : plain_step_d3(s, stream, launches, ev);
}

int plain_init(const PlainState &s, int mode, cudaStream_t stream) {
    return s.mesh.dim == 2 ? plain_init_dim<2>(s, mode, stream) : plain_init_d3(s, mode, stream);
}

int gather_macros(const double *rho, const double *u, const double *T, const double *q, const int *new2old, int C,
                  double *out, int sms, cudaStream_t stream) {
    k_gather_macros<<<grid_for((size_t)C, sms), kBlock, 0, stream>>>(rho, u, T, q, new2old, C, out);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}
#else
#error "plain_fp64.cu is compiled with -DMESO_PLAIN_DIM=2 or -DMESO_PLAIN_DIM=3"
#endif

}  // namespace meso
