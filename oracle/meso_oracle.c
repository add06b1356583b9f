/*
 * meso_oracle.c -- CPU restatement of the meso-lts step.  TEST INFRASTRUCTURE:
 * the reference results the GPU library is tested against, and the timed CPU
 * baseline; see meso_oracle.h.  Every function cites the reference lines it restates
 * (paths relative to the meso-lts project root).  Compile with
 * -ffp-contract=off: expressions are written in the reference's evaluation
 * order and must not be contracted into FMAs.
 */
#define _POSIX_C_SOURCE 200809L
#include "meso_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define VSMALL 1e-30 /* include/core/math.h:4 */
#define PI 3.14159265358979323846

/* ---- Vector with the operator semantics of src/core/math/vector.cpp ------ */
typedef struct {
    double x, y, z;
} V;
static inline V vmk(double x, double y, double z) { V r = {x, y, z}; return r; }
static inline V vadd(V a, V b) { return vmk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V vsub(V a, V b) { return vmk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V vneg(V a) { return vmk(-a.x, -a.y, -a.z); }
static inline V vmul(V a, double s) { return vmk(a.x * s, a.y * s, a.z * s); }           /* Vector*s and s*Vector */
static inline V vdiv(V a, double s) { double r = 1.0 / s; return vmk(a.x * r, a.y * r, a.z * r); } /* :220-223 */
static inline double vdot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }       /* :233-235 */
static inline V vld(const double *p, int i) { return vmk(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }

typedef struct {
    int start, size;
} Slice;

struct meso_oracle {
    int dim, C, F, NV, solver, nth, nmarks;
    /* mesh, original order */
    double *vol;
    V *cpos;
    int *cf_ptr, *cf, *cn_ptr, *cn;
    double *lw;
    V *ldr, *Cx, *Cy, *Cz;
    int *fown, *fnei, *fmark;
    V *fpos, *fn0, *fn1;
    double *farea;
    meso_mark_desc *marks;
    uint8_t *mask;
    double total_volume;
    V *xi;
    double *w;
    int *sym;
    /* settings */
    meso_params par;
    double dt, half_dt, R, T0, Pr, miu0, vhs, Cv, gamma, venkata_k;
    int K, D;
    double RT, tau; /* BGK */
    /* fields: [p][id] as the reference's DistributionFunction */
    double *g, *h, *gf, *hf, *flux_g, *flux_h;
    double *rho, *T, *fm0, *fm2;
    V *u, *q, *fm1;
    /* per-step scratch */
    double *rho_new, *T_new, *tau_n, *tau_new;
    V *u_new;
    double *snap_g, *snap_h; /* [nb][NV] boundary snapshots */
    int *bface, nb, *bslot; /* boundary faces and face -> slot */
    double *wall_sum;        /* [nth][nb][2] */
    double *part;            /* [nth][max(C,F)][8] partial moments */
    double *red;             /* [max(C,F)][8] reduced moments */
    V *grad_g, *grad_h;      /* [nth][C] gradient scratch */
    /* residual state (solver.h:49, field.cpp:223-249) */
    double *rho_res, *T_res;
    V *u_res, *q_res;
    int step, run_state, converged, converge_state;
    double last_res[8]; /* the last check's residual list, in the reference's print order */
    int round_fp32;     /* test hook: round the stored g - g0, h - h0 to FP32 after every step, 1 to
                           nearest, 2 stochastically */
    int nres;
    double solution_time;
    Slice *slices;
    pthread_barrier_t bar;
    int stop_flag;
};

/* ---- get_task_distribution (src/core/mesompi/mpi.cpp:60-70) --------------- */
static void task_distribution(int total, int n, Slice *out) {
    int per = total / n, extra = total % n;
    for (int i = 0; i < n; ++i) {
        out[i].start = i * per + (i < extra ? i : extra);
        out[i].size = per + (i < extra ? 1 : 0);
    }
}

/* ---- equilibria: cdugks_shakhov.cpp:181-211, cdugks.cpp:116-121 ------------ */
static inline double tau_f(const meso_oracle *o, double rho, double t) {
    return o->miu0 * pow(t / o->T0, o->vhs) / (rho * o->R * t);
}
static inline double g_maxwell(const meso_oracle *o, double rho, double t, double cc) {
    if (o->D == 2) {
        double over_RT2 = 0.5 / (o->R * t);
        return rho * over_RT2 / PI * exp(-cc * over_RT2);
    }
    double RT = o->R * t;
    return rho / pow(2.0 * PI * RT, 1.5) * exp(-cc * 0.5 / RT);
}
static inline double h_maxwell(const meso_oracle *o, double t, double gm) { return (o->K + 3.0 - o->D) * (o->R * t) * gm; }
static inline double g_shakhov(const meso_oracle *o, double rho, double t, double cc, double cq, double gm) {
    double RT = o->R * t;
    double p = rho * RT;
    return (1.0 - o->Pr) * (cq / (5.0 * p * RT)) * (cc / RT - o->D - 2.0) * gm + gm;
}
static inline double h_shakhov(const meso_oracle *o, double rho, double t, double cc, double cq, double gm) {
    double RT = o->R * t;
    double p = rho * RT;
    double h_m = h_maxwell(o, t, gm);
    return (1.0 - o->Pr) * (cq / (5.0 * p)) * ((cc / RT - o->D) * (o->K + 3.0 - o->D) - 2.0 * o->K) * gm + h_m;
}
static inline double f_maxwell(const meso_oracle *o, double rho, V u, V xi) {
    double over_RT = 1.0 / o->RT;
    double ku_RT = vdot(u, xi) * over_RT;
    double uu_RT = vdot(u, u) * over_RT;
    return rho * (1.0 + ku_RT + (ku_RT * ku_RT - uu_RT) * 0.5);
}
/* Boundary::Compressible::solve_pressure (src/solver/boundary/pressure_boundary.cpp:15-18) */
static double solve_pressure(double P0, double R, double T, V U, double gamma) {
    double Ma = sqrt(U.x * U.x + U.y * U.y + U.z * U.z) / sqrt(gamma * R * T);
    return P0 / pow(1.0 + (gamma - 1.0) / 2.0 * (Ma * Ma), gamma / (gamma - 1.0));
}

#define G(a, p, i, n) ((a)[(size_t)(p) * (size_t)(n) + (size_t)(i)])

/* ---- fvmMesh::grad (src/mesh/mesh_numerical.cpp:24-49) --------------------- */
static void grad_field(const meso_oracle *o, const double *f, int p, V *out) {
    for (int c = 0; c < o->C; ++c) {
        V S = vmk(0.0, 0.0, 0.0);
        double fc = G(f, p, c, o->C);
        for (int j = o->cn_ptr[c]; j < o->cn_ptr[c + 1]; ++j) {
            double wj = o->lw[j];
            S = vadd(S, vmul(o->ldr[j], wj * (G(f, p, o->cn[j], o->C) - fc)));
        }
        out[c] = vmk(vdot(o->Cx[c], S), vdot(o->Cy[c], S), vdot(o->Cz[c], S));
    }
}

/* ---- venkata_limiter (src/solver/limiter.cpp:7-31) -------------------------- */
static double venkata(const meso_oracle *o, const double *f, int p, double dw, int cell, double k, double eps) {
    if (fabs(dw) <= eps) return 1.0;
    double kh = k * pow(o->vol[cell], 1.0 / (double)o->dim);
    double omega = kh * kh * kh;
    double w0 = G(f, p, cell, o->C), wmax = w0, wmin = w0;
    for (int j = o->cn_ptr[cell]; j < o->cn_ptr[cell + 1]; ++j) {
        double wn = G(f, p, o->cn[j], o->C);
        if (wn > wmax) wmax = wn;
        if (wn < wmin) wmin = wn;
    }
    double a = dw > 0.0 ? wmax - w0 : wmin - w0;
    double aa = a * a, ab = a * dw, bb = dw * dw;
    return (aa + 2.0 * ab + omega) / (aa + 2.0 * bb + ab + omega);
}

/* ---- face reconstruction of one velocity:
 *      cdugks.cpp:125-153 (BGK) and cdugks_shakhov.cpp:215-298 (Shakhov) ----- */
static void reconstruct_p(meso_oracle *o, int tid, int p, int ndist) {
    const int C = o->C, F = o->F;
    V *gr[2] = {o->grad_g + (size_t)tid * C, o->grad_h + (size_t)tid * C};
    double *fc[2] = {o->g, o->h};
    double *ff[2] = {o->gf, o->hf};
    V xi = o->xi[p];
    const int shakhov = o->solver == MESO_SOLVER_CDUGKS_SHAKHOV;
    const int grad_on = o->par.gradient_switch;
    const int lim = shakhov && o->par.limiter_switch;
    for (int d = 0; d < ndist; ++d) {
        if (grad_on) grad_field(o, fc[d], p, gr[d]);
        else if (!shakhov)
            for (int c = 0; c < C; ++c) gr[d][c] = vmk(0.0, 0.0, 0.0); /* zero_vector_field, cdugks.cpp:129 */
    }
    for (int fi = 0; fi < F; ++fi) {
        V nv = o->fn0[fi];
        int own = o->fown[fi], nei = o->fnei[fi];
        double nv_xi = vdot(nv, xi);
        for (int d = 0; d < ndist; ++d) {
            const double *f = fc[d];
            double val;
            if (shakhov && !grad_on) { /* zeroGradient branch, cdugks_shakhov.cpp:277-298 */
                if (nv_xi >= VSMALL) val = G(f, p, own, C);
                else if (nv_xi < -VSMALL) val = G(f, p, nei, C);
                else val = 0.5 * (G(f, p, own, C) + G(f, p, nei, C));
            } else if (nv_xi >= VSMALL) {
                V dr = vsub(o->fpos[fi], o->cpos[own]);
                double phi = 1.0;
                if (lim) phi = venkata(o, f, p, vdot(dr, gr[d][own]), own, o->venkata_k, 1.0e-10);
                double dd = vdot(vsub(dr, vmul(xi, o->half_dt)), gr[d][own]);
                val = G(f, p, own, C) + (shakhov ? phi * dd : dd);
            } else if (nv_xi < -VSMALL) {
                V dr = vsub(o->fpos[fi], o->cpos[nei]);
                double phi = 1.0;
                if (lim) phi = venkata(o, f, p, vdot(dr, gr[d][nei]), nei, o->venkata_k, VSMALL);
                double dd = vdot(vsub(dr, vmul(xi, o->half_dt)), gr[d][nei]);
                val = G(f, p, nei, C) + (shakhov ? phi * dd : dd);
            } else {
                V dro = vsub(o->fpos[fi], o->cpos[own]), drn = vsub(o->fpos[fi], o->cpos[nei]);
                double po = 1.0, pn = 1.0;
                if (lim) {
                    po = venkata(o, f, p, vdot(dro, gr[d][own]), own, o->venkata_k, VSMALL);
                    pn = venkata(o, f, p, vdot(drn, gr[d][nei]), nei, o->venkata_k, VSMALL);
                }
                double a = vdot(vsub(dro, vmul(xi, o->half_dt)), gr[d][own]);
                double b = vdot(vsub(drn, vmul(xi, o->half_dt)), gr[d][nei]);
                if (shakhov) val = 0.5 * (G(f, p, own, C) + G(f, p, nei, C) + po * a + pn * b);
                else val = 0.5 * (G(f, p, own, C) + G(f, p, nei, C) + a + b);
            }
            G(ff[d], p, fi, F) = val;
        }
    }
}

/* Sum the per-thread partials of `nv` values for items [lo, hi). */
static void reduce_partials(meso_oracle *o, int n_items, int nv, int lo, int hi) {
    for (int i = lo; i < hi; ++i)
        for (int k = 0; k < nv; ++k) {
            double s = 0.0;
            for (int t = 0; t < o->nth; ++t) {
                double v = o->part[((size_t)t * n_items + i) * 8 + k];
                s = (t == 0) ? v : s + v;
            }
            o->red[(size_t)i * 8 + k] = s;
        }
}

static inline void range_of(int n, int nth, int tid, int *lo, int *hi) {
    int per = (n + nth - 1) / nth;
    *lo = tid * per;
    *hi = *lo + per < n ? *lo + per : n;
    if (*lo > n) *lo = n;
}

static inline double *P8(meso_oracle *o, int tid, int n_items, int i) {
    return o->part + ((size_t)tid * n_items + i) * 8;
}

static void barrier(meso_oracle *o) {
    if (o->nth > 1) pthread_barrier_wait(&o->bar);
}

/* ============================================================================
 * One Shakhov step: reconstruct (cdugks_shakhov.cpp:213-608) and fvm_update
 * (:610-722), as executed by one velocity slice `tid`.
 * ==========================================================================*/
static void shakhov_step(meso_oracle *o, int tid) {
    const int C = o->C, F = o->F, NV = o->NV;
    const Slice sl = o->slices[tid];
    int lo, hi;
    (void)NV;
    for (int p = sl.start; p < sl.start + sl.size; ++p) reconstruct_p(o, tid, p, 2);
    barrier(o);
    /* face m0, m1, m2 (:300-322) */
    for (int fi = 0; fi < F; ++fi) {
        double *a = P8(o, tid, F, fi);
        double m0 = 0.0, m2 = 0.0;
        V m1 = vmk(0, 0, 0);
        for (int p = sl.start; p < sl.start + sl.size; ++p) {
            V xi = o->xi[p];
            double kk = vdot(xi, xi);
            double g = G(o->gf, p, fi, F), h = G(o->hf, p, fi, F);
            m0 += o->w[p] * g;
            m1 = vadd(m1, vmul(xi, o->w[p] * g));
            m2 += o->w[p] * (kk * g + h);
        }
        a[0] = m0; a[1] = m1.x; a[2] = m1.y; a[3] = m1.z; a[4] = m2;
    }
    barrier(o);
    range_of(F, o->nth, tid, &lo, &hi);
    reduce_partials(o, F, 5, lo, hi);
    barrier(o);
    /* face m3 with u (:323-339); keep m0..m2 in red[0..4] */
    for (int fi = 0; fi < F; ++fi) {
        const double *m = o->red + (size_t)fi * 8;
        double rho = m[0];
        V u = vdiv(vmk(m[1], m[2], m[3]), rho);
        V m3 = vmk(0, 0, 0);
        for (int p = sl.start; p < sl.start + sl.size; ++p) {
            V c = vsub(o->xi[p], u);
            double cc = vdot(c, c);
            double g = G(o->gf, p, fi, F), h = G(o->hf, p, fi, F);
            m3 = vadd(m3, vmul(vmul(c, o->w[p]), cc * g + h));
        }
        double *a = P8(o, tid, F, fi);
        a[5] = m3.x; a[6] = m3.y; a[7] = m3.z;
    }
    barrier(o);
    for (int i = lo; i < hi; ++i)
        for (int k = 5; k < 8; ++k) {
            double s = 0.0;
            for (int t = 0; t < o->nth; ++t) {
                double v = o->part[((size_t)t * F + i) * 8 + k];
                s = (t == 0) ? v : s + v;
            }
            o->red[(size_t)i * 8 + k] = s;
        }
    barrier(o);
    /* face equilibrium and blend (:340-362) */
    for (int fi = 0; fi < F; ++fi) {
        const double *m = o->red + (size_t)fi * 8;
        double rho = m[0];
        V rhoU = vmk(m[1], m[2], m[3]);
        double rhoE = 0.5 * m[4];
        V u = vdiv(rhoU, rho);
        double T = (rhoE / rho - vdot(vmul(u, 0.5), u)) / o->Cv;
        double tau = tau_f(o, rho, T);
        V q = vmul(vmk(m[5], m[6], m[7]), tau / (2.0 * tau + o->half_dt * o->Pr));
        double C_s = o->half_dt / (2.0 * tau + o->half_dt);
        for (int p = sl.start; p < sl.start + sl.size; ++p) {
            V c = vsub(o->xi[p], u);
            double cc = vdot(c, c), cq = vdot(c, q);
            double g_m = g_maxwell(o, rho, T, cc);
            double g_s = g_shakhov(o, rho, T, cc, cq, g_m);
            double h_s = h_shakhov(o, rho, T, cc, cq, g_m);
            G(o->gf, p, fi, F) = (1.0 - C_s) * G(o->gf, p, fi, F) + C_s * g_s;
            G(o->hf, p, fi, F) = (1.0 - C_s) * G(o->hf, p, fi, F) + C_s * h_s;
        }
    }
    barrier(o);
    /* snapshot of boundary face columns (the GatherFieldList reads of :501-502, :569-570) */
    range_of(o->nb, o->nth, tid, &lo, &hi);
    for (int b = lo; b < hi; ++b) {
        int fi = o->bface[b];
        for (int p = 0; p < o->NV; ++p) {
            o->snap_g[(size_t)b * o->NV + p] = G(o->gf, p, fi, F);
            o->snap_h[(size_t)b * o->NV + p] = G(o->hf, p, fi, F);
        }
    }
    barrier(o);
    /* boundary pass 1 (:364-522) */
    for (int b = 0; b < o->nb; ++b) {
        int fi = o->bface[b];
        const meso_mark_desc *mk = &o->marks[o->fmark[fi]];
        V nv = o->fn1[fi];
        int nb_ = o->fown[fi];
        V u_w = vmk(mk->velocity[0], mk->velocity[1], mk->velocity[2]);
        double *ws = o->wall_sum + ((size_t)tid * o->nb + b) * 2;
        ws[0] = ws[1] = 0.0;
        int type = mk->type;
        if (type == MESO_BC_PRESSURE_INLET || type == MESO_BC_FARFIELD_INLET || type == MESO_BC_FREESTREAM_INLET ||
            type == MESO_BC_PRESSURE_OUTLET || type == MESO_BC_FARFIELD_OUTLET) {
            double rr, TT;
            V uu;
            if (type == MESO_BC_PRESSURE_INLET) { /* :374-394 */
                double T_m = o->T[nb_];
                V u_m = o->u[nb_];
                uu = vmul(nv, vdot(u_m, nv));
                TT = mk->temperature;
                double p_in = solve_pressure(mk->pressure, o->R, T_m, uu, o->gamma);
                rr = p_in / (o->R * TT);
            } else if (type == MESO_BC_FARFIELD_INLET) { /* :395-411 */
                rr = mk->density;
                uu = u_w;
                TT = mk->temperature;
            } else if (type == MESO_BC_FREESTREAM_INLET) {
                /* :412-429 with the patch pressure (the reference divides the loop index, :419) */
                TT = mk->temperature;
                rr = mk->pressure / (o->R * TT);
                uu = u_w;
            } else if (type == MESO_BC_PRESSURE_OUTLET) { /* :430-452 */
                V u_m = o->u[nb_];
                double T_m = o->T[nb_];
                double p_e = solve_pressure(mk->pressure, o->R, T_m, u_m, o->gamma);
                rr = p_e / (o->R * T_m);
                V nv_e = vneg(nv);
                uu = vmul(nv_e, vdot(u_m, nv_e));
                TT = mk->temperature;
            } else { /* farfield outlet :453-467 */
                rr = o->rho[nb_];
                TT = o->T[nb_];
                uu = o->u[nb_];
            }
            for (int p = sl.start; p < sl.start + sl.size; ++p) {
                if (vdot(o->xi[p], nv) >= VSMALL) {
                    V c = vsub(o->xi[p], uu);
                    double g_m = g_maxwell(o, rr, TT, vdot(c, c));
                    G(o->gf, p, fi, F) = g_m;
                    G(o->hf, p, fi, F) = h_maxwell(o, TT, g_m);
                }
            }
        } else if (type == MESO_BC_WALL || type == MESO_BC_SLIP_WALL) { /* :468-497 */
            double T_w = 0.0;
            if (mk->temperature_type == MESO_PATCH_ZERO_GRADIENT) T_w = o->T[nb_];
            else if (mk->temperature_type == MESO_PATCH_FIXED_VALUE) T_w = mk->temperature;
            double rho_w = 0.0, rho_w0 = 0.0;
            for (int p = sl.start; p < sl.start + sl.size; ++p) {
                double kn = vdot(o->xi[p], nv);
                if (kn >= VSMALL) {
                    V c = vsub(o->xi[p], u_w);
                    double g_m = g_maxwell(o, 1.0, T_w, vdot(c, c));
                    rho_w0 += kn * o->w[p] * g_m;
                } else {
                    rho_w -= kn * o->w[p] * G(o->gf, p, fi, F);
                }
            }
            ws[0] = rho_w;
            ws[1] = rho_w0;
        } else if (type == MESO_BC_SYMMETRY) { /* :498-517 */
            int dir = mk->direction;
            const double *sg = o->snap_g + (size_t)b * o->NV, *sh = o->snap_h + (size_t)b * o->NV;
            for (int p = sl.start; p < sl.start + sl.size; ++p) {
                double kn = vdot(o->xi[p], nv);
                int s = o->sym[3 * p + dir];
                if (kn >= VSMALL) {
                    G(o->gf, p, fi, F) = sg[s];
                    G(o->hf, p, fi, F) = sh[s];
                } else {
                    if (kn < -VSMALL) continue;
                    G(o->gf, p, fi, F) = 0.5 * (G(o->gf, p, fi, F) + sg[s]);
                    G(o->hf, p, fi, F) = 0.5 * (G(o->hf, p, fi, F) + sh[s]);
                }
            }
        }
    }
    barrier(o);
    /* boundary pass 2 (:523-606) */
    for (int b = 0; b < o->nb; ++b) {
        int fi = o->bface[b];
        const meso_mark_desc *mk = &o->marks[o->fmark[fi]];
        if (mk->type != MESO_BC_WALL && mk->type != MESO_BC_SLIP_WALL) continue;
        double rw = 0.0, rw0 = 0.0;
        for (int t = 0; t < o->nth; ++t) {
            const double *ws = o->wall_sum + ((size_t)t * o->nb + b) * 2;
            rw = (t == 0) ? ws[0] : rw + ws[0];
            rw0 = (t == 0) ? ws[1] : rw0 + ws[1];
        }
        double rho_w = rw / rw0;
        V u_p = vmk(mk->velocity[0], mk->velocity[1], mk->velocity[2]);
        double T_p = mk->temperature;
        V nv = o->fn1[fi];
        if (mk->type == MESO_BC_WALL) {
            for (int p = sl.start; p < sl.start + sl.size; ++p) {
                double kn = vdot(o->xi[p], nv);
                if (kn >= VSMALL) {
                    V c = vsub(o->xi[p], u_p);
                    double g_m = g_maxwell(o, rho_w, T_p, vdot(c, c));
                    double h_m = h_maxwell(o, T_p, g_m);
                    G(o->gf, p, fi, F) = g_m;
                    G(o->hf, p, fi, F) = h_m;
                } else {
                    if (kn < -VSMALL) continue;
                    V c = vsub(o->xi[p], u_p);
                    double g_m = g_maxwell(o, rho_w, T_p, vdot(c, c));
                    double h_m = h_maxwell(o, T_p, g_m);
                    G(o->gf, p, fi, F) = 0.5 * (g_m + G(o->gf, p, fi, F));
                    G(o->hf, p, fi, F) = 0.5 * (h_m + G(o->hf, p, fi, F));
                }
            }
        } else {
            int dir = mk->direction;
            double au = mk->alpha_u, aT = mk->alpha_T;
            const double *sg = o->snap_g + (size_t)b * o->NV, *sh = o->snap_h + (size_t)b * o->NV;
            for (int p = sl.start; p < sl.start + sl.size; ++p) {
                double kn = vdot(o->xi[p], nv);
                if (kn >= VSMALL) {
                    V c = vsub(o->xi[p], u_p);
                    double g_m = g_maxwell(o, rho_w, T_p, vdot(c, c));
                    double h_m = h_maxwell(o, T_p, g_m);
                    double g_r = sg[o->sym[3 * p + dir]], h_r = sh[o->sym[3 * p + dir]];
                    G(o->gf, p, fi, F) = (1.0 - au) * g_m + au * g_r;
                    G(o->hf, p, fi, F) = (1.0 - aT) * h_m + aT * h_r;
                } else {
                    if (kn < -VSMALL) continue;
                    V c = vsub(o->xi[p], u_p);
                    double g_m = g_maxwell(o, rho_w, T_p, vdot(c, c));
                    double h_m = h_maxwell(o, T_p, g_m);
                    double g_r = sg[o->sym[3 * p + dir]], h_r = sh[o->sym[3 * p + dir]];
                    G(o->gf, p, fi, F) = 0.5 * ((1.0 - au) * g_m + au * g_r + G(o->gf, p, fi, F));
                    G(o->hf, p, fi, F) = 0.5 * ((1.0 - aT) * h_m + aT * h_r + G(o->hf, p, fi, F));
                }
            }
        }
    }
    barrier(o);
    /* flux and flux moments (:616-641) */
    for (int c = 0; c < C; ++c) {
        double m0 = 0.0, m2 = 0.0;
        V m1 = vmk(0, 0, 0);
        for (int p = sl.start; p < sl.start + sl.size; ++p) {
            V xi = o->xi[p];
            double fg = 0.0, fh = 0.0;
            for (int j = o->cf_ptr[c]; j < o->cf_ptr[c + 1]; ++j) {
                int fi = o->cf[j];
                V nv = (o->fown[fi] == c) ? o->fn0[fi] : o->fn1[fi];
                double knA = vdot(xi, nv) * o->farea[fi];
                fg += knA * G(o->gf, p, fi, F);
                fh += knA * G(o->hf, p, fi, F);
            }
            G(o->flux_g, p, c, C) = fg;
            G(o->flux_h, p, c, C) = fh;
            m0 += o->w[p] * fg;
            m1 = vadd(m1, vmul(xi, o->w[p] * fg));
            m2 += o->w[p] * (vdot(xi, xi) * fg + fh);
        }
        double *a = P8(o, tid, C, c);
        a[0] = m0; a[1] = m1.x; a[2] = m1.y; a[3] = m1.z; a[4] = m2;
    }
    barrier(o);
    range_of(C, o->nth, tid, &lo, &hi);
    reduce_partials(o, C, 5, lo, hi);
    /* macroscopic update (:644-668), per cell */
    for (int c = lo; c < hi; ++c) {
        const double *m = o->red + (size_t)c * 8;
        o->fm0[c] = m[0];
        o->fm1[c] = vmk(m[1], m[2], m[3]);
        o->fm2[c] = m[4];
        double dt_v = o->dt / o->vol[c];
        double rho_n = o->rho[c];
        V u_n = o->u[c];
        double T_n = o->T[c];
        V rhoU_n = vmul(u_n, rho_n);
        double rhoE_n = rho_n * (0.5 * vdot(u_n, u_n) + o->Cv * T_n);
        o->tau_n[c] = tau_f(o, rho_n, T_n);
        double rho = rho_n - dt_v * m[0];
        V rhoU = vsub(rhoU_n, vmul(o->fm1[c], dt_v));
        double rhoE = rhoE_n - dt_v * 0.5 * m[4];
        V u = vdiv(rhoU, rho);
        double T = (rhoE / rho - vdot(u, u) * 0.5) / o->Cv;
        o->rho_new[c] = rho;
        o->u_new[c] = u;
        o->T_new[c] = T;
        o->tau_new[c] = tau_f(o, rho, T);
    }
    barrier(o);
    /* evolution and heat flux (:666-696) */
    for (int c = 0; c < C; ++c) {
        double dt_v = o->dt / o->vol[c];
        double rho_n = o->rho[c], T_n = o->T[c], tau_n = o->tau_n[c];
        V u_n = o->u[c], q_n = o->q[c];
        double rho = o->rho_new[c], T = o->T_new[c], tau = o->tau_new[c];
        V u = o->u_new[c];
        double cm = o->half_dt / (o->half_dt - 2.0 * tau_n);
        double Cc = tau / (tau + o->half_dt);
        double C_s = o->half_dt / (2.0 * tau);
        V m3 = vmk(0, 0, 0);
        for (int p = sl.start; p < sl.start + sl.size; ++p) {
            V xi = o->xi[p];
            V c_n = vsub(xi, u_n);
            double cc_n = vdot(c_n, c_n), cq_n = vdot(c_n, q_n);
            double g_m_n = g_maxwell(o, rho_n, T_n, cc_n);
            double g_s_n = g_shakhov(o, rho_n, T_n, cc_n, cq_n, g_m_n);
            double h_s_n = h_shakhov(o, rho_n, T_n, cc_n, cq_n, g_m_n);
            double g_n = cm * g_s_n + (1.0 - cm) * G(o->g, p, c, C);
            double h_n = cm * h_s_n + (1.0 - cm) * G(o->h, p, c, C);
            V cv = vsub(xi, u);
            double cc = vdot(cv, cv), cq = vdot(cv, q_n);
            double g_m = g_maxwell(o, rho, T, cc);
            double g_s = g_shakhov(o, rho, T, cc, cq, g_m);
            double h_s = h_shakhov(o, rho, T, cc, cq, g_m);
            double g = Cc * (g_n + o->half_dt * (g_s / tau + (g_s_n - g_n) / tau_n) - dt_v * G(o->flux_g, p, c, C));
            double h = Cc * (h_n + o->half_dt * (h_s / tau + (h_s_n - h_n) / tau_n) - dt_v * G(o->flux_h, p, c, C));
            m3 = vadd(m3, vmul(vmul(cv, 0.5 * o->w[p]), cc * g + h));
            G(o->g, p, c, C) = (1.0 - C_s) * g + C_s * g_s;
            G(o->h, p, c, C) = (1.0 - C_s) * h + C_s * h_s;
        }
        double *a = P8(o, tid, C, c);
        a[5] = m3.x; a[6] = m3.y; a[7] = m3.z;
    }
    barrier(o);
}

/* interp_IDW of one cell (src/mesh/mesh_numerical.cpp:51-94) reading, for each
 * neighbour, the value the reference's cell loop sees at that point: cells
 * before `c` already updated, cells after it still at step n. */
static void mask_repair(meso_oracle *o, int c) {
    double sw = 0.0, sr = 0.0, sT = 0.0;
    V su = vmk(0, 0, 0), sq = vmk(0, 0, 0);
    for (int j = o->cn_ptr[c]; j < o->cn_ptr[c + 1]; ++j) {
        int nb = o->cn[j];
        double wi = 1.0 / vdot(o->ldr[j], o->ldr[j]);
        int upd = nb < c;
        sw += wi;
        sr += wi * (upd ? o->rho_new[nb] : o->rho[nb]);
        sT += wi * (upd ? o->T_new[nb] : o->T[nb]);
        su = vadd(su, vmul(upd ? o->u_new[nb] : o->u[nb], wi));
        sq = vadd(sq, vmul(o->q[nb], wi)); /* q_cell is replaced only after the cell loop */
    }
    double rho = sr / sw, T = sT / sw;
    V u = vdiv(su, sw), q = vdiv(sq, sw);
    o->rho_new[c] = rho;
    o->u_new[c] = u;
    o->T_new[c] = T;
    for (int p = 0; p < o->NV; ++p) {
        V cv = vsub(o->xi[p], u);
        double cc = vdot(cv, cv), cq = vdot(cv, q);
        double gm = g_maxwell(o, rho, T, cc);
        G(o->g, p, c, o->C) = g_shakhov(o, rho, T, cc, cq, gm);
        G(o->h, p, c, o->C) = h_shakhov(o, rho, T, cc, cq, gm);
    }
}

/* Monitor, commit and q (cdugks_shakhov.cpp:697-721); thread 0 only. */
static void shakhov_finish(meso_oracle *o) {
    const int C = o->C;
    for (int c = 0; c < C; ++c) {
        int bad = isnan(o->rho_new[c]);
        int badT = (o->T_new[c] < 0.0) || isnan(o->T_new[c]);
        for (int k = 0; k < bad + badT; ++k) {
            if (o->mask && o->mask[c]) mask_repair(o, c);
            else o->run_state = 0;
        }
    }
    reduce_partials(o, C, 8, 0, C);
    for (int c = 0; c < C; ++c) {
        const double *m = o->red + (size_t)c * 8;
        o->rho[c] = o->rho_new[c];
        o->u[c] = o->u_new[c];
        o->T[c] = o->T_new[c];
        o->q[c] = vmk(m[5], m[6], m[7]);
    }
}

/* ============================================================================
 * BGK solvers: CDUGKS (cdugks.cpp:123-335) and DUGKS (dugks.cpp:124-344).
 * ==========================================================================*/
static void bgk_step(meso_oracle *o, int tid) {
    const int C = o->C, F = o->F;
    const Slice sl = o->slices[tid];
    int lo, hi;
    const double half_dt = o->half_dt, tau = o->tau;
    for (int p = sl.start; p < sl.start + sl.size; ++p) reconstruct_p(o, tid, p, 1);
    barrier(o);
    /* face m0, m1 (cdugks.cpp:154-170) */
    for (int fi = 0; fi < F; ++fi) {
        double m0 = 0.0;
        V m1 = vmk(0, 0, 0);
        for (int p = sl.start; p < sl.start + sl.size; ++p) {
            double f = G(o->gf, p, fi, F);
            m0 += o->w[p] * f;
            m1 = vadd(m1, vmul(o->xi[p], o->w[p] * f));
        }
        double *a = P8(o, tid, F, fi);
        a[0] = m0; a[1] = m1.x; a[2] = m1.y; a[3] = m1.z;
    }
    barrier(o);
    range_of(F, o->nth, tid, &lo, &hi);
    reduce_partials(o, F, 4, lo, hi);
    barrier(o);
    /* blend (:171-183) */
    double c_eq = half_dt / (2.0 * tau + half_dt);
    for (int fi = 0; fi < F; ++fi) {
        const double *m = o->red + (size_t)fi * 8;
        double rho = m[0];
        V u = vdiv(vmk(m[1], m[2], m[3]), rho);
        for (int p = sl.start; p < sl.start + sl.size; ++p) {
            double f_eq = f_maxwell(o, rho, u, o->xi[p]);
            G(o->gf, p, fi, F) = (1.0 - c_eq) * G(o->gf, p, fi, F) + c_eq * f_eq;
        }
    }
    barrier(o);
    /* boundary (:185-277) */
    for (int b = 0; b < o->nb; ++b) {
        int fi = o->bface[b];
        const meso_mark_desc *mk = &o->marks[o->fmark[fi]];
        V nv = o->fn1[fi];
        int nb_ = o->fown[fi];
        V u_w = vmk(mk->velocity[0], mk->velocity[1], mk->velocity[2]);
        double *ws = o->wall_sum + ((size_t)tid * o->nb + b) * 2;
        ws[0] = ws[1] = 0.0;
        if (mk->type == MESO_BC_FARFIELD_INLET || mk->type == MESO_BC_FARFIELD_OUTLET) {
            double rr = mk->type == MESO_BC_FARFIELD_INLET ? mk->density : o->rho[nb_];
            V uu = mk->type == MESO_BC_FARFIELD_INLET ? u_w : o->u[nb_];
            for (int p = sl.start; p < sl.start + sl.size; ++p)
                if (vdot(o->xi[p], nv) >= VSMALL) G(o->gf, p, fi, F) = f_maxwell(o, rr, uu, o->xi[p]);
        } else if (mk->type == MESO_BC_WALL) {
            double rho_w = 0.0, rho_w0 = 0.0;
            for (int p = sl.start; p < sl.start + sl.size; ++p) {
                double kn = vdot(o->xi[p], nv);
                if (kn >= VSMALL) rho_w0 += kn * o->w[p] * f_maxwell(o, 1.0, u_w, o->xi[p]);
                else rho_w -= kn * o->w[p] * G(o->gf, p, fi, F);
            }
            ws[0] = rho_w;
            ws[1] = rho_w0;
        }
    }
    barrier(o);
    for (int b = 0; b < o->nb; ++b) {
        int fi = o->bface[b];
        const meso_mark_desc *mk = &o->marks[o->fmark[fi]];
        if (mk->type != MESO_BC_WALL) continue;
        double rw = 0.0, rw0 = 0.0;
        for (int t = 0; t < o->nth; ++t) {
            const double *ws = o->wall_sum + ((size_t)t * o->nb + b) * 2;
            rw = (t == 0) ? ws[0] : rw + ws[0];
            rw0 = (t == 0) ? ws[1] : rw0 + ws[1];
        }
        V nv = o->fn1[fi];
        V u_w = vmk(mk->velocity[0], mk->velocity[1], mk->velocity[2]);
        for (int p = sl.start; p < sl.start + sl.size; ++p) {
            double kn = vdot(o->xi[p], nv);
            if (kn >= VSMALL) {
                double rho_w = rw / rw0;
                G(o->gf, p, fi, F) = f_maxwell(o, rho_w, u_w, o->xi[p]);
            } else {
                if (kn < -VSMALL) continue;
                double rho_w = rw / rw0;
                G(o->gf, p, fi, F) = 0.5 * (f_maxwell(o, rho_w, u_w, o->xi[p]) + G(o->gf, p, fi, F));
            }
        }
    }
    barrier(o);
    if (o->solver == MESO_SOLVER_CDUGKS) {
        /* flux and flux moments (cdugks.cpp:283-304) */
        for (int c = 0; c < C; ++c) {
            double m0 = 0.0;
            V m1 = vmk(0, 0, 0);
            for (int p = sl.start; p < sl.start + sl.size; ++p) {
                V xi = o->xi[p];
                double flux = 0.0;
                for (int j = o->cf_ptr[c]; j < o->cf_ptr[c + 1]; ++j) {
                    int fi = o->cf[j];
                    V nv = (o->fown[fi] == c) ? o->fn0[fi] : o->fn1[fi];
                    flux += vdot(xi, nv) * o->farea[fi] * G(o->gf, p, fi, F);
                }
                G(o->flux_g, p, c, C) = flux;
                m0 += o->w[p] * flux;
                m1 = vadd(m1, vmul(xi, o->w[p] * flux));
            }
            double *a = P8(o, tid, C, c);
            a[0] = m0; a[1] = m1.x; a[2] = m1.y; a[3] = m1.z;
        }
        barrier(o);
        range_of(C, o->nth, tid, &lo, &hi);
        reduce_partials(o, C, 4, lo, hi);
        barrier(o);
        /* update and evolution (:306-333) */
        double cm = half_dt / (half_dt - 2.0 * tau);
        double Cc = tau / (tau + half_dt);
        double c_eq2 = half_dt / (2.0 * tau);
        for (int c = 0; c < C; ++c) {
            const double *m = o->red + (size_t)c * 8;
            double dt_v = o->dt / o->vol[c];
            double rho_n = o->rho[c];
            V u_n = o->u[c];
            double rho = rho_n - dt_v * m[0];
            V u = vdiv(vsub(vmul(u_n, rho_n), vmul(vmk(m[1], m[2], m[3]), dt_v)), rho_n);
            if (c >= lo && c < hi) {
                o->rho_new[c] = rho;
                o->u_new[c] = u;
            }
            for (int p = sl.start; p < sl.start + sl.size; ++p) {
                V xi = o->xi[p];
                double f_eq_n = f_maxwell(o, rho_n, u_n, xi);
                double f_n = cm * f_eq_n + (1.0 - cm) * G(o->g, p, c, C);
                double f_eq = f_maxwell(o, rho, u, xi);
                G(o->g, p, c, C) = (1.0 - c_eq2) * (Cc * (f_n + half_dt * (f_eq / tau + (f_eq_n - f_n) / tau) -
                                                          dt_v * G(o->flux_g, p, c, C))) +
                                   c_eq2 * f_eq;
            }
        }
        barrier(o);
    } else {
        /* DUGKS: flux, f-tilde update, moments, f-bar-plus (dugks.cpp:282-344) */
        double C_bp_to_t = (o->dt + half_dt) / (half_dt - 2.0 * tau);
        for (int c = 0; c < C; ++c) {
            double dt_v = o->dt / o->vol[c];
            double rho = o->rho[c];
            V u = o->u[c];
            double m0 = 0.0;
            V m1 = vmk(0, 0, 0);
            for (int p = sl.start; p < sl.start + sl.size; ++p) {
                V xi = o->xi[p];
                double flux = 0.0;
                for (int j = o->cf_ptr[c]; j < o->cf_ptr[c + 1]; ++j) {
                    int fi = o->cf[j];
                    V nv = (o->fown[fi] == c) ? o->fn0[fi] : o->fn1[fi];
                    flux += vdot(xi, nv) * o->farea[fi] * G(o->gf, p, fi, F);
                }
                double f_eq = f_maxwell(o, rho, u, xi);
                double f_bp = G(o->g, p, c, C);
                double f_t = (1.0 - C_bp_to_t) * f_bp + C_bp_to_t * f_eq;
                double f = (4.0 * f_bp - f_t) / 3.0 - dt_v * flux;
                G(o->g, p, c, C) = f;
                m0 += o->w[p] * f;
                m1 = vadd(m1, vmul(xi, o->w[p] * f));
            }
            double *a = P8(o, tid, C, c);
            a[0] = m0; a[1] = m1.x; a[2] = m1.y; a[3] = m1.z;
        }
        barrier(o);
        range_of(C, o->nth, tid, &lo, &hi);
        reduce_partials(o, C, 4, lo, hi);
        barrier(o);
        double C_t_to_bp = (o->dt + half_dt) / (2.0 * tau + o->dt);
        for (int c = 0; c < C; ++c) {
            const double *m = o->red + (size_t)c * 8;
            double rho = m[0];
            V u = vdiv(vmk(m[1], m[2], m[3]), rho);
            if (c >= lo && c < hi) {
                o->rho_new[c] = rho;
                o->u_new[c] = u;
            }
            for (int p = sl.start; p < sl.start + sl.size; ++p) {
                double f_eq = f_maxwell(o, rho, u, o->xi[p]);
                G(o->g, p, c, C) = (1.0 - C_t_to_bp) * G(o->g, p, c, C) + C_t_to_bp * f_eq;
            }
        }
        barrier(o);
    }
}

/* ---- residual and convergence (field.cpp:223-249, core.cpp:45-51) --------- */
static double res_s(const meso_oracle *o, double *old, const double *nw) {
    double r = 0.0;
    for (int c = 0; c < o->C; ++c) r += fabs((nw[c] - old[c]) / old[c]) * (o->vol[c] / o->total_volume);
    memcpy(old, nw, sizeof(double) * o->C);
    return r;
}
static V res_v(const meso_oracle *o, V *old, const V *nw) {
    V r = vmk(0, 0, 0);
    for (int c = 0; c < o->C; ++c) {
        V v = vmk(fabs((nw[c].x - old[c].x) / old[c].x), fabs((nw[c].y - old[c].y) / old[c].y),
                  fabs((nw[c].z - old[c].z) / old[c].z));
        r = vadd(r, vmul(v, o->vol[c] / o->total_volume));
    }
    memcpy(old, nw, sizeof(V) * o->C);
    return r;
}

/* do_step bookkeeping after the physics (cdugks_shakhov.cpp:727-757 etc.) */
static void after_step(meso_oracle *o) {
    o->step++;
    o->solution_time += o->dt;
    int ri = o->par.residual_interval;
    if (ri <= 0 || o->step % ri != 0) return;
    double list[8];
    int n = 0;
    double rr = res_s(o, o->rho_res, o->rho);
    V ru = res_v(o, o->u_res, o->u);
    if (o->solver == MESO_SOLVER_CDUGKS_SHAKHOV) {
        double rT = res_s(o, o->T_res, o->T);
        V rq = res_v(o, o->q_res, o->q);
        list[n++] = rr;
        list[n++] = rT;
        list[n++] = ru.x;
        list[n++] = ru.y;
        if (o->dim == 3) list[n++] = ru.z;
        list[n++] = rq.x;
        list[n++] = rq.y;
        if (o->dim == 3) list[n++] = rq.z;
    } else {
        list[n++] = rr;
        list[n++] = ru.x;
        list[n++] = ru.y;
        if (o->dim == 3) list[n++] = ru.z;
    }
    int conv = 1;
    for (int i = 0; i < n; ++i) conv = conv && (list[i] <= o->par.residual_limit);
    for (int i = 0; i < n; ++i) o->last_res[i] = list[i];
    o->nres = n;
    if (conv) o->converge_state++;
    else o->converge_state = 0;
    if (o->converge_state >= 10) {
        o->run_state = 0;
        o->converged = 1;
    }
}

/* Test hook (not part of the reference's algorithm): the stored distributions rounded as a
 * storage of g - g0 and h - h0 in FP32 would round them, with g0 the Maxwellian at (rho0, u = 0,
 * T0) and h0 = (K + 1) R T0 g0 (2-D), everything else in FP64.  Isolates the storage rounding of
 * an FP32-storage step. */
/* 32-bit mix of (a, b, c) (a multiply-xorshift hash), uniform in [0, 1) as a double */
static double hash_unit(uint32_t a, uint32_t b, uint32_t c) {
    uint32_t h = a * 0x9E3779B1u ^ (b + 0x7F4A7C15u) * 0x85EBCA77u ^ (c + 0x165667B1u) * 0xC2B2AE3Du;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    h *= 0x297A2D39u;
    h ^= h >> 15;
    return (double)h * (1.0 / 4294967296.0);
}

/* x rounded to FP32: to nearest (mode 1) or stochastically (mode 2: up with probability equal to
   the distance from the float below, in units of the gap, drawn from hash_unit(key...)) */
static double to_fp32(double x, int mode, uint32_t k0, uint32_t k1, uint32_t k2) {
    const float f = (float)x;
    if (mode != 2 || (double)f == x) return (double)f;
    const float lo = (double)f < x ? f : nextafterf(f, -INFINITY);
    const float hi = nextafterf(lo, INFINITY);
    const double p = (x - (double)lo) / ((double)hi - (double)lo);
    return hash_unit(k0, k1, k2) < p ? (double)hi : (double)lo;
}

static void round_state_fp32(meso_oracle *o) {
    const double RT0 = o->R * o->T0, over = 0.5 / RT0;
    const int mode = o->round_fp32;
    for (int p = 0; p < o->NV; ++p) {
        const double x = o->xi[p].x, y = o->xi[p].y;
        const double g0 = o->par.rho0 * over / PI * exp(-(x * x + y * y) * over);
        const double h0 = (o->K + 1.0) * RT0 * g0;
        for (int c = 0; c < o->C; ++c) {
            double *gp = &G(o->g, p, c, o->C), *hp = &G(o->h, p, c, o->C);
            *gp = g0 + to_fp32(*gp - g0, mode, (uint32_t)c, (uint32_t)(2 * p), (uint32_t)o->step);
            *hp = h0 + to_fp32(*hp - h0, mode, (uint32_t)c, (uint32_t)(2 * p + 1), (uint32_t)o->step);
        }
    }
}

typedef struct {
    meso_oracle *o;
    int tid, nsteps, *done;
} Job;

static void *run_steps(void *arg) {
    Job *j = (Job *)arg;
    meso_oracle *o = j->o;
    for (int s = 0; s < j->nsteps; ++s) {
        if (o->stop_flag) break;
        if (o->solver == MESO_SOLVER_CDUGKS_SHAKHOV) {
            shakhov_step(o, j->tid);
            if (j->tid == 0) shakhov_finish(o);
            if (j->tid == 0 && o->round_fp32) round_state_fp32(o);
        } else {
            bgk_step(o, j->tid);
            if (j->tid == 0) {
                memcpy(o->rho, o->rho_new, sizeof(double) * o->C);
                memcpy(o->u, o->u_new, sizeof(V) * o->C);
            }
        }
        if (j->tid == 0) {
            after_step(o);
            (*j->done)++;
            if (!o->run_state) o->stop_flag = 1;
        }
        barrier(o);
    }
    return NULL;
}

/* ---------------------------------------------------------------- public API */
static void *xcalloc(size_t n, size_t s) { return calloc(n ? n : 1, s); }

static void set_params(meso_oracle *o, const meso_params *p) {
    o->par = *p;
    o->dt = p->dt;
    o->half_dt = o->solver == MESO_SOLVER_CDUGKS_SHAKHOV ? p->dt * 0.5 : 0.5 * p->dt;
    o->R = p->R;
    o->T0 = p->T0;
    o->Pr = p->Pr;
    o->miu0 = p->mu0;
    o->vhs = p->vhs_index;
    o->K = p->K;
    o->gamma = (o->K + 5.0) / (o->K + 3.0);
    o->Cv = (o->K + 3.0) * o->R * 0.5;
    o->venkata_k = p->venkata_k;
    if (o->solver != MESO_SOLVER_CDUGKS_SHAKHOV) {
        o->RT = p->R * p->T0;
        double c_sound = sqrt(o->RT);
        o->tau = (p->L0 * p->Ma) / (p->Re * c_sound);
    }
}

int mo_create(const meso_mesh_desc *m, const meso_dvs_desc *d, const meso_mark_desc *marks, int32_t nmarks,
              const meso_params *par, const uint8_t *mask, int32_t nthreads, meso_oracle **out) {
    if (!m || !d || !marks || !par || !out || m->ncell <= 0 || d->nv <= 0) return MESO_ERR_INVALID;
    meso_oracle *o = (meso_oracle *)calloc(1, sizeof(meso_oracle));
    int C = m->ncell, F = m->nface, NV = d->nv;
    o->dim = m->dim;
    o->D = m->dim;
    o->C = C;
    o->F = F;
    o->NV = NV;
    o->solver = par->solver;
    o->nth = nthreads < 1 ? 1 : (nthreads > NV ? NV : nthreads);
    o->nmarks = nmarks;
    o->total_volume = m->total_volume;
    o->vol = (double *)xcalloc(C, sizeof(double));
    o->cpos = (V *)xcalloc(C, sizeof(V));
    o->Cx = (V *)xcalloc(C, sizeof(V));
    o->Cy = (V *)xcalloc(C, sizeof(V));
    o->Cz = (V *)xcalloc(C, sizeof(V));
    o->cf_ptr = (int *)xcalloc(C + 1, sizeof(int));
    o->cn_ptr = (int *)xcalloc(C + 1, sizeof(int));
    int nf = m->cell_face_ptr[C], nn = m->cell_nbr_ptr[C];
    o->cf = (int *)xcalloc(nf, sizeof(int));
    o->cn = (int *)xcalloc(nn, sizeof(int));
    o->lw = (double *)xcalloc(nn, sizeof(double));
    o->ldr = (V *)xcalloc(nn, sizeof(V));
    memcpy(o->vol, m->cell_vol, sizeof(double) * C);
    memcpy(o->cf_ptr, m->cell_face_ptr, sizeof(int) * (C + 1));
    memcpy(o->cn_ptr, m->cell_nbr_ptr, sizeof(int) * (C + 1));
    memcpy(o->cf, m->cell_face, sizeof(int) * nf);
    memcpy(o->cn, m->cell_nbr, sizeof(int) * nn);
    if (nn) memcpy(o->lw, m->lsq_w, sizeof(double) * nn);
    for (int j = 0; j < nn; ++j) o->ldr[j] = vld(m->lsq_dr, j);
    for (int c = 0; c < C; ++c) {
        o->cpos[c] = vld(m->cell_pos, c);
        o->Cx[c] = vld(m->lsq_c, 3 * c);
        o->Cy[c] = vld(m->lsq_c, 3 * c + 1);
        o->Cz[c] = vld(m->lsq_c, 3 * c + 2);
    }
    o->fown = (int *)xcalloc(F, sizeof(int));
    o->fnei = (int *)xcalloc(F, sizeof(int));
    o->fmark = (int *)xcalloc(F, sizeof(int));
    o->fpos = (V *)xcalloc(F, sizeof(V));
    o->fn0 = (V *)xcalloc(F, sizeof(V));
    o->fn1 = (V *)xcalloc(F, sizeof(V));
    o->farea = (double *)xcalloc(F, sizeof(double));
    o->marks = (meso_mark_desc *)xcalloc(nmarks, sizeof(meso_mark_desc));
    memcpy(o->marks, marks, sizeof(meso_mark_desc) * nmarks);
    o->bface = (int *)xcalloc(F, sizeof(int));
    for (int f = 0; f < F; ++f) {
        o->fown[f] = m->face_cell[2 * f];
        o->fnei[f] = m->face_cell[2 * f + 1];
        o->fmark[f] = m->face_mark[f];
        o->fpos[f] = vld(m->face_pos, f);
        o->fn0[f] = vld(m->face_normal, f);
        o->fn1[f] = vneg(o->fn0[f]);
        o->farea[f] = m->face_area[f];
        if (o->fmark[f] < 0 || o->fmark[f] >= nmarks) {
            mo_destroy(o);
            return MESO_ERR_INVALID;
        }
        if (marks[o->fmark[f]].type != MESO_BC_FLUID_INTERIOR) o->bface[o->nb++] = f;
    }
    if (mask) {
        o->mask = (uint8_t *)xcalloc(C, 1);
        memcpy(o->mask, mask, C);
    }
    o->xi = (V *)xcalloc(NV, sizeof(V));
    o->w = (double *)xcalloc(NV, sizeof(double));
    o->sym = (int *)xcalloc(3 * (size_t)NV, sizeof(int));
    for (int p = 0; p < NV; ++p) {
        o->xi[p] = vld(d->xi, p);
        o->w[p] = d->w[p];
        if (d->sym)
            for (int k = 0; k < 3; ++k) o->sym[3 * p + k] = d->sym[3 * p + k];
    }
    meso_params pp = *par;
    if (pp.solver == MESO_SOLVER_DUGKS) {
        double mm = d->max_magnitude;
        pp.dt = pp.CFL * (m->min_cell_size / mm); /* dugks.cpp:47 */
    }
    set_params(o, &pp);
    size_t cv = (size_t)C * NV, fv = (size_t)F * NV;
    int two = o->solver == MESO_SOLVER_CDUGKS_SHAKHOV;
    o->g = (double *)xcalloc(cv, sizeof(double));
    o->h = two ? (double *)xcalloc(cv, sizeof(double)) : NULL;
    o->gf = (double *)xcalloc(fv, sizeof(double));
    o->hf = two ? (double *)xcalloc(fv, sizeof(double)) : NULL;
    o->flux_g = (double *)xcalloc(cv, sizeof(double));
    o->flux_h = two ? (double *)xcalloc(cv, sizeof(double)) : NULL;
    o->rho = (double *)xcalloc(C, sizeof(double));
    o->T = (double *)xcalloc(C, sizeof(double));
    o->u = (V *)xcalloc(C, sizeof(V));
    o->q = (V *)xcalloc(C, sizeof(V));
    o->fm0 = (double *)xcalloc(C, sizeof(double));
    o->fm2 = (double *)xcalloc(C, sizeof(double));
    o->fm1 = (V *)xcalloc(C, sizeof(V));
    o->rho_new = (double *)xcalloc(C, sizeof(double));
    o->T_new = (double *)xcalloc(C, sizeof(double));
    o->tau_n = (double *)xcalloc(C, sizeof(double));
    o->tau_new = (double *)xcalloc(C, sizeof(double));
    o->u_new = (V *)xcalloc(C, sizeof(V));
    o->snap_g = (double *)xcalloc((size_t)(o->nb ? o->nb : 1) * NV, sizeof(double));
    o->snap_h = (double *)xcalloc((size_t)(o->nb ? o->nb : 1) * NV, sizeof(double));
    o->wall_sum = (double *)xcalloc((size_t)o->nth * (o->nb ? o->nb : 1) * 2, sizeof(double));
    size_t items = (size_t)(C > F ? C : F);
    o->part = (double *)xcalloc((size_t)o->nth * items * 8, sizeof(double));
    o->red = (double *)xcalloc(items * 8, sizeof(double));
    o->grad_g = (V *)xcalloc((size_t)o->nth * C, sizeof(V));
    o->grad_h = (V *)xcalloc((size_t)o->nth * C, sizeof(V));
    o->rho_res = (double *)xcalloc(C, sizeof(double));
    o->T_res = (double *)xcalloc(C, sizeof(double));
    o->u_res = (V *)xcalloc(C, sizeof(V));
    o->q_res = (V *)xcalloc(C, sizeof(V));
    o->slices = (Slice *)xcalloc(o->nth, sizeof(Slice));
    task_distribution(NV, o->nth, o->slices);
    if (!o->g || !o->gf || !o->flux_g || !o->part || (two && (!o->h || !o->hf || !o->flux_h))) {
        mo_destroy(o);
        return MESO_ERR_OOM;
    }
    if (o->nth > 1) pthread_barrier_init(&o->bar, NULL, (unsigned)o->nth);
    *out = o;
    return MESO_OK;
}

void mo_destroy(meso_oracle *o) {
    if (!o) return;
    void *ptrs[] = {o->vol, o->cpos, o->Cx, o->Cy, o->Cz, o->cf_ptr, o->cn_ptr, o->cf, o->cn, o->lw, o->ldr,
                    o->fown, o->fnei, o->fmark, o->fpos, o->fn0, o->fn1, o->farea, o->marks, o->bface, o->mask,
                    o->xi, o->w, o->sym, o->g, o->h, o->gf, o->hf, o->flux_g, o->flux_h, o->rho, o->T, o->u,
                    o->q, o->fm0, o->fm2, o->fm1, o->rho_new, o->T_new, o->tau_n, o->tau_new, o->u_new,
                    o->snap_g, o->snap_h, o->wall_sum, o->part, o->red, o->grad_g, o->grad_h, o->rho_res,
                    o->T_res, o->u_res, o->q_res, o->slices};
    for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); ++i) free(ptrs[i]);
    if (o->nth > 1) pthread_barrier_destroy(&o->bar);
    free(o);
}

/* initial() (cdugks.cpp:41-114, dugks.cpp:41-115, cdugks_shakhov.cpp:62-179) */
int mo_init(meso_oracle *o, const double *rho, const double *u, const double *T, const double *q, int32_t mode) {
    if (!o || !rho || !u) return MESO_ERR_INVALID;
    const int C = o->C, NV = o->NV;
    const int shakhov = o->solver == MESO_SOLVER_CDUGKS_SHAKHOV;
    if (shakhov && !T) return MESO_ERR_INVALID;
    for (int c = 0; c < C; ++c) {
        double r = rho[c];
        V uu = vld(u, c);
        double TT = T ? T[c] : 0.0;
        V qq = (q && shakhov) ? vld(q, c) : vmk(0, 0, 0);
        double m0 = 0.0, m2 = 0.0;
        V m1 = vmk(0, 0, 0), m3 = vmk(0, 0, 0);
        for (int p = 0; p < NV; ++p) {
            V xi = o->xi[p];
            if (!shakhov) {
                double f = f_maxwell(o, r, uu, xi);
                G(o->g, p, c, C) = f;
                m0 += o->w[p] * f;
                m1 = vadd(m1, vmul(xi, o->w[p] * f));
            } else if (mode == 0) {
                V cv = vsub(xi, uu);
                double cc = vdot(cv, cv);
                double kk = vdot(xi, xi);
                double g = g_maxwell(o, r, TT, cc);
                double h = h_maxwell(o, TT, g);
                G(o->g, p, c, C) = g;
                G(o->h, p, c, C) = h;
                m0 += o->w[p] * g;
                m1 = vadd(m1, vmul(xi, o->w[p] * g));
                m2 += o->w[p] * (kk * g + h);
                m3 = vadd(m3, vmul(vmul(cv, o->w[p]), cc * g + h));
            } else {
                V cv = vsub(xi, uu);
                double cc = vdot(cv, cv), cq = vdot(cv, qq);
                double g_m = g_maxwell(o, r, TT, cc);
                G(o->g, p, c, C) = g_shakhov(o, r, TT, cc, cq, g_m);
                G(o->h, p, c, C) = h_shakhov(o, r, TT, cc, cq, g_m);
            }
        }
        if (mode == 0) {
            o->rho[c] = m0;
            o->u[c] = vdiv(m1, m0);
            if (shakhov) {
                double rhoE = 0.5 * m2;
                V uc = vdiv(m1, m0);
                o->T[c] = (rhoE / m0 - vdot(vmul(uc, 0.5), uc)) / o->Cv;
                o->q[c] = vmul(m3, 0.5);
            }
        } else {
            o->rho[c] = r;
            o->u[c] = uu;
            o->T[c] = TT;
            o->q[c] = qq;
        }
    }
    memcpy(o->rho_res, o->rho, sizeof(double) * C);
    memcpy(o->u_res, o->u, sizeof(V) * C);
    memcpy(o->T_res, o->T, sizeof(double) * C);
    memcpy(o->q_res, o->q, sizeof(V) * C);
    o->step = 0;
    o->solution_time = 0.0;
    o->run_state = 1;
    o->converged = 0;
    o->converge_state = 0;
    return MESO_OK;
}

int mo_step(meso_oracle *o, int32_t nsteps, int32_t *steps_done) {
    if (!o || nsteps < 0) return MESO_ERR_INVALID;
    int done = 0;
    o->stop_flag = !o->run_state;
    if (o->nth == 1) {
        Job j = {o, 0, nsteps, &done};
        run_steps(&j);
    } else {
        pthread_t *th = (pthread_t *)calloc(o->nth, sizeof(pthread_t));
        Job *jobs = (Job *)calloc(o->nth, sizeof(Job));
        for (int t = 0; t < o->nth; ++t) {
            jobs[t].o = o;
            jobs[t].tid = t;
            jobs[t].nsteps = nsteps;
            jobs[t].done = &done;
        }
        for (int t = 1; t < o->nth; ++t) pthread_create(&th[t], NULL, run_steps, &jobs[t]);
        run_steps(&jobs[0]);
        for (int t = 1; t < o->nth; ++t) pthread_join(th[t], NULL);
        free(th);
        free(jobs);
    }
    if (steps_done) *steps_done = done;
    return (!o->run_state && !o->converged) ? MESO_ERR_NAN : MESO_OK;
}

int mo_get_macros(const meso_oracle *o, double *rho, double *u, double *T, double *q) {
    if (!o) return MESO_ERR_INVALID;
    for (int c = 0; c < o->C; ++c) {
        if (rho) rho[c] = o->rho[c];
        if (u) { u[3 * c] = o->u[c].x; u[3 * c + 1] = o->u[c].y; u[3 * c + 2] = o->u[c].z; }
        if (T) T[c] = o->T[c];
        if (q) { q[3 * c] = o->q[c].x; q[3 * c + 1] = o->q[c].y; q[3 * c + 2] = o->q[c].z; }
    }
    return MESO_OK;
}

int mo_get_flux_moments(const meso_oracle *o, double *m0, double *m1, double *m2) {
    if (!o) return MESO_ERR_INVALID;
    for (int c = 0; c < o->C; ++c) {
        if (m0) m0[c] = o->fm0[c];
        if (m1) { m1[3 * c] = o->fm1[c].x; m1[3 * c + 1] = o->fm1[c].y; m1[3 * c + 2] = o->fm1[c].z; }
        if (m2) m2[c] = o->fm2[c];
    }
    return MESO_OK;
}

int mo_get_state(const meso_oracle *o, int32_t *step, int32_t *run_state, int32_t *converged, double *t) {
    if (!o) return MESO_ERR_INVALID;
    if (step) *step = o->step;
    if (run_state) *run_state = o->run_state;
    if (converged) *converged = o->converged;
    if (t) *t = o->solution_time;
    return MESO_OK;
}

int mo_set_storage_rounding(meso_oracle *o, int32_t on) {
    if (!o || o->solver != MESO_SOLVER_CDUGKS_SHAKHOV || o->dim != 2) return MESO_ERR_INVALID;
    if (on < 0 || on > 2) return MESO_ERR_INVALID;
    o->round_fp32 = on;
    return MESO_OK;
}

int mo_get_residual(const meso_oracle *o, double *list, int32_t *n) {
    if (!o || !list || !n) return MESO_ERR_INVALID;
    for (int i = 0; i < o->nres; ++i) list[i] = o->last_res[i];
    *n = o->nres;
    return MESO_OK;
}

double mo_get_f(const meso_oracle *o, int32_t d, int32_t p, int32_t c) {
    const double *a = d == 0 ? o->g : o->h;
    if (!a || p < 0 || p >= o->NV || c < 0 || c >= o->C) return NAN;
    return G(a, p, c, o->C);
}

int mo_set_params(meso_oracle *o, const meso_params *p) {
    if (!o || !p || p->solver != o->solver) return MESO_ERR_INVALID;
    set_params(o, p);
    return MESO_OK;
}
