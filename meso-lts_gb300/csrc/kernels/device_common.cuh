// Device-side tables and helpers shared by the step kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "meso_gpu.h"

namespace meso {

constexpr double kVSMALL = 1e-30;  // include/core/math.h:4
constexpr double kPI = 3.14159265358979323846;

// Renumbered mesh + DVS tables on the device (all FP64 geometry as built on the host).
struct DMesh {
    int dim, C, F, NV, nb;
    const double *vol;      // [C]
    const double *cpos;     // [C*3]
    const int *cf_ptr;      // [C+1]
    const int *cf_face;     // cell faces in the reference's local order
    const int *cn_ptr;      // [C+1]
    const int *cn_cell;     // neighbours
    const double *lsq_w;    // per neighbour entry
    const double *lsq_dr;   // per neighbour entry, 3 each
    const double *lsq_c;    // [C*9] Cx, Cy, Cz
    const int *fown, *fnei; // [F]
    const double *farea;    // [F]
    const double *fpos;     // [F*3]
    const double *fn;       // [F*3] normal_vector[0]
    const int *fmark;       // [F]
    const int *bface;       // [nb] faces whose mark is not fluid-interior
    const double *xix, *xiy, *xiz, *w;  // [NV]
    const int *sym;         // [NV*3]
    const meso_mark_desc *marks;
    const uint8_t *mask;    // [C] cell mask switch (may be null)
    // 2-D tensor-product velocity sets (NC, GH, hGH, D2Q9): xi_p = (tx[tix[p]], ty[tiy[p]]), so the
    // Maxwellian's exponential factors into one per component; ntx = 0 for other sets
    int ntx, nty;
    const double *tx, *ty;
    const int *tix, *tiy;
};

// Per-step scalars, derived on the host exactly as the reference derives them.
struct KParams {
    double dt, hdt;          // timeStep, half_dt
    double R, T0, Kd, Dd;    // gas constant, ref temperature, gas-k, dimension (as doubles)
    double Pr, mu0, vhs;     // Prandtl, ref viscosity, vhs index
    double Cv, gamma;        // (K+3)R/2, (K+5)/(K+3)
    double RT, over_RT, tau; // BGK: R*T0, 1/RT, relaxation time
    double cm, Cc, c_eq;     // BGK evolution constants (cdugks.cpp:306-308)
    double c_eq_face;        // BGK face blend (cdugks.cpp:171)
    double C_bp_to_t, C_t_to_bp;  // DUGKS (dugks.cpp:300,331)
    double venkata_k;
    int gradient, limiter;
};

// Device step/monitor state.  stop_step < step means a previous step produced
// an unmasked bad cell: every kernel of later steps returns at entry.
struct DStatus {
    int step;           // steps completed on the device
    int stop_step;      // first step with an unmasked NaN / T<0 cell (INT_MAX if none)
    int bad_count;      // bad cells seen (all steps)
    int first_bad;      // smallest renumbered id of a bad cell
    int repair_count;   // masked cells queued for repair this step
    int repairs_total;
    int timeout;        // a bounded device wait gave up (the step's results are invalid)
    int halt;           // set when the solve converges (k32_residual): it takes no more steps
};

__device__ __forceinline__ bool step_stopped(const DStatus *st) { return st->stop_step < st->step || st->halt; }

}  // namespace meso
