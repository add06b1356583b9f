// Host-visible interface of the plain FP64 step kernels (plain_fp64.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "device_common.cuh"

namespace meso {

// Device buffers of one plain-FP64 solve.  f1/face1/... are null for the BGK solvers.
struct PlainState {
    int solver;
    int num_sms;
    DMesh mesh;
    KParams kp;
    DStatus *status;
    double *f0, *f1;          // [C*NV] cell distributions (g, h for Shakhov)
    double *face0, *face1;    // [F*NV] face values
    double *grad0, *grad1;    // [C*NV*dim] gradients
    double *flux0, *flux1;    // [C*NV] cell fluxes
    double *snap0, *snap1;    // [nb*NV] boundary snapshots
    double *rho, *u, *T, *q;  // [C], [3C], [C], [3C]
    double *fm0, *fm1, *fm2;  // flux moments [C], [3C], [C]
    int *repair_list;         // [C]
};

constexpr int PLAIN_NPHASE = 6;
extern const char *const kPlainPhases[PLAIN_NPHASE];
// One step; ev (may be null) receives PLAIN_NPHASE + 1 events around the phases.
int plain_step(const PlainState &s, cudaStream_t stream, int64_t *launches, cudaEvent_t *ev = nullptr);
int plain_init(const PlainState &s, int mode, cudaStream_t stream);
// The 3-D step and initial state, from the second compilation of plain_fp64.cu: the 2-D kernels
// contract multiply-adds into FMAs (every 2-D parity gate holds at 1e-12 that way, and the FP64
// pipe bounds this form), the 3-D ones keep each product rounded on its own, as the reference's
// host arithmetic does (on the tetrahedral golden, contraction moved rho by 2e-11).
int plain_step_d3(const PlainState &s, cudaStream_t stream, int64_t *launches, cudaEvent_t *ev);
int plain_init_d3(const PlainState &s, int mode, cudaStream_t stream);
// rho [C], u [3C], T [C], q [3C] (renumbered, on the device) -> out [8C] in original cell order
// (rho, u, T, q one after the other), out[new2old[i]] = rho[i] and so on.
int gather_macros(const double *rho, const double *u, const double *T, const double *q, const int *new2old, int C,
                  double *out, int sms, cudaStream_t stream);

}  // namespace meso
