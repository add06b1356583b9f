/*
 * meso_oracle.h -- CPU restatement of the meso-lts step, TEST INFRASTRUCTURE.
 *
 * This library gives the results the GPU step is tested against, and the timed
 * CPU baseline.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load it; the product never does.
 *
 * It consumes the same flat descriptors as the product's C ABI
 * (include/meso_gpu.h) and follows the reference's loop structure and
 * arithmetic order line by line (src/solver/boltzmann/{cdugks,dugks,
 * cdugks_shakhov}.cpp), with distributions stored as the reference stores
 * them: [velocity][cell].  With nthreads > 1 the velocity set is split into
 * contiguous slices exactly as MESO::MPI::get_task_distribution does
 * (src/core/mesompi/mpi.cpp:60-70), every slice sums its own partial moments
 * and the partials are added in slice order -- the reference's DVS-parallel
 * MPI path on shared memory.  With nthreads == 1 it reproduces the
 * single-rank reference bit for bit (same libm, -ffp-contract=off).
 *
 * Parity is pinned against the reference binary built by oracle/build_ref.sh
 * (fixtures in tests/golden/).
 */
#ifndef MESO_ORACLE_H
#define MESO_ORACLE_H

#include <stdint.h>

#include "meso_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct meso_oracle meso_oracle;

int mo_create(const meso_mesh_desc *mesh, const meso_dvs_desc *dvs, const meso_mark_desc *marks, int32_t nmarks,
              const meso_params *params, const uint8_t *mask, int32_t nthreads, meso_oracle **out);
void mo_destroy(meso_oracle *o);
/* initial(): mode 0 = group-patch equilibrium + moment macros, mode 1 = read-np-data path */
int mo_init(meso_oracle *o, const double *rho, const double *u, const double *T, const double *q, int32_t mode);
/* nsteps x do_step(); stops when run_state turns false */
int mo_step(meso_oracle *o, int32_t nsteps, int32_t *steps_done);
int mo_get_macros(const meso_oracle *o, double *rho, double *u, double *T, double *q);
int mo_get_flux_moments(const meso_oracle *o, double *m0, double *m1, double *m2);
int mo_get_state(const meso_oracle *o, int32_t *step, int32_t *run_state, int32_t *converged, double *solution_time);
/* the last residual check's list (Res[Rho], Res[T], Res[u], ... in the reference's print order;
 * cdugks_shakhov.cpp:729-746, cdugks.cpp:343-355) and its length (0 before the first check) */
int mo_get_residual(const meso_oracle *o, double *list, int32_t *n);
/* test hook (2-D Shakhov only): after every step round the stored g - g0, h - h0 to FP32 (g0 the
 * Maxwellian at rho0, u = 0, T0), everything else staying FP64 -- the storage rounding of an
 * FP32-storage step in isolation; not part of the reference's algorithm */
int mo_set_storage_rounding(meso_oracle *o, int32_t on);
/* distribution of velocity p at cell c (d = 0: f or g, 1: h) */
double mo_get_f(const meso_oracle *o, int32_t d, int32_t p, int32_t c);
int mo_set_params(meso_oracle *o, const meso_params *params);

#ifdef __cplusplus
}
#endif
#endif
