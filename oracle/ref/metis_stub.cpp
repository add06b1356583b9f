// METIS entry points for the reference build in oracle/_ref/.
//
// Test infrastructure only.  meso-lts calls METIS solely from
// Mesh::partition (src/mesh/metis.cpp:6-64), reached by the `--mesh` tool
// path and never by a solver step.  With one rank that function returns
// before calling METIS; these definitions only satisfy the linker.
#include "mesh/metis.h"

extern "C" {
int METIS_SetDefaultOptions(idx_t *options) {
    for (int i = 0; i < METIS_NOPTIONS; ++i) options[i] = -1;
    return METIS_OK;
}

int METIS_PartGraphKway(idx_t *nvtxs, idx_t *, idx_t *, idx_t *, idx_t *, idx_t *, idx_t *, idx_t *,
                        real_t *, real_t *, idx_t *, idx_t *objval, idx_t *part) {
    for (idx_t i = 0; i < *nvtxs; ++i) part[i] = 0;
    *objval = 0;
    return METIS_OK;
}
}
