// Device set-up of one FP32 instance (tile plan, FP32 tables, state buffers)
// and of the launch state that runs one or several instances together.
#pragma once

#include <vector>

#include "kernels/fp32_step.h"
#include "tiles.h"

struct meso_ctx;

namespace meso_host {

// Tile size, velocity groups per tile: chosen by the autotuner or the defaults.
struct Fp32Tuning {
    int tile_cells = 64;
    int ngroup = 0;  // 0: pick from the SM count
};

// Renumbering + tile plan that fits the kernel limits (shrinks the tile size until it does).
bool plan_fp32(const meso_mesh_desc &m, int tile_cells, Renumbering &rn, TilePlan &plan);

// Allocates and uploads the instance of context c (c->rn must be the tiled renumbering).
int build_fp32_instance(meso_ctx *c, const meso_mesh_desc *m, const meso_dvs_desc *d, const TilePlan &plan,
                        int ngroup, int vpl = 0);

// Launch state over a list of instances (device copies of their F32Inst + work items).
int build_fp32_launch(const std::vector<meso::F32Inst> &insts, int num_sms, meso::Fp32State &s,
                      std::vector<void *> &owned);
void free_fp32_launch(meso::Fp32State &s, std::vector<void *> &owned);

int default_ngroup(int ntile, int chunks, int num_sms);

}  // namespace meso_host
