// Device set-up of one FP32 instance (tile plan, FP32 tables, state buffers)
// and of the launch state that runs one or several instances together.
#pragma once

#include <vector>

#include "kernels/fp32_step.h"
#include "tiles.h"

struct meso_ctx;

namespace meso_host {

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

// A piece of an instance's tile work: velocity chunks [ch0, ch1) of one tile, which write the
// tile's heat-flux partial row `grp`; `run` is the CTA the piece was cut for (-1: any CTA).
struct TilePiece {
    int tile, grp, ch0, ch1, run;
};
// The pieces of an instance (F32Inst::split, ngroup): each tile's chunks once, in pieces that are
// its groups 0, 1, ... (a split tile may have fewer than ngroup; its other partial rows are never
// written and stay as zeroed when allocated).
std::vector<TilePiece> tile_pieces(int ntile, int chunks, int ngroup, int split);
// Groups per tile of a split over `split` runs (the largest number of pieces of one tile).
int split_ngroup(int ntile, int chunks, int split);

}  // namespace meso_host
