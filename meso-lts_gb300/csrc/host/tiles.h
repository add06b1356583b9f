// Tile plan for the FP32 step: cells grouped into compact tiles, each tile
// with its one- and two-ring halo and the local stencils the kernels use.
//
// Tiles come from recursive coordinate bisection of the cell centroids, so a
// tile is a compact patch (its halo grows with its perimeter, not with its
// cell count); tiles are numbered in bisection order and the cells inside a
// tile by reverse Cuthill-McKee.  Faces are sorted by their owner, so the
// faces a tile owns form one contiguous range.
#pragma once

#include <cstdint>
#include <vector>

#include "meso_gpu.h"
#include "renumber.h"

namespace meso_host {

struct TilePlan {
    int ntile = 0, max_cells = 0, max_slots = 0, max_gslots = 0, max_owned = 0, max_gentries = 0, max_cf = 0;
    int max_tf = 0;
    std::vector<int> tile_cstart, tile_ncell;        // [ntile]
    std::vector<int> tile_slot_ptr, slot_cell;       // slots: tile cells, 1-ring halo, 2-ring halo
    std::vector<int> tile_gslots;                    // [ntile] slots with a gradient (tile + 1-ring)
    std::vector<int> tile_gsp_off;                   // [ntile] index in gs_ptr of the tile's first gradient slot
    std::vector<int> gs_ptr;                         // per gradient slot (+1 per tile): absolute entry offsets
    std::vector<uint16_t> gs_nbr;                    // neighbour slot per entry
    std::vector<float> gs_ax, gs_ay;                 // w_j (Cx . dr_j), w_j (Cy . dr_j)
    std::vector<int> tile_fstart;                    // [ntile+1] owned face range
    std::vector<uint16_t> face_own_slot, face_nei_slot;  // per face, in its owner tile
    // faces that touch a tile cell, each once per tile (the update kernel evaluates each once)
    std::vector<int> tile_tf_ptr;                    // [ntile+1]
    std::vector<int> tf_face;                        // renumbered face id
    std::vector<uint8_t> cf_tf;                      // per cell-face entry: tile-face index, | 0x80 when the cell
                                                     // is the face's neighbour (flux counted negative)
};

// Renumbering that tiles the mesh (cells grouped by tile, faces by owner).
Renumbering renumber_tiled(const meso_mesh_desc &m, int tile_cells, std::vector<int> &tile_sizes);

// Builds the tables on the renumbered mesh.  Returns false if a tile exceeds
// the kernel limits (slots, gradient slots, owned faces, cells).
bool build_tile_plan(const meso_mesh_desc &m, const Renumbering &rn, const std::vector<int> &tile_sizes,
                     int max_slots, int max_gslots, int max_owned, int max_cells, TilePlan &plan);

}  // namespace meso_host
