// Single-GPU renumbering: reverse Cuthill-McKee cell order and faces sorted
// by their (renumbered) owner, so the cells of a tile and the faces between
// them sit close together in HBM.  Orientation (which cell owns a face) is
// never changed, so per-face arithmetic is identical to the original order.
#pragma once

#include <vector>

#include "meso_gpu.h"

namespace meso_host {

struct Renumbering {
    std::vector<int> cell_new2old, cell_old2new;
    std::vector<int> face_new2old, face_old2new;
};

Renumbering renumber(const meso_mesh_desc &m, bool identity = false);

}  // namespace meso_host
