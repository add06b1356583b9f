// A loaded case: Config + mesh + DVS + settings, flattened into the C-ABI
// descriptors of include/meso_gpu.h.  This is what the reference solver
// constructors build (cdugks.cpp:7-39, dugks.cpp:7-39,
// cdugks_shakhov.cpp:35-60) before their first step.
#pragma once

#include "config.h"
#include "meso_gpu.h"

#include <memory>

struct meso_case {
    MESO::Solver::Config config;
    MESO::fvmMesh::Mesh mesh;
    MESO::DVS::VelocitySet dvs;
    meso_params params{};
    std::string solver_name, case_name, case_dir;
    int32_t max_step = 100000, write_interval = 1000;
    int32_t read_np_data = 0, output_latest = 1, output_np = 0;

    // flattened tables (original .neu order)
    std::vector<double> cell_pos, cell_vol, lsq_w, lsq_dr, lsq_c, face_pos, face_area, face_normal;
    std::vector<int32_t> cell_group, cell_face_ptr, cell_face, cell_nbr_ptr, cell_nbr, face_cell, face_mark;
    std::vector<double> dvs_xi, dvs_w;
    std::vector<int32_t> dvs_sym;
    std::vector<meso_mark_desc> marks;  // one per mesh face group (index = Face::group_id)
    std::vector<std::string> mark_names;

    void mesh_desc(meso_mesh_desc &d) const;
    void dvs_desc(meso_dvs_desc &d) const;
    // Re-read [settings] (update_config) into params; returns true if anything changed.
    bool reload_settings();
    void initial_fields(double *rho, double *u, double *T, uint8_t *mask) const;
};

namespace meso_host {
// Builds a case; throws std::invalid_argument on malformed input.
std::unique_ptr<meso_case> load_case(const std::string &case_file);
// [settings] -> meso_params for the given solver (the reference's ctor + update_config reads).
void params_from_config(const MESO::Solver::Config &cfg, int solver, const MESO::fvmMesh::Mesh &mesh,
                        const MESO::DVS::VelocitySet &dvs, meso_params &p);
int solver_kind(const std::string &name);  // -1 if unknown
}  // namespace meso_host
