// meso_solver.hpp -- C++ drop-in for the meso-lts solver classes, over the C-ABI of meso_gpu.h.
//
// The reference runs each solve through handle_solver<SolverClass> (src/meso/exec.cpp:141-165):
//
//     SolverClass solver(parser, config);
//     solver.initial();
//     solver.output();
//     for (int i = 0; (i < solver.max_step()) || (solver.max_step() < 0); ++i) {
//         solver.do_step();
//         if (not solver.get_run_state()) break;
//         if (solver.step % solver.write_interval() == 0) solver.output();
//     }
//     solver.output();
//
// MESO::GPU::Solver has the members that loop and output() use, with the reference's names and
// meaning (include/solver/boltzmann/cdugks_shakhov.h:4-60, include/solver/solver.h:22-46): step,
// solution_time, rho_cell, vel_cell, T_cell, q_cell, mesh and dvs_mesh (read-only views),
// initial(), do_step(), output(), get_run_state(), max_step(), write_interval().  One class serves the three solver kinds; the case
// file's "solver" key picks the kind, as main.cpp:49-54 does.  Errors surface as the reference's
// exceptions: std::invalid_argument for bad input, std::runtime_error otherwise.  The macroscopic
// Fields are copied from the device when read through sync() (do_step() syncs at the residual
// interval and when the run state turns false, output() and the destructor need no sync).
#ifndef MESO_SOLVER_HPP
#define MESO_SOLVER_HPP

#include <fstream>
#include <functional>
#include <iomanip>
#include <stdexcept>
#include <string>
#include <vector>

#include <algorithm>
#include <cstdio>

#include "meso_gpu.h"

namespace MESO {
namespace GPU {

// Vector and Field<T>: the parts of include/core/vector.h and include/mesh/object.h:42-75 a caller
// of the solver reads: len, flag, values, operator[], get_mesh, MeshCellValueToField, heft,
// set_zero and output (field.cpp:98-173).
struct Vector {
    double x = 0.0, y = 0.0, z = 0.0;
    double &operator[](int k) { return k == 0 ? x : (k == 1 ? y : z); }
    double operator[](int k) const { return k == 0 ? x : (k == 1 ? y : z); }
};

// Read-only views of the solver's mesh and velocity mesh (include/mesh/object.h:93-128,
// include/mesh/mesh.h): the members a caller of the solver reads; the geometry itself lives in
// the library.
struct CellView {
    int id = 0;
    Vector position;
    double volume = 0.0;
    std::vector<int> face_id, neighbors;
};
struct FaceView {
    int id = 0;
    Vector position;
    double area = 0.0;
    int cell_id[2] = {-1, -1};
    Vector normal_vector[2];
};
struct MeshView {
    int NCELL = 0, NFACE = 0, NDFVL = 2;
    double total_volume = 0.0, min_cell_size = 0.0;
    std::vector<CellView> cells;
    std::vector<FaceView> faces;
    int dimension() const { return NDFVL; }
};

enum { cell_field_flag, face_field_flag, node_field_flag };

template <class T> struct Field {
    int len = 0;
    int flag = cell_field_flag;
    std::vector<T> values;
    const MeshView *mesh_ptr = nullptr;  // the solver's mesh (cell fields)
    T &operator[](int i) { return values[(size_t)i]; }
    const T &operator[](int i) const { return values[(size_t)i]; }
    const MeshView *get_mesh() const { return mesh_ptr; }
    // values[i] = func(cell i) over the mesh's cells
    void MeshCellValueToField(const std::function<T(const CellView &)> &func) {
        for (int i = 0; i < len; ++i) values[(size_t)i] = func(mesh_ptr->cells[(size_t)i]);
    }

    // Component id (0 x, 1 y, 2 z) of a vector field as a scalar field.
    Field<double> heft(int id) const {
        Field<double> r;
        r.len = len;
        r.flag = flag;
        r.values.resize(values.size());
        for (size_t i = 0; i < values.size(); ++i) r.values[i] = values[i][id];
        return r;
    }
    void set_zero() { std::fill(values.begin(), values.end(), T()); }
    // One value (a vector as "x y z") per line, 18 significant digits; an unopenable file is
    // skipped with a warning on stderr, as the reference logs one and returns.
    void output(const std::string &file_name) const {
        std::ofstream fp(file_name, std::ios::out | std::ios::trunc);
        if (!fp.is_open()) {
            std::fprintf(stderr, "Cannot open file: %s\n", file_name.c_str());
            return;
        }
        for (const T &v : values) write(fp, v);
    }

private:
    static void write(std::ofstream &fp, double v) { fp << std::setprecision(18) << v << std::endl; }
    static void write(std::ofstream &fp, const Vector &v) {
        fp << std::setprecision(18) << v.x << " " << std::setprecision(18) << v.y << " " << std::setprecision(18)
           << v.z << std::endl;
    }
};

class Solver {
public:
    int step = 0;
    double solution_time = 0.0;
    Field<double> rho_cell, T_cell;
    Field<Vector> vel_cell, q_cell;
    MeshView mesh;      // physical mesh (original Gambit order)
    MeshView dvs_mesh;  // velocity mesh: cell position = xi, volume = weight

    // precision: MESO_FP64 (the parity form), MESO_FP32, or -1 for the case file's "gpu-precision"
    explicit Solver(const std::string &case_file, int precision = -1) {
        meso_case *k = nullptr;
        check(meso_case_load(case_file.c_str(), &k));
        meso_mesh_desc m;
        int32_t rnp = 0, ol = 0, onp = 0;
        meso_dvs_desc d;
        int rc = meso_case_mesh(k, &m);
        if (rc == MESO_OK) rc = meso_case_dvs(k, &d);
        if (rc == MESO_OK) rc = meso_case_loop_settings(k, &max_step_, &write_interval_, &rnp, &ol, &onp);
        if (rc == MESO_OK) views(m, d);
        meso_case_free(k);
        check(rc);
        ncell_ = m.ncell;
        check(meso_ctx_create_from_case(case_file.c_str(), precision, &ctx_));
        resize();
    }
    ~Solver() { meso_ctx_destroy(ctx_); }
    Solver(const Solver &) = delete;
    Solver &operator=(const Solver &) = delete;

    void initial() {
        check(meso_initial(ctx_));
        refresh_status();
        sync();
    }

    void do_step() {
        int32_t done = 0;
        const int rc = meso_step(ctx_, 1, &done);
        if (rc != MESO_OK && rc != MESO_ERR_NAN) check(rc);  // NaN: run_state turns false, as in the reference
        refresh_status();
        meso_params p;
        check(meso_get_params(ctx_, &p));
        if (!run_state_ || (p.residual_interval > 0 && step % p.residual_interval == 0)) sync();
    }

    // FP32 contexts (2-D Shakhov): an FP64 defect correction every `interval` steps, 0 = off
    // (meso_fp32_refine).
    void refine(int interval) { check(meso_fp32_refine(ctx_, interval)); }

    void output() { check(meso_output(ctx_)); }
    bool get_run_state() const { return run_state_; }
    int max_step() const { return max_step_; }
    int write_interval() const { return write_interval_; }

    // Copies the macroscopic fields from the device (original cell order).
    void sync() {
        std::vector<double> u(3 * (size_t)ncell_), q(3 * (size_t)ncell_);
        check(meso_get_macros(ctx_, rho_cell.values.data(), u.data(), T_cell.values.data(), q.data()));
        for (int i = 0; i < ncell_; ++i) {
            vel_cell.values[(size_t)i] = {u[3 * (size_t)i], u[3 * (size_t)i + 1], u[3 * (size_t)i + 2]};
            q_cell.values[(size_t)i] = {q[3 * (size_t)i], q[3 * (size_t)i + 1], q[3 * (size_t)i + 2]};
        }
    }

    meso_ctx *handle() { return ctx_; }

private:
    static void check(int rc) {
        if (rc == MESO_OK) return;
        if (rc == MESO_ERR_INVALID || rc == MESO_ERR_IO) throw std::invalid_argument(meso_last_error());
        throw std::runtime_error(meso_last_error());
    }
    void views(const meso_mesh_desc &m, const meso_dvs_desc &d) {
        mesh.NCELL = m.ncell;
        mesh.NFACE = m.nface;
        mesh.NDFVL = m.dim;
        mesh.total_volume = m.total_volume;
        mesh.min_cell_size = m.min_cell_size;
        mesh.cells.resize((size_t)m.ncell);
        for (int i = 0; i < m.ncell; ++i) {
            CellView &c = mesh.cells[(size_t)i];
            c.id = i;
            c.position = {m.cell_pos[3 * i], m.cell_pos[3 * i + 1], m.cell_pos[3 * i + 2]};
            c.volume = m.cell_vol[i];
            c.face_id.assign(m.cell_face + m.cell_face_ptr[i], m.cell_face + m.cell_face_ptr[i + 1]);
            c.neighbors.assign(m.cell_nbr + m.cell_nbr_ptr[i], m.cell_nbr + m.cell_nbr_ptr[i + 1]);
        }
        mesh.faces.resize((size_t)m.nface);
        for (int f = 0; f < m.nface; ++f) {
            FaceView &v = mesh.faces[(size_t)f];
            v.id = f;
            v.position = {m.face_pos[3 * f], m.face_pos[3 * f + 1], m.face_pos[3 * f + 2]};
            v.area = m.face_area[f];
            v.cell_id[0] = m.face_cell[2 * f];
            v.cell_id[1] = m.face_cell[2 * f + 1];
            v.normal_vector[0] = {m.face_normal[3 * f], m.face_normal[3 * f + 1], m.face_normal[3 * f + 2]};
            v.normal_vector[1] = {-v.normal_vector[0].x, -v.normal_vector[0].y, -v.normal_vector[0].z};
        }
        dvs_mesh.NCELL = d.nv;
        dvs_mesh.NDFVL = m.dim;
        dvs_mesh.cells.resize((size_t)d.nv);
        for (int p = 0; p < d.nv; ++p) {
            CellView &c = dvs_mesh.cells[(size_t)p];
            c.id = p;
            c.position = {d.xi[3 * p], d.xi[3 * p + 1], d.xi[3 * p + 2]};
            c.volume = d.w[p];
            dvs_mesh.total_volume += d.w[p];
        }
    }
    void resize() {
        rho_cell.len = T_cell.len = vel_cell.len = q_cell.len = ncell_;
        rho_cell.mesh_ptr = T_cell.mesh_ptr = &mesh;
        vel_cell.mesh_ptr = q_cell.mesh_ptr = &mesh;
        rho_cell.values.assign((size_t)ncell_, 0.0);
        T_cell.values.assign((size_t)ncell_, 0.0);
        vel_cell.values.assign((size_t)ncell_, Vector());
        q_cell.values.assign((size_t)ncell_, Vector());
    }
    void refresh_status() {
        meso_status st;
        check(meso_get_status(ctx_, &st));
        step = st.step;
        solution_time = st.solution_time;
        run_state_ = st.run_state != 0;
    }

    meso_ctx *ctx_ = nullptr;
    int ncell_ = 0;
    int32_t max_step_ = 0, write_interval_ = 1;
    bool run_state_ = true;
};

// The reference's per-solve loop (src/meso/exec.cpp:141-165) over the GPU solver.
inline int handle_solver(Solver &solver) {
    solver.initial();
    solver.output();
    for (int i = 0; (i < solver.max_step()) || (solver.max_step() < 0); ++i) {
        solver.do_step();
        if (!solver.get_run_state()) break;
        if (solver.write_interval() > 0 && solver.step % solver.write_interval() == 0) solver.output();
    }
    solver.output();
    return 0;
}

}  // namespace GPU
}  // namespace MESO

#endif  // MESO_SOLVER_HPP
