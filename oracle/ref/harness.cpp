// In-process driver for the unmodified meso-lts solver classes.
//
// Test infrastructure only.  Built by oracle/build_ref.sh together with the
// reference sources into oracle/_ref/meso_ref; never linked into the product.
// It mirrors the reference step loop (src/meso/exec.cpp:141-165): ctor ->
// initial() -> N x do_step(), stopping when get_run_state() turns false,
// then writes the macroscopic cell fields (and optionally the mesh/DVS tables
// the solver built) as raw little-endian binary for the parity tests.
//
//   meso_ref <case-file> <nsteps> <out.bin> [--mesh <mesh.bin>] [--every K] [--output 1] [--mesh-only 1]
//
// --mesh-only 1 writes the mesh/DVS tables (--mesh) after the solver's constructor and exits
// before initial() allocates the distribution functions.
//
// --output 1 calls the solver's own output() after initial() and after the
// last step, as handle_solver does (exec.cpp:150-164): grid.plt, step-N/
// data.plt and latest/ text files under the case-name folder.
//
// The case file's relative paths are resolved against the current directory,
// exactly as the reference does; run it from the case directory.
#include "meso.h"

#include <chrono>
#include <cstdio>
#include <string>
#include <vector>

namespace {

struct Out {
    FILE *fp;
    explicit Out(const std::string &p) : fp(std::fopen(p.c_str(), "wb")) {
        if (!fp) throw std::runtime_error("cannot open " + p);
    }
    ~Out() { if (fp) std::fclose(fp); }
    void i32(int v) { std::fwrite(&v, 4, 1, fp); }
    void f64(double v) { std::fwrite(&v, 8, 1, fp); }
    void vec(const MESO::Vector &v) { f64(v.x); f64(v.y); f64(v.z); }
};

// Record layout (all little endian):
//   int32 magic 0x4D45534F, int32 ncell, int32 step, int32 run_state,
//   f64 solution_time, f64 step_loop_seconds,
//   f64 rho[ncell], f64 u[3*ncell], f64 T[ncell], f64 q[3*ncell]
template <class S>
void write_macros(Out &o, S &s, const MESO::Field<MESO::Scalar> *T, const MESO::Field<MESO::Vector> *q,
                  double secs) {
    const int n = s.mesh.NCELL;
    o.i32(0x4D45534F);
    o.i32(n);
    o.i32(s.step);
    o.i32(s.get_run_state() ? 1 : 0);
    o.f64(s.solution_time);
    o.f64(secs);
    for (int i = 0; i < n; ++i) o.f64(s.rho_cell.values[i]);
    for (int i = 0; i < n; ++i) o.vec(s.vel_cell.values[i]);
    for (int i = 0; i < n; ++i) o.f64(T ? T->values[i] : 0.0);
    for (int i = 0; i < n; ++i) o.vec(q ? q->values[i] : MESO::Vector());
}

// Mesh/DVS tables as the reference builds them (object.cpp:94-172, geom.cpp,
// dvs_generator.cpp), for checking the product's host geometry bit for bit.
void write_mesh(const std::string &path, MESO::fvmMesh::Mesh &m, MESO::fvmMesh::Mesh &dvs) {
    Out o(path);
    o.i32(0x4D455348);
    o.i32(m.dimension());
    o.i32(m.NCELL);
    o.i32(m.NFACE);
    o.i32(m.NNODE);
    o.f64(m.min_cell_size);
    o.f64(m.total_volume);
    for (auto &c : m.cells) {
        o.i32(c.geom_type);
        o.i32(c.group_id);
        o.vec(c.position);
        o.f64(c.volume);
        o.i32((int)c.face_id.size());
        for (int f : c.face_id) o.i32(f);
        o.i32((int)c.neighbors.size());
        for (size_t j = 0; j < c.neighbors.size(); ++j) {
            o.i32(c.neighbors[j]);
            o.f64(c.least_square.weight[j]);
            o.vec(c.least_square.dr[j]);
        }
        o.vec(c.least_square.Cx);
        o.vec(c.least_square.Cy);
        o.vec(c.least_square.Cz);
    }
    for (auto &f : m.faces) {
        o.i32(f.cell_id[0]);
        o.i32(f.cell_id[1]);
        o.i32(f.group_id);
        o.vec(f.position);
        o.f64(f.area);
        o.vec(f.normal_vector[0]);
        o.vec(f.normal_vector[1]);
    }
    o.i32(dvs.NCELL);
    o.f64(dvs.max_cell_magnitude);
    for (auto &c : dvs.cells) {
        o.vec(c.position);
        o.f64(c.volume);
        o.i32(c.symmetry.id[0]);
        o.i32(c.symmetry.id[1]);
        o.i32(c.symmetry.id[2]);
    }
}

template <class S>
int run(MESO::ArgParser &parser, MESO::Solver::Config &config, int nsteps, const std::string &out,
        const std::string &mesh_out, int every, int output, int mesh_only) {
    S s(parser, config);
    if (!mesh_out.empty()) write_mesh(mesh_out, s.mesh, s.dvs_mesh);
    if (mesh_only) return 0;
    s.initial();
    if (output) s.output();
    auto t0 = std::chrono::steady_clock::now();
    for (int i = 0; i < nsteps; ++i) {
        s.do_step();
        if (!s.get_run_state()) break;
        if (every > 0 && s.step % every == 0 && s.step < nsteps) {
            // intermediate snapshot: <out>.<step>
            double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            Out o(out + "." + std::to_string(s.step));
            if constexpr (std::is_same_v<S, MESO::Solver::CDUGKS_SHAKHOV>)
                write_macros(o, s, &s.T_cell, &s.q_cell, secs);
            else
                write_macros(o, s, nullptr, nullptr, secs);
        }
    }
    double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (output) s.output();
    Out o(out);
    if constexpr (std::is_same_v<S, MESO::Solver::CDUGKS_SHAKHOV>)
        write_macros(o, s, &s.T_cell, &s.q_cell, secs);
    else
        write_macros(o, s, nullptr, nullptr, secs);
    return 0;
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s <case> <nsteps> <out.bin> [--mesh f] [--every K]\n", argv[0]);
        return 2;
    }
    std::string case_file = argv[1];
    int nsteps = std::atoi(argv[2]);
    std::string out = argv[3];
    std::string mesh_out;
    int every = 0, output = 0, mesh_only = 0;
    for (int i = 4; i + 1 < argc; i += 2) {
        std::string k = argv[i];
        if (k == "--mesh") mesh_out = argv[i + 1];
        else if (k == "--every") every = std::atoi(argv[i + 1]);
        else if (k == "--output") output = std::atoi(argv[i + 1]);
        else if (k == "--mesh-only") mesh_only = std::atoi(argv[i + 1]);
    }
    char a0[] = "meso_ref", a1[] = "--case";
    std::vector<char> a2(case_file.begin(), case_file.end());
    a2.push_back('\0');
    char *pargv[] = {a0, a1, a2.data(), nullptr};
    int pargc = 3;
    MESO::ArgParser parser(pargc, pargv);
    logger.level = 100;  // silence the reference logger
    MESO::MPI::Initialize(&pargc, reinterpret_cast<char ***>(&pargv));
    MESO::Solver::Config config(case_file);
    auto solver = config.get<std::string>("solver", "<solver>", false);
    int rc = 3;
    try {
        if (solver == "dugks@incompressible")
            rc = run<MESO::Solver::DUGKS>(parser, config, nsteps, out, mesh_out, every, output, mesh_only);
        else if (solver == "cdugks@incompressible")
            rc = run<MESO::Solver::CDUGKS>(parser, config, nsteps, out, mesh_out, every, output, mesh_only);
        else if (solver == "cdugks@shakhov")
            rc = run<MESO::Solver::CDUGKS_SHAKHOV>(parser, config, nsteps, out, mesh_out, every, output, mesh_only);
        else
            std::fprintf(stderr, "unknown solver %s\n", solver.c_str());
    } catch (const std::exception &e) {
        std::fprintf(stderr, "reference threw: %s\n", e.what());
        rc = 4;
    }
    MESO::MPI::Finalize();
    return rc;
}
