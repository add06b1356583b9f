// meso_gpu_run: the reference's per-solve loop (src/meso/exec.cpp:141-165) over the GPU solver.
//
//   meso_gpu_run <case-file> [fp64|fp32] [--refine K] [--dump <file>] [--fields <prefix>]
//
// Runs initial(), output(), do_step() until max-step or run_state false (output() every
// write-interval), output(), as the reference's meso-mpi does for one case file, with the
// MESO::GPU::Solver drop-in (include/meso_solver.hpp).  --dump writes the final macroscopic fields
// as raw doubles: ncell, step, solution_time, rho[ncell], u[3 ncell], T[ncell], q[3 ncell].
// --fields writes them through the Field API as text: <prefix>rho.dat, <prefix>u.dat (the x
// component, Field::heft(0)), <prefix>vel.dat (vectors).  --refine K (FP32 Shakhov cases) adds an
// FP64 defect correction every K steps (meso_fp32_refine).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "meso_solver.hpp"

int main(int argc, char **argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s <case-file> [fp64|fp32] [--refine K] [--dump <file>] [--fields <prefix>]\n",
                     argv[0]);
        return 2;
    }
    int precision = -1;
    std::string dump, fields;
    int refine = 0;
    for (int i = 2; i < argc; ++i) {
        if (!std::strcmp(argv[i], "fp64")) precision = MESO_FP64;
        else if (!std::strcmp(argv[i], "fp32")) precision = MESO_FP32;
        else if (!std::strcmp(argv[i], "--dump") && i + 1 < argc) dump = argv[++i];
        else if (!std::strcmp(argv[i], "--fields") && i + 1 < argc) fields = argv[++i];
        else if (!std::strcmp(argv[i], "--refine") && i + 1 < argc) refine = std::atoi(argv[++i]);
    }
    try {
        MESO::GPU::Solver solver(argv[1], precision);
        if (refine > 0) solver.refine(refine);
        MESO::GPU::handle_solver(solver);
        solver.sync();
        std::printf("step %d  solution_time %.17g  run_state %d\n", solver.step, solver.solution_time,
                    solver.get_run_state() ? 1 : 0);
        double mass = 0.0, wsum = 0.0;
        MESO::GPU::Field<double> m = solver.rho_cell;  // rho V per cell through the Field API
        m.MeshCellValueToField([&](const MESO::GPU::CellView &c) { return solver.rho_cell[c.id] * c.volume; });
        for (int i = 0; i < m.len; ++i) mass += m[i];
        for (const auto &c : solver.dvs_mesh.cells) wsum += c.volume;
        std::printf("cells %d  faces %d  velocities %d  mass %.17g  weights %.17g\n", solver.mesh.NCELL,
                    solver.mesh.NFACE, solver.dvs_mesh.NCELL, mass, wsum);
        if (!fields.empty()) {
            solver.rho_cell.output(fields + "rho.dat");
            solver.vel_cell.heft(0).output(fields + "u.dat");
            solver.vel_cell.output(fields + "vel.dat");
        }
        if (!dump.empty()) {
            FILE *f = std::fopen(dump.c_str(), "wb");
            if (!f) throw std::runtime_error("cannot write " + dump);
            const double head[3] = {(double)solver.rho_cell.len, (double)solver.step, solver.solution_time};
            std::fwrite(head, sizeof(double), 3, f);
            std::fwrite(solver.rho_cell.values.data(), sizeof(double), solver.rho_cell.values.size(), f);
            for (const auto &v : solver.vel_cell.values) std::fwrite(&v, sizeof(double), 3, f);
            std::fwrite(solver.T_cell.values.data(), sizeof(double), solver.T_cell.values.size(), f);
            for (const auto &v : solver.q_cell.values) std::fwrite(&v, sizeof(double), 3, f);
            std::fclose(f);
        }
    } catch (const std::invalid_argument &e) {
        std::fprintf(stderr, "invalid argument: %s\n", e.what());
        return 1;
    } catch (const std::exception &e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
