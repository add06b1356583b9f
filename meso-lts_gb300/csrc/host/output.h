// Solver output in the reference's file formats.
#pragma once

#include <string>
#include <vector>

#include "case.h"

namespace meso_host {

// output() of the reference solvers:
//   CDUGKS / CDUGKS_SHAKHOV  cdugks.cpp:373-423, cdugks_shakhov.cpp:791-855
//     <case>/grid.plt at step 0, <case>/step-N/data.plt, <case>/latest/*, np files
//   DUGKS                    dugks.cpp:385-412  (<case>/result-N.dat.plt, np-data/)
// All vectors in original cell order; T, q, flux moments ignored by the BGK solvers.
void write_solver_output(const meso_case &k, int step, double solution_time, const std::vector<double> &rho,
                         const std::vector<double> &u, const std::vector<double> &T, const std::vector<double> &q,
                         const std::vector<double> &m0, const std::vector<double> &m1, const std::vector<double> &m2);

// Mesh::output_grid (mesh_output.cpp:182-215): the Tecplot grid file of the case's mesh.
void write_grid(const meso_case &k, const std::string &file);

}  // namespace meso_host
