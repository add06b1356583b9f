// Tecplot and numpy-text writers with the reference's layout
// (src/mesh/mesh_output.cpp:111-331, src/solver/field.cpp:139-173).
#include "output.h"

#include <sys/stat.h>

#include <fstream>
#include <iomanip>
#include <sstream>

namespace meso_host {
namespace {

using MESO::fvmMesh::Mesh;

void mkdir_p(const std::string &dir) {
    std::string cur;
    std::stringstream ss(dir);
    std::string part;
    if (!dir.empty() && dir[0] == '/') cur = "/";
    while (std::getline(ss, part, '/')) {
        if (part.empty()) continue;
        cur += part + "/";
        ::mkdir(cur.c_str(), 0755);
    }
}

void write_nodes(std::ostream &fp, const Mesh &m) {
    const int dim = m.dimension();
    for (int axis = 0; axis < dim; ++axis) {
        int count = 0;
        fp << "\n## Node-" << (axis == 0 ? "x" : axis == 1 ? "y" : "z") << "\n";
        for (auto &n : m.nodes) {
            fp << "\t" << std::setprecision(15) << n.position[axis];
            if (count++ >= 30) {
                fp << "\n";
                count = 0;
            }
        }
        fp << "\n";
    }
}

void write_geom(std::ostream &fp, const Mesh &m) {
    fp << "\n## geom\n";
    for (auto &c : m.cells) {
        std::vector<int> n(c.node_id.size());
        for (size_t i = 0; i < n.size(); ++i) n[i] = c.node_id[i] + 1;
        switch (c.geom_type) {
            case MESO::Geom::Quad: fp << " " << n[0] << " " << n[1] << " " << n[2] << " " << n[3]; break;
            case MESO::Geom::Tria: fp << " " << n[0] << " " << n[1] << " " << n[2] << " " << n[0]; break;
            case MESO::Geom::Brick:
                fp << " " << n[0] << " " << n[1] << " " << n[3] << " " << n[2] << " " << n[4] << " " << n[5] << " "
                   << n[7] << " " << n[6];
                break;
            case MESO::Geom::Wedge:
                fp << " " << n[0] << " " << n[1] << " " << n[2] << " " << n[2] << " " << n[3] << " " << n[4] << " "
                   << n[5] << " " << n[5];
                break;
            case MESO::Geom::Tetra:
                fp << " " << n[0] << " " << n[1] << " " << n[2] << " " << n[2] << " " << n[3] << " " << n[3] << " "
                   << n[3] << " " << n[3];
                break;
            case MESO::Geom::Pyram:
                fp << " " << n[0] << " " << n[1] << " " << n[3] << " " << n[2] << " " << n[4] << " " << n[4] << " "
                   << n[4] << " " << n[4];
                break;
            default: break;
        }
        fp << "\n";
    }
}

void output_grid(const std::string &file, const Mesh &m) {
    std::ofstream fp(file, std::ios::out | std::ios::trunc);
    if (!fp) return;
    const int dim = m.dimension();
    fp << "TITLE = \"Grid\"\nFileType = \"GRID\"\nVARIABLES = \"X\",\"Y\"\n";
    if (dim == 3) fp << ",\"Z\"";
    fp << "\nZONE T=\"Grid\", N=" << m.NNODE << ", E=" << m.NCELL
       << ", DATAPACKING=BLOCK, ZONETYPE=" << (dim == 2 ? "FEQUADRILATERAL" : "FEBRICK") << "\n";
    write_nodes(fp, m);
    write_geom(fp, m);
}

void output_data(const std::string &file, const Mesh &m, const std::vector<const std::vector<double> *> &vals,
                 const std::vector<std::string> &names, double t) {
    std::ofstream fp(file, std::ios::out | std::ios::trunc);
    if (!fp) return;
    const int dim = m.dimension();
    fp << "TITLE = \"SolutionData\"\nFileType = \"SOLUTION\"\nVARIABLES = ";
    for (size_t i = 0; i < vals.size(); ++i) {
        fp << "\"" << names[i] << "\"";
        if (i + 1 == vals.size()) break;
        fp << ", ";
    }
    fp << "\nZONE T=\"Data\", N=" << m.NNODE << ", E=" << m.NCELL << ", VARLOCATION=(["
       << (vals.size() == 1 ? std::string("1") : "1-" + std::to_string(vals.size()))
       << "]=CELLCENTERED), DATAPACKING=BLOCK, ZONETYPE=" << (dim == 2 ? "FEQUADRILATERAL" : "FEBRICK")
       << ", SOLUTIONTIME=" << t << "\n";
    int count = 0;  // carried across fields, as in mesh_output.cpp:228-247
    for (size_t i = 0; i < vals.size(); ++i) {
        fp << "\n## " << names[i] << "\n";
        for (double v : *vals[i]) {
            fp << "\t" << std::setprecision(18) << v;
            if (count++ >= 30) {
                fp << "\n";
                count = 0;
            }
        }
        fp << "\n";
    }
}

void output_result(const std::string &file, const Mesh &m, const std::vector<const std::vector<double> *> &vals,
                   const std::vector<std::string> &names, int step, double t) {
    std::ofstream fp(file + ".dat.plt", std::ios::out | std::ios::trunc);
    if (!fp) return;
    const int dim = m.dimension(), vc = (int)vals.size();
    fp << "VARIABLES = \"X\", \"Y\"";
    if (dim == 3) fp << " ,\"Z\"";
    for (auto &n : names) fp << " ,\"" << n << "\"";
    fp << "\nZONE T=\"" << (step >= 0 ? "SolutionData(step=" + std::to_string(step) + ")" : "SolutionData")
       << "\", N=" << m.NNODE << ", E=" << m.NCELL << ", VARLOCATION=([1-" << dim << "]=NODAL, [";
    if (vc == 1) fp << dim + 1;
    else fp << dim + 1 << "-" << dim + vc;
    fp << "]=CELLCENTERED), DATAPACKING=BLOCK, ZONETYPE=" << (dim == 2 ? "FEQUADRILATERAL" : "FEBRICK");
    if (t >= 0.0) fp << ", SOLUTIONTIME=" << t;
    fp << "\n";
    write_nodes(fp, m);
    for (int i = 0; i < vc; ++i) {
        int count = 0;
        fp << "\n## CellVar-" << names[i] << "\n";
        for (double v : *vals[i]) {
            fp << "\t" << std::setprecision(15) << v;
            if (count++ >= 30) {
                fp << "\n";
                count = 0;
            }
        }
        fp << "\n";
    }
    write_geom(fp, m);
}

void write_scalar(const std::string &file, const std::vector<double> &v) {
    std::ofstream fp(file, std::ios::out | std::ios::trunc);
    for (double x : v) fp << std::setprecision(18) << x << "\n";
}
void write_vector(const std::string &file, const std::vector<double> &v) {
    std::ofstream fp(file, std::ios::out | std::ios::trunc);
    for (size_t i = 0; i + 2 < v.size(); i += 3)
        fp << std::setprecision(18) << v[i] << " " << std::setprecision(18) << v[i + 1] << " "
           << std::setprecision(18) << v[i + 2] << "\n";
}
std::vector<double> comp(const std::vector<double> &v, int k) {
    std::vector<double> r(v.size() / 3);
    for (size_t i = 0; i < r.size(); ++i) r[i] = v[3 * i + k];
    return r;
}

}  // namespace

void write_grid(const meso_case &k, const std::string &file) { output_grid(file, k.mesh); }

void write_solver_output(const meso_case &k, int step, double t, const std::vector<double> &rho,
                         const std::vector<double> &u, const std::vector<double> &T, const std::vector<double> &q,
                         const std::vector<double> &m0, const std::vector<double> &m1, const std::vector<double> &m2) {
    const Mesh &m = k.mesh;
    const int dim = m.dimension();
    const std::string base = k.case_name;
    mkdir_p(base);
    auto U = comp(u, 0), V = comp(u, 1), W = comp(u, 2);
    const int solver = k.params.solver;
    if (solver == MESO_SOLVER_DUGKS) {
        std::string f = base + "/result-" + std::to_string(step);
        if (dim == 2) output_result(f, m, {&rho, &U, &V}, {"Rho", "U", "V"}, step, t);
        else output_result(f, m, {&rho, &U, &V, &W}, {"Rho", "U", "V", "W"}, step, t);
        if (k.output_np) {
            mkdir_p(base + "/np-data");
            write_scalar(base + "/np-data/Rho", rho);
            write_vector(base + "/np-data/vel", u);
        }
        return;
    }
    if (step == 0) output_grid(base + "/grid.plt", m);
    const std::string path = base + "/step-" + std::to_string(step) + "/";
    const std::string latest = base + "/latest/";
    mkdir_p(path);
    mkdir_p(latest);
    if (solver == MESO_SOLVER_CDUGKS) {
        if (dim == 2) output_data(path + "/data.plt", m, {&rho, &U, &V}, {"Rho", "U", "V"}, t);
        else output_data(path + "/data.plt", m, {&rho, &U, &V, &W}, {"Rho", "U", "V", "W"}, t);
        if (k.output_latest) {
            write_scalar(latest + "Rho", rho);
            write_vector(latest + "U", u);
        }
        if (k.output_np) {
            write_scalar(path + "Rho", rho);
            write_vector(path + "U", u);
        }
        return;
    }
    auto qx = comp(q, 0), qy = comp(q, 1), qz = comp(q, 2);
    if (dim == 2)
        output_data(path + "/data.plt", m, {&rho, &U, &V, &T, &qx, &qy}, {"Rho", "U", "V", "T", "qx", "qy"}, t);
    else
        output_data(path + "/data.plt", m, {&rho, &U, &V, &W, &T, &qx, &qy, &qz},
                    {"Rho", "U", "V", "W", "T", "qx", "qy", "qz"}, t);
    auto dump = [&](const std::string &dir) {
        write_scalar(dir + "Rho", rho);
        write_vector(dir + "U", u);
        write_scalar(dir + "T", T);
        write_vector(dir + "q", q);
        write_scalar(dir + "fluxM0", m0);
        write_vector(dir + "fluxM1", m1);
        write_scalar(dir + "fluxM2", m2);
    };
    if (k.output_latest) dump(latest);
    if (k.output_np) dump(path);
}

}  // namespace meso_host
