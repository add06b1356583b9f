// Case loading and flattening.  See case.h.
//
// Reference correspondence (meso-lts):
//   solver dispatch strings           src/meso/main.cpp:41-61
//   BasicSolver settings              src/solver/basic_solver.cpp:18-36
//   CDUGKS ctor / initial params      src/solver/boltzmann/cdugks.cpp:7-47
//   DUGKS ctor / initial params       src/solver/boltzmann/dugks.cpp:7-48
//   CDUGKS_SHAKHOV update_config/ctor src/solver/boltzmann/cdugks_shakhov.cpp:7-60
//   initial fields from [group]s      cdugks.cpp:66-93, cdugks_shakhov.cpp:103-132
#include "case.h"

#include <cstring>

namespace meso_host {

int solver_kind(const std::string &name) {
    if (name == "dugks@incompressible") return MESO_SOLVER_DUGKS;
    if (name == "cdugks@incompressible") return MESO_SOLVER_CDUGKS;
    if (name == "cdugks@shakhov") return MESO_SOLVER_CDUGKS_SHAKHOV;
    return -1;
}

void params_from_config(const MESO::Solver::Config &cfg, int solver, const MESO::fvmMesh::Mesh &mesh,
                        const MESO::DVS::VelocitySet &dvs, meso_params &p) {
    p.solver = solver;
    p.residual_limit = cfg.get<double>("residual-limit", 1e-6, false);
    p.residual_interval = 100;
    if (solver == MESO_SOLVER_CDUGKS_SHAKHOV) {
        p.Pr = cfg.get<double>("Pr", 0.67);
        p.dt = cfg.get<double>("timeStep", 1.0e-5);
        p.R = cfg.get<double>("gas-constant", 0.5);
        p.K = cfg.get<int>("gas-k", 0);
        p.rho0 = cfg.get<double>("ref-density", 1.0);
        p.L0 = cfg.get<double>("ref-length", 1.0);
        p.T0 = cfg.get<double>("ref-temperature", 1.0);
        p.mu0 = cfg.get<double>("ref-viscosity", 1.60e-05);
        p.vhs_index = cfg.get<double>("vhs-index", 0.81);
        p.gradient_switch = cfg.get<bool>("gradient-switch", true) ? 1 : 0;
        p.limiter_switch = cfg.get<bool>("limiter-switch", false) ? 1 : 0;
        // venkata-limiter-k is read only with the gradient off (cdugks_shakhov.cpp:21-28)
        if (!p.gradient_switch && p.limiter_switch) p.venkata_k = cfg.get<double>("venkata-limiter-k", 1.0);
    } else {
        p.R = cfg.get<double>("gas-constant", 0.5);
        p.T0 = cfg.get<double>("ref-temperature", 1.0);
        p.rho0 = cfg.get<double>("ref-density", 1.0);
        p.L0 = cfg.get<double>("ref-length", 1.0);
        p.Ma = cfg.get<double>("Ma", 0.1);
        p.Re = cfg.get<double>("Re", 400.0);
        p.gradient_switch = cfg.get<bool>("gradient-switch", true) ? 1 : 0;
        if (solver == MESO_SOLVER_DUGKS) {
            p.CFL = cfg.get<double>("CFL", 0.8);
            p.dt = p.CFL * (mesh.min_cell_size / dvs.mesh.max_cell_magnitude);
        } else {
            p.dt = cfg.get<double>("timeStep", 2.5e-3);
        }
    }
}

std::unique_ptr<meso_case> load_case(const std::string &case_file) {
    using namespace MESO;
    auto c = std::make_unique<meso_case>();
    c->config = Solver::Config(case_file);
    auto &cfg = c->config;
    c->case_dir = cfg.base_dir;
    c->solver_name = cfg.get<String>("solver", "<solver>", false);
    int kind = solver_kind(c->solver_name);
    if (kind < 0) throw std::invalid_argument("Load solver: " + c->solver_name + " failed.");
    c->case_name = cfg.resolve(cfg.get<String>("case-name", "unnamed", false));
    c->output_latest = cfg.get<bool>("output-latest", true, false);
    c->output_np = cfg.get<bool>("output-np", false, false);
    c->max_step = cfg.get<int>("max-step", 100000, false);
    c->write_interval = cfg.get<int>("write-interval", 1000, false);
    c->read_np_data = cfg.get<bool>("read-np-data", false, false);
    double mesh_scale = cfg.get<double>("mesh-scale", 1.0, false);

    c->mesh = fvmMesh::load_gambit(cfg.resolve(cfg.get<String>("mesh-file", "<mesh-file>")), mesh_scale);
    auto &mesh = c->mesh;
    const int D = mesh.dimension();
    if (D != 2 && D != 3) throw std::invalid_argument("mesh dimension must be 2 or 3");

    String dvs_file = cfg.resolve(cfg.get<String>("dvs-file", "<mesh-file>"));
    String dvs_type = cfg.get<String>("dvs-type", "<dvs-type>");
    if (kind == MESO_SOLVER_CDUGKS_SHAKHOV) {
        double R = cfg.get<double>("gas-constant", 0.5), T0 = cfg.get<double>("ref-temperature", 1.0);
        if (dvs_type == "Newton-Cotes") c->dvs = DVS::generate_dvs(dvs_file, DVS::NewtonCotesParams{D});
        else if (dvs_type == "half-range-Gauss-Hermite")
            c->dvs = DVS::generate_dvs(dvs_file, DVS::HalfRangeGHParams{D, R * T0});
        else if (dvs_type == "Sparse") c->dvs = DVS::read_mesh_file(dvs_file);
        else c->dvs = DVS::load_gambit_dvs(dvs_file);
    } else {
        if (dvs_type != "Gauss-Hermite") throw std::invalid_argument("dvs-mesh type error.");
        double RT = cfg.get<double>("gas-constant", 0.5) * cfg.get<double>("ref-temperature", 1.0);
        c->dvs = DVS::generate_dvs(dvs_file, DVS::GaussHermiteParams{D, RT});
    }
    params_from_config(cfg, kind, mesh, c->dvs, c->params);
    String prec = cfg.get<String>("gpu-precision", "fp64", false);
    c->params.precision = (prec == "fp32" || prec == "FP32") ? MESO_FP32 : MESO_FP64;

    // ---- flatten the mesh
    const int C = mesh.NCELL, F = mesh.NFACE;
    c->cell_pos.resize(3 * C);
    c->cell_vol.resize(C);
    c->cell_group.resize(C);
    c->lsq_c.resize(9 * C);
    c->cell_face_ptr.assign(1, 0);
    c->cell_nbr_ptr.assign(1, 0);
    for (int i = 0; i < C; ++i) {
        auto &cell = mesh.cells[i];
        if (cell.id != i) throw std::invalid_argument("gambit: cells must be numbered 1..NELEM in order");
        c->cell_pos[3 * i] = cell.position.x;
        c->cell_pos[3 * i + 1] = cell.position.y;
        c->cell_pos[3 * i + 2] = cell.position.z;
        c->cell_vol[i] = cell.volume;
        c->cell_group[i] = cell.group_id;
        for (int f : cell.face_id) c->cell_face.push_back(f);
        c->cell_face_ptr.push_back((int)c->cell_face.size());
        auto &ls = cell.least_square;
        for (int j = 0; j < (int)cell.neighbors.size(); ++j) {
            c->cell_nbr.push_back(cell.neighbors[j]);
            c->lsq_w.push_back(ls.weight[j]);
            c->lsq_dr.push_back(ls.dr[j].x);
            c->lsq_dr.push_back(ls.dr[j].y);
            c->lsq_dr.push_back(ls.dr[j].z);
        }
        c->cell_nbr_ptr.push_back((int)c->cell_nbr.size());
        const Vector *cc[3] = {&ls.Cx, &ls.Cy, &ls.Cz};
        for (int k = 0; k < 3; ++k) {
            c->lsq_c[9 * i + 3 * k] = cc[k]->x;
            c->lsq_c[9 * i + 3 * k + 1] = cc[k]->y;
            c->lsq_c[9 * i + 3 * k + 2] = cc[k]->z;
        }
    }
    c->face_cell.resize(2 * F);
    c->face_pos.resize(3 * F);
    c->face_area.resize(F);
    c->face_normal.resize(3 * F);
    c->face_mark.resize(F);
    for (int f = 0; f < F; ++f) {
        auto &face = mesh.faces[f];
        c->face_cell[2 * f] = face.cell_id[0];
        c->face_cell[2 * f + 1] = face.cell_id[1];
        c->face_pos[3 * f] = face.position.x;
        c->face_pos[3 * f + 1] = face.position.y;
        c->face_pos[3 * f + 2] = face.position.z;
        c->face_area[f] = face.area;
        c->face_normal[3 * f] = face.normal_vector[0].x;
        c->face_normal[3 * f + 1] = face.normal_vector[0].y;
        c->face_normal[3 * f + 2] = face.normal_vector[0].z;
        c->face_mark[f] = face.group_id;
    }
    // one mark descriptor per face group of the mesh
    for (size_t g = 0; g < mesh.face_names.size(); ++g) {
        const String &name = mesh.face_names[g];
        auto it = cfg.marks.find(name);
        if (it == cfg.marks.end()) {
            bool used = false;
            for (auto &f : mesh.faces) used = used || f.group_id == (int)g;
            if (used) throw std::invalid_argument("get_face_group() missing key=" + name);
        }
        meso_mark_desc md{};
        if (it != cfg.marks.end()) {
            const auto &m = it->second;
            md.type = m.type;
            md.temperature_type = m.patch.get_type("temperature");
            md.direction = m.patch.get_int("direction");
            md.density = m.patch.get_scalar("density");
            md.temperature = m.patch.get_scalar("temperature");
            md.pressure = m.patch.get_scalar("pressure");
            Vector v = m.patch.get_vector("velocity");
            md.velocity[0] = v.x;
            md.velocity[1] = v.y;
            md.velocity[2] = v.z;
            md.alpha_u = m.patch.get_scalar("slip-wall-alpha-u");
            md.alpha_T = m.patch.get_scalar("slip-wall-alpha-T");
        }
        c->marks.push_back(md);
        c->mark_names.push_back(name);
    }
    // ---- flatten the DVS
    const auto &dm = c->dvs.mesh;
    const int NV = dm.NCELL;
    if (NV <= 0) throw std::invalid_argument("empty discrete velocity set");
    c->dvs_xi.resize(3 * NV);
    c->dvs_w.resize(NV);
    c->dvs_sym.resize(3 * NV);
    for (int p = 0; p < NV; ++p) {
        auto &pc = dm.cells[p];
        c->dvs_xi[3 * p] = pc.position.x;
        c->dvs_xi[3 * p + 1] = pc.position.y;
        c->dvs_xi[3 * p + 2] = pc.position.z;
        c->dvs_w[p] = pc.volume;
        for (int k = 0; k < 3; ++k) {
            int s = pc.symmetry.id[k];
            if (s < 0 || s >= NV) throw std::invalid_argument("DVS symmetry index out of range");
            c->dvs_sym[3 * p + k] = s;
        }
    }
    // validate the groups now (the reference throws on the first lookup in initial())
    for (auto &cell : mesh.cells) (void)cfg.get_cell_group(cell, mesh);
    return c;
}

}  // namespace meso_host

void meso_case::mesh_desc(meso_mesh_desc &d) const {
    std::memset(&d, 0, sizeof(d));
    d.dim = mesh.dimension();
    d.ncell = mesh.NCELL;
    d.nface = mesh.NFACE;
    d.cell_pos = cell_pos.data();
    d.cell_vol = cell_vol.data();
    d.cell_group = cell_group.data();
    d.cell_face_ptr = cell_face_ptr.data();
    d.cell_face = cell_face.data();
    d.cell_nbr_ptr = cell_nbr_ptr.data();
    d.cell_nbr = cell_nbr.data();
    d.lsq_w = lsq_w.data();
    d.lsq_dr = lsq_dr.data();
    d.lsq_c = lsq_c.data();
    d.face_cell = face_cell.data();
    d.face_pos = face_pos.data();
    d.face_area = face_area.data();
    d.face_normal = face_normal.data();
    d.face_mark = face_mark.data();
    d.min_cell_size = mesh.min_cell_size;
    d.total_volume = mesh.total_volume;
}

void meso_case::dvs_desc(meso_dvs_desc &d) const {
    std::memset(&d, 0, sizeof(d));
    d.nv = dvs.mesh.NCELL;
    d.xi = dvs_xi.data();
    d.w = dvs_w.data();
    d.sym = dvs_sym.data();
    d.tensor_n = dvs.tensor_n;
    d.axis = dvs.axis.empty() ? nullptr : dvs.axis.data();
    d.max_magnitude = dvs.mesh.max_cell_magnitude;
}

bool meso_case::reload_settings() {
    meso_params np = params;
    config.update_config(false);
    meso_host::params_from_config(config, params.solver, mesh, dvs, np);
    np.precision = params.precision;
    np.solver = params.solver;
    np.K = params.K;
    if (params.solver == MESO_SOLVER_CDUGKS_SHAKHOV) {
        // venkata_k keeps its value unless re-read at step 0 (cdugks_shakhov.cpp:21-28)
        np.venkata_k = params.venkata_k;
    }
    if (params.solver != MESO_SOLVER_CDUGKS_SHAKHOV && params.solver != MESO_SOLVER_DUGKS) return false;
    if (params.solver == MESO_SOLVER_DUGKS) {
        // DUGKS re-reads the file but dt/tau are fixed at initial() (dugks.cpp:41-48, 381)
        return false;
    }
    bool changed = std::memcmp(&np, &params, sizeof(np)) != 0;
    params = np;
    return changed;
}

void meso_case::initial_fields(double *rho, double *u, double *T, uint8_t *mask) const {
    using namespace MESO;
    for (auto &cell : mesh.cells) {
        const auto &g = config.get_cell_group(cell, mesh);
        const auto &pt = g.patch;
        int i = cell.id;
        if (rho)
            rho[i] = pt.get_type("density") == Solver::PatchType::fromFile ? pt.get_file_scalar("density", i)
                                                                          : pt.get_scalar("density");
        if (u) {
            Vector v = pt.get_type("velocity") == Solver::PatchType::fromFile ? pt.get_file_vector("velocity", i)
                                                                             : pt.get_vector("velocity");
            u[3 * i] = v.x;
            u[3 * i + 1] = v.y;
            u[3 * i + 2] = v.z;
        }
        if (T)
            T[i] = pt.get_type("temperature") == Solver::PatchType::fromFile ? pt.get_file_scalar("temperature", i)
                                                                            : pt.get_scalar("temperature");
        if (mask) mask[i] = pt.get_switch("mask") ? 1 : 0;
    }
}
