// Case-file parsing and DVS generation.  See config.h.
//
// Reference correspondence (meso-lts):
//   mark_type_map, Config::Config, update_config   src/solver/config.cpp:5-108
//   Config::get<T>                                 src/solver/config.cpp:110-152
//   get_cell_group / get_face_group                src/solver/config.cpp:154-177
//   Patch::set_value and getters                   src/solver/boundary/patch.cpp:5-85
//   Gauss-Hermite / half-range GH / Newton-Cotes   src/solver/dvs/dvs_generator.cpp:15-244
//   Sparse velocity list                           src/solver/dvs/dvs_generator.cpp:246-276
// Deviation, documented in the design notes: the 3-D Gauss-Hermite and
// half-range GH sets use the quadrature weights w_i w_j w_k (the reference
// multiplies abscissae, dvs_generator.cpp:59,133); 2-D sets are unaffected.
#include "config.h"

#include <cmath>
#include <map>

namespace MESO::Solver {

const Dict<int> mark_type_map = {
    {"fluid-interior", fluid_interior},   {"farfield-inlet", farfield_inlet},
    {"pressure-inlet", pressure_inlet},   {"freestream-inlet", freestream_inlet},
    {"farfield-outlet", farfield_outlet}, {"pressure-outlet", pressure_outlet},
    {"wall", wall},                       {"slip-wall", slip_wall},
    {"symmetry", symmetry},
};

namespace {
String dir_of(const String &p) {
    auto pos = p.find_last_of('/');
    return pos == String::npos ? String(".") : p.substr(0, pos);
}
String join(const String &dir, const String &p) {
    if (p.empty() || p[0] == '/' || dir.empty() || dir == ".") return p;
    return dir + "/" + p;
}
}  // namespace

void Patch::set_value(StringList &s) {
    if (s.size() < 2) return;
    const String &name = s[0];
    const String &ts = s[1];
    auto need = [&](size_t k) {
        if (s.size() < k) throw std::invalid_argument("Patch::set_value: too few values for " + name);
    };
    if (ts == "calculated") {
        type[name] = PatchType::calculated;
    } else if (ts == "fixedValue") {
        type[name] = PatchType::fixedValue;
        need(4);
        const String &vts = s[2];
        if (vts == "objectType") ints[name] = std::stoi(s[3]);
        else if (vts == "scalar") scalars[name] = std::stod(s[3]);
        else if (vts == "vector") {
            need(6);
            vectors[name] = {std::stod(s[3]), std::stod(s[4]), std::stod(s[5])};
        } else
            throw std::invalid_argument("Patch::set_value caught unsupported type: " + name + " - " + ts);
    } else if (ts == "zeroGradient") {
        type[name] = PatchType::zeroGradient;
    } else if (ts == "fromFile") {
        type[name] = PatchType::fromFile;
        need(4);
        const String &vts = s[2];
        String file = join(base_dir, s[3]);
        if (vts == "objectType") ints_list[name] = Utils::read_np_file<int>(file);
        else if (vts == "scalar") scalars_list[name] = Utils::read_np_file<double>(file);
        else if (vts == "vector") vectors_list[name] = Utils::read_np_file<Vector>(file);
        else throw std::invalid_argument("Patch::set_value caught unsupported type: " + name + " - " + ts);
    } else if (ts == "switch") {
        type[name] = PatchType::switchType;
        switches[name] = s.size() > 2 && s[2] == "True";
    }
}

template <class M, class K> static typename M::mapped_type lookup(const M &m, const K &k) {
    auto it = m.find(k);
    return it == m.end() ? typename M::mapped_type() : it->second;
}

ObjectType Patch::get_type(const String &k) const { return lookup(type, k); }
bool Patch::get_switch(const String &k) const { return lookup(switches, k); }
ObjectType Patch::get_int(const String &k) const { return lookup(ints, k); }
Scalar Patch::get_scalar(const String &k) const { return lookup(scalars, k); }
Vector Patch::get_vector(const String &k) const { return lookup(vectors, k); }
ObjectType Patch::get_file_int(const String &k, ObjectId id) const { return ints_list.at(k).at(id); }
Scalar Patch::get_file_scalar(const String &k, ObjectId id) const { return scalars_list.at(k).at(id); }
Vector Patch::get_file_vector(const String &k, ObjectId id) const { return vectors_list.at(k).at(id); }

Config::Config(const String &fp) : file_path(fp), base_dir(dir_of(fp)) {
    Mark m;
    m.id = 1;
    m.name = m.type_name = "fluid-interior";
    m.type = fluid_interior;
    marks[m.name] = m;
    update_config(true);
}

String Config::resolve(const String &p) const { return join(base_dir, p); }

void Config::update_config(bool update_patch) {
    StringList lines = Utils::read_lines(file_path);
    const int n = (int)lines.size();
    auto is_block = [](const StringList &d) { return !d.empty() && (d[0] == "[mark]" || d[0] == "[group]"); };
    for (int i = 0; i < n; ++i) {
        StringList d = Utils::split(lines[i]);
        if (d.empty() || d[0] == "#") continue;
        if (d[0] == "[settings]") {
            ++i;
            while (i < n) {
                d = Utils::split(lines[i]);
                if (d.empty() || d[0] == "#") { ++i; continue; }
                if (is_block(d)) { --i; break; }
                if (d.size() >= 2) settings[d[0]] = d[1];
                ++i;
            }
        } else if (d[0] == "[mark]") {
            Mark mark;
            mark.id = (int)marks.size() + 1;
            mark.patch.base_dir = base_dir;
            ++i;
            while (i < n) {
                d = Utils::split(lines[i]);
                if (d.empty() || d[0] == "#") { ++i; continue; }
                if (is_block(d)) { --i; break; }
                if (update_patch) {
                    if (d[0] == "name" && d.size() > 1) mark.name = d[1];
                    else if (d[0] == "type" && d.size() > 1) {
                        mark.type_name = d[1];
                        auto it = mark_type_map.find(d[1]);
                        if (it == mark_type_map.end())
                            throw std::invalid_argument("unknown boundary type: " + d[1]);
                        mark.type = it->second;
                    } else
                        mark.patch.set_value(d);
                }
                ++i;
            }
            if (update_patch) marks[mark.name] = mark;
        } else if (d[0] == "[group]") {
            Group g;
            g.id = (int)groups.size() + 1;
            g.patch.base_dir = base_dir;
            ++i;
            while (i < n) {
                d = Utils::split(lines[i]);
                if (d.empty() || d[0] == "#") { ++i; continue; }
                if (is_block(d)) { --i; break; }
                if (update_patch) {
                    if (d[0] == "name" && d.size() > 1) g.name = d[1];
                    else g.patch.set_value(d);
                }
                ++i;
            }
            if (update_patch) groups[g.name] = g;
        }
    }
}

template <> String Config::get(const String &k, String dv, bool) const {
    auto it = settings.find(k);
    return it == settings.end() ? dv : it->second;
}
template <> int Config::get(const String &k, int dv, bool) const {
    auto it = settings.find(k);
    return it == settings.end() ? dv : std::stoi(it->second);
}
template <> double Config::get(const String &k, double dv, bool) const {
    auto it = settings.find(k);
    return it == settings.end() ? dv : std::stod(it->second);
}
template <> bool Config::get(const String &k, bool dv, bool) const {
    auto it = settings.find(k);
    return it == settings.end() ? dv : (it->second == "True");
}

const Group &Config::get_cell_group(const fvmMesh::Cell &cell, const fvmMesh::Mesh &mesh) const {
    const String &key = mesh.cell_names.at(cell.group_id);
    auto it = groups.find(key);
    if (it == groups.end()) throw std::invalid_argument("get_cell_group() missing key=" + key);
    return it->second;
}

const Mark &Config::get_face_group(const fvmMesh::Face &face, const fvmMesh::Mesh &mesh) const {
    const String &key = mesh.face_names.at(face.group_id);
    auto it = marks.find(key);
    if (it == marks.end()) throw std::invalid_argument("get_face_group() missing key=" + key);
    return it->second;
}

}  // namespace MESO::Solver

namespace MESO::DVS {

namespace {
StringList dvs_lines(const String &file, const char *tag) {
    StringList lines = Utils::read_lines(file);
    if (lines.empty()) throw std::invalid_argument("empty DVS file " + file);
    auto d = Utils::split(lines[0]);
    if (d.empty() || d[0] != tag) throw std::invalid_argument(String("generate_dvs<") + tag + "> type error");
    return lines;
}

void finish(VelocitySet &vs) {
    double mx = 0.0;
    for (auto &c : vs.mesh.cells) {
        double m = c.position.magnitude();
        if (mx < m) mx = m;
    }
    vs.mesh.update_mesh_params();
    vs.mesh.max_cell_magnitude = mx;
}

void read_xw(const StringList &lines, double xs, double ws, List<double> &x, List<double> &w) {
    const int n = (int)lines.size() - 1;
    x.resize(n);
    w.resize(n);
    for (int i = 0; i < n; ++i) {
        auto d = Utils::split(lines[i + 1]);
        if (d.size() < 2) throw std::invalid_argument("DVS: bad abscissa/weight line");
        x[i] = xs * std::stod(d[0]);
        w[i] = ws * std::stod(d[1]);
    }
}

// Cells in "x fastest" order: id = i + j*n (+ k*n*n), symmetry = mirror index per axis.
void tensor_x_fast(VelocitySet &vs, int dim, const List<double> &x, const List<double> &w) {
    const int n = (int)x.size();
    auto sym = [n](int i) { return n - i - 1; };
    if (dim == 2) {
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) {
                fvmMesh::Cell c(i + j * n);
                c.position = {x[i], x[j], 0.0};
                c.volume = w[i] * w[j];
                c.symmetry.id[0] = sym(i) + j * n;
                c.symmetry.id[1] = i + sym(j) * n;
                c.symmetry.id[2] = i + j * n;
                vs.mesh.cells.push_back(c);
            }
    } else {
        for (int k = 0; k < n; ++k)
            for (int j = 0; j < n; ++j)
                for (int i = 0; i < n; ++i) {
                    fvmMesh::Cell c(i + (j + k * n) * n);
                    c.position = {x[i], x[j], x[k]};
                    c.volume = w[i] * w[j] * w[k];
                    c.symmetry.id[0] = sym(i) + (j + k * n) * n;
                    c.symmetry.id[1] = i + (sym(j) + k * n) * n;
                    c.symmetry.id[2] = i + (j + sym(k) * n) * n;
                    vs.mesh.cells.push_back(c);
                }
    }
    vs.tensor_n = n;
    vs.axis = x;
}
}  // namespace

VelocitySet generate_dvs(const String &file, const GaussHermiteParams &p) {
    auto lines = dvs_lines(file, "Gauss-Hermite");
    List<double> x, w;
    read_xw(lines, std::sqrt(2.0 * p.RT), 1.0 / std::sqrt(M_PI), x, w);
    const int n = (int)x.size();
    VelocitySet vs;
    // i-major order of dvs_generator.cpp:42-65: list index = i*n + j (x slowest).
    if (p.dimension == 2) {
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                fvmMesh::Cell c(i + j * n);
                c.position = {x[i], x[j], 0.0};
                c.volume = w[i] * w[j];
                vs.mesh.cells.push_back(c);
            }
    } else {
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j)
                for (int k = 0; k < n; ++k) {
                    fvmMesh::Cell c(i + (j + k * n) * n);
                    c.position = {x[i], x[j], x[k]};
                    c.volume = w[i] * w[j] * w[k];
                    vs.mesh.cells.push_back(c);
                }
    }
    finish(vs);
    return vs;  // symmetry ids stay 0 as in the reference; not a tensor set in x-fast order
}

VelocitySet generate_dvs(const String &file, const HalfRangeGHParams &p) {
    auto lines = dvs_lines(file, "half-range-Gauss-Hermite");
    List<double> x, w;
    read_xw(lines, std::sqrt(2.0 * p.RT), 1.0, x, w);
    VelocitySet vs;
    tensor_x_fast(vs, p.dimension, x, w);
    finish(vs);
    return vs;
}

VelocitySet generate_dvs(const String &file, const NewtonCotesParams &p) {
    auto lines = dvs_lines(file, "Newton-Cotes");
    if (lines.size() < 2) throw std::invalid_argument("Newton-Cotes: missing '<n> <mount> <scale>' line");
    auto d = Utils::split(lines[1]);
    if (d.size() < 3) throw std::invalid_argument("Newton-Cotes: bad parameter line");
    const int n = std::stoi(d[0]);
    const int mount = std::stoi(d[1]);
    const double scale = std::stod(d[2]);
    static const std::map<int, List<double>> nc_weight = {
        {1, {1. / 2., 1. / 2.}},
        {2, {1. / 6., 4. / 6., 1. / 6.}},
        {3, {1. / 8., 3. / 8., 3. / 8., 1. / 8.}},
        {4, {7. / 90., 16. / 45., 2. / 15., 16. / 45., 7. / 90.}},
        {5, {19. / 288., 25. / 96., 25. / 144., 25. / 144., 25. / 96., 19. / 288.}},
        {6, {41. / 840., 9. / 35., 9. / 280., 34. / 105., 9. / 280., 9. / 35., 41. / 840.}}};
    auto it = nc_weight.find(n);
    if (it == nc_weight.end() || mount < 1) throw std::invalid_argument("Newton-Cotes: order must be 1..6");
    const auto &pw = it->second;
    const int total = n * mount + 1;
    const double dh = 2.0 * scale / mount;
    List<double> x(total), w(total, 0.0);
    for (int i = 0; i < total; ++i) x[i] = scale * double(2 * i + 1 - total) / double(total - 1);
    for (int i = 0; i < mount; ++i)
        for (int j = 0; j < n + 1; ++j) w[i * n + j] += pw[j] * dh;
    VelocitySet vs;
    tensor_x_fast(vs, p.dimension, x, w);
    finish(vs);
    return vs;
}

VelocitySet read_mesh_file(const String &file) {
    auto lines = dvs_lines(file, "Sparse");
    VelocitySet vs;
    for (int i = 1; i < (int)lines.size(); ++i) {
        auto d = Utils::split(lines[i]);
        if (d.size() < 4) throw std::invalid_argument("Sparse DVS: bad line");
        fvmMesh::Cell c(i - 1);
        c.position = {std::stod(d[0]), std::stod(d[1]), std::stod(d[2])};
        c.volume = std::stod(d[3]);
        vs.mesh.cells.push_back(c);
    }
    finish(vs);
    return vs;
}

VelocitySet load_gambit_dvs(const String &file) {
    VelocitySet vs;
    vs.mesh = fvmMesh::load_gambit(file, 1.0);
    return vs;
}

}  // namespace MESO::DVS
