// Host mesh layer implementation.  See mesh.h.
//
// Reference correspondence (meso-lts, paths relative to the project root):
//   Utils::split / read_lines      src/core/core.cpp:12-22, src/core/file_reader.cpp:7-26
//   Geom::* areas, volumes, normal src/mesh/geom.cpp:31-131, 213-258
//   face key                       src/mesh/geom.cpp:133-162
//   Mesh::generate_face            src/mesh/object.cpp:38-84
//   Mesh::build_geom               src/mesh/object.cpp:94-172
//   Cell::compute_least_square     src/mesh/geom.cpp:165-211
//   Gambit reader                  src/mesh/mesh_reader.cpp:8-139
//   Field output / np I/O          src/solver/field.cpp:97-173, 253-273; src/core/core.cpp:100-134
// Built with -ffp-contract=off: every expression below is evaluated in the
// reference's order so geometry matches it bit for bit.
#include "mesh.h"

#include <algorithm>
#include <array>
#include <cstdint>
#include <fstream>
#include <iomanip>
#include <map>
#include <sstream>
#include <unordered_map>

namespace MESO {

// Whitespace-separated tokens (the tokens `std::istream >> std::string` yields in the "C" locale),
// scanned directly: mesh files have one record per line and hundreds of thousands of tokens.
StringList Utils::split(const String &s) {
    StringList out;
    out.reserve(8);
    const char *p = s.data(), *e = p + s.size();
    auto ws = [](char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r'; };
    while (p < e) {
        while (p < e && ws(*p)) ++p;
        const char *b = p;
        while (p < e && !ws(*p)) ++p;
        if (p > b) out.emplace_back(b, p);
    }
    return out;
}

StringList Utils::read_lines(const String &file) {
    std::ifstream fp(file);
    if (!fp.is_open()) throw std::invalid_argument("file open error: " + file);
    StringList lines;
    String line;
    while (std::getline(fp, line)) {
        line.erase(std::remove(line.begin(), line.end(), '\r'), line.end());
        line.erase(std::remove(line.begin(), line.end(), '\n'), line.end());
        if (!line.empty()) lines.push_back(line);
    }
    return lines;
}

template <> List<int> Utils::read_np_file<int>(const String &file) {
    List<int> r;
    for (auto &l : read_lines(file)) {
        auto d = split(l);
        if (!d.empty()) r.push_back(std::stoi(d[0]));
    }
    return r;
}
template <> List<double> Utils::read_np_file<double>(const String &file) {
    List<double> r;
    for (auto &l : read_lines(file)) {
        auto d = split(l);
        if (!d.empty()) r.push_back(std::stod(d[0]));
    }
    return r;
}
template <> List<Vector> Utils::read_np_file<Vector>(const String &file) {
    List<Vector> r;
    for (auto &l : read_lines(file)) {
        auto d = split(l);
        if (d.size() >= 3) r.emplace_back(std::stod(d[0]), std::stod(d[1]), std::stod(d[2]));
    }
    return r;
}

template <> void read_np_data<Scalar>(const String &file, Field<Scalar> &field) {
    auto lines = Utils::read_lines(file);
    for (int i = 0; i < (int)lines.size() && i < field.len; ++i) field[i] = std::stod(lines[i]);
}
template <> void read_np_data<Vector>(const String &file, Field<Vector> &field) {
    auto lines = Utils::read_lines(file);
    for (int i = 0; i < (int)lines.size() && i < field.len; ++i) {
        auto d = Utils::split(lines[i]);
        if (d.size() < 3) throw std::invalid_argument("read_np_data: bad vector line in " + file);
        field[i] = {std::stod(d[0]), std::stod(d[1]), std::stod(d[2])};
    }
}

template <> Field<Scalar> Field<Vector>::heft(int id) const {
    Field<Scalar> r(*mesh_ptr, flag);
    for (int i = 0; i < len; ++i) r.values[i] = values[i][id];
    return r;
}

template <> void Field<Scalar>::output(const String &file) const {
    std::ofstream fp(file, std::ios::out | std::ios::trunc);
    if (!fp.is_open()) return;
    for (auto &v : values) fp << std::setprecision(18) << v << '\n';
}
template <> void Field<Vector>::output(const String &file) const {
    std::ofstream fp(file, std::ios::out | std::ios::trunc);
    if (!fp.is_open()) return;
    for (auto &v : values)
        fp << std::setprecision(18) << v.x << " " << std::setprecision(18) << v.y << " "
           << std::setprecision(18) << v.z << '\n';
}

// ---------------------------------------------------------------- geometry
int Geom::face_num(ObjectType t) {
    switch (t) {
        case Tria: return 3;
        case Quad: case Tetra: return 4;
        case Wedge: case Pyram: return 5;
        case Brick: return 6;
        default: throw std::invalid_argument("face_num: unsupported geom_type");
    }
}

int Geom::node_num(ObjectType t) {
    switch (t) {
        case Edge: return 2;
        case Tria: return 3;
        case Quad: case Tetra: return 4;
        case Pyram: return 5;
        case Wedge: return 6;
        case Brick: return 8;
        default: throw std::invalid_argument("node_num: unsupported geom_type");
    }
}

namespace {
using NodeList = List<fvmMesh::Node>;

Vector edge_vector(int s, int e, const NodeList &n) { return n[e].position - n[s].position; }

Vector centroid(const NodeList &n) {
    Vector p(0.0, 0.0, 0.0);
    for (auto &it : n) p += it.position;
    return p * (1.0 / double(n.size()));
}

double area_tria(const NodeList &n) { return 0.5 * (edge_vector(0, 1, n) ^ edge_vector(0, 2, n)).magnitude(); }
double area_quad(const NodeList &n) { return area_tria({n[0], n[1], n[2]}) + area_tria({n[0], n[3], n[2]}); }
double vol_tetra(const NodeList &n) {
    Vector p1 = edge_vector(0, 1, n), p2 = edge_vector(0, 2, n), p3 = edge_vector(0, 3, n);
    return std::abs(p1 * (p2 ^ p3)) / 6.0;
}
double vol_pyram(const NodeList &n) {
    return vol_tetra({n[0], n[1], n[2], n[4]}) + vol_tetra({n[1], n[2], n[3], n[4]});
}
double vol_wedge(const NodeList &n) {
    return vol_pyram({n[0], n[2], n[5], n[3], n[1]}) + vol_tetra({n[1], n[3], n[4], n[5]});
}
double vol_brick(const NodeList &n) {
    return vol_wedge({n[0], n[1], n[5], n[2], n[3], n[7]}) + vol_wedge({n[0], n[4], n[5], n[2], n[6], n[7]});
}

double face_area(ObjectType t, const NodeList &n) {
    switch (t) {
        case Geom::Edge: return edge_vector(0, 1, n).magnitude();
        case Geom::Tria: return area_tria(n);
        case Geom::Quad: return area_quad(n);
        default: throw std::invalid_argument("calculate_area: unsupported geom_type");
    }
}

double cell_volume(ObjectType t, const NodeList &n) {
    switch (t) {
        case Geom::Tria: return area_tria(n);
        case Geom::Quad: return area_quad(n);
        case Geom::Brick: return vol_brick(n);
        case Geom::Wedge: return vol_wedge(n);
        case Geom::Tetra: return vol_tetra(n);
        case Geom::Pyram: return vol_pyram(n);
        default: throw std::invalid_argument("calculate_volume: unsupported geom_type");
    }
}

double angle_2d(const Vector &a, const Vector &b) { return std::acos((a * b) / (a.magnitude() * b.magnitude())); }

// Outward normal from the owner cell (geom.cpp:109-131).  In 2D it is built
// through acos/cos, which is why axis-aligned faces carry ~1e-17 residues.
Vector face_normal(ObjectType t, const Vector &cell_pos, const Vector &face_pos, const NodeList &n) {
    Vector vcf = face_pos - cell_pos;
    Vector vfn = edge_vector(0, 1, n).normalize();
    if (t == Geom::Edge) {
        double ax = angle_2d(vfn, {1.0, 0.0, 0.0});
        double ay = angle_2d(vfn, {0.0, 1.0, 0.0});
        if (ay <= M_PI_2) ax = M_PI_2 + ax;
        else ax = M_PI_2 - ax;
        Vector nv = Vector(std::cos(ax), std::sin(ax), 0.0).normalize();
        return (nv * vcf >= 0.0) ? nv : -nv;
    }
    Vector nv = (edge_vector(1, 0, n) ^ edge_vector(1, 2, n)).normalize();
    return (nv * vcf >= 0.0) ? nv : -nv;
}

// Canonical cyclic node sequence of a face: start at the smallest node and
// walk towards its smaller neighbour.  Two faces are the same face exactly
// when these sequences are equal (the reference's string key, geom.cpp:133-162).
void face_key(const ObjectId *nl, int len, ObjectId *key) {
    int pos = 0, mn = nl[0];
    for (int i = 0; i < len; ++i)
        if (nl[i] < mn) { pos = i; mn = nl[i]; }
    int lp = pos == 0 ? len - 1 : pos - 1;
    int rp = pos == len - 1 ? 0 : pos + 1;
    bool dir = nl[rp] < nl[lp];
    for (int c = 0; c < len; ++c) {
        key[c] = nl[pos];
        pos = dir ? pos + 1 : pos - 1;
        if (pos < 0) pos = len - 1;
        if (pos > len - 1) pos = 0;
    }
}

// Face shapes and local node lists per cell shape (object.cpp:18-34).
const List<ObjectType> &face_geoms(ObjectType t) {
    static const std::map<int, List<ObjectType>> m = {
        {Geom::Quad, {Geom::Edge, Geom::Edge, Geom::Edge, Geom::Edge}},
        {Geom::Tria, {Geom::Edge, Geom::Edge, Geom::Edge}},
        {Geom::Brick, {Geom::Quad, Geom::Quad, Geom::Quad, Geom::Quad, Geom::Quad, Geom::Quad}},
        {Geom::Wedge, {Geom::Quad, Geom::Quad, Geom::Quad, Geom::Tria, Geom::Tria}},
        {Geom::Tetra, {Geom::Tria, Geom::Tria, Geom::Tria, Geom::Tria}},
        {Geom::Pyram, {Geom::Quad, Geom::Tria, Geom::Tria, Geom::Tria, Geom::Tria}}};
    auto it = m.find(t);
    if (it == m.end()) throw std::invalid_argument("generate_face: unsupported cell type");
    return it->second;
}
const List<List<int>> &face_nodes(ObjectType t) {
    static const std::map<int, List<List<int>>> m = {
        {Geom::Quad, {{0, 1}, {1, 2}, {2, 3}, {3, 0}}},
        {Geom::Tria, {{0, 1}, {1, 2}, {2, 0}}},
        {Geom::Brick, {{0, 1, 5, 4}, {1, 3, 7, 5}, {3, 2, 6, 7}, {2, 0, 4, 6}, {1, 0, 2, 3}, {4, 5, 7, 6}}},
        {Geom::Wedge, {{0, 1, 4, 3}, {1, 2, 5, 4}, {2, 0, 3, 5}, {0, 2, 1}, {3, 4, 5}}},
        {Geom::Tetra, {{1, 0, 2}, {0, 1, 3}, {1, 2, 3}, {2, 0, 3}}},
        {Geom::Pyram, {{0, 2, 3, 1}, {0, 1, 4}, {1, 3, 4}, {3, 2, 4}, {2, 0, 4}}}};
    return m.at(t);
}
}  // namespace

namespace fvmMesh {

Cell::Cell(ObjectId i, ObjectType t, List<ObjectId> nodes) : geom_type(t), id(i), node_id(std::move(nodes)) {
    face_id.assign(Geom::face_num(t), -1);
}

// Canonical face key (at most four nodes) padded with -1, hashed for the face table.
struct FaceKey4 {
    std::array<ObjectId, 4> n;
    bool operator==(const FaceKey4 &o) const { return n == o.n; }
};
struct FaceKey4Hash {
    size_t operator()(const FaceKey4 &k) const {
        uint64_t h = 1469598103934665603ull;
        for (ObjectId v : k.n) h = (h ^ (uint64_t)(uint32_t)v) * 1099511628211ull;
        return (size_t)h;
    }
};

void Mesh::generate_face() {
    // edge, quad, tria faces; a face is found again exactly when its canonical key matches
    std::unordered_map<FaceKey4, ObjectId, FaceKey4Hash> maps[3];
    for (auto &m : maps) m.reserve(2 * cells.size() + 16);
    faces.reserve(faces.size() + 3 * cells.size() + 16);
    for (auto &cell : cells) {
        const auto &fg = face_geoms(cell.geom_type);
        const auto &fn = face_nodes(cell.geom_type);
        for (int fi = 0; fi < Geom::face_num(cell.geom_type); ++fi) {
            ObjectType gt = fg[fi];
            const int len = (int)fn[fi].size();
            ObjectId nl[4];
            for (int q = 0; q < len; ++q) nl[q] = cell.node_id.at(fn[fi][q]);
            int which = gt == Geom::Edge ? 0 : (gt == Geom::Quad ? 1 : 2);
            FaceKey4 key;
            key.n.fill(-1);
            face_key(nl, len, key.n.data());
            auto it = maps[which].find(key);
            if (it == maps[which].end()) {
                int fid = (int)faces.size();
                faces.emplace_back(fid, gt, List<ObjectId>(nl, nl + len));
                maps[which][key] = fid;
                auto &f = faces.back();
                f.cell_id = {cell.id, cell.id};
                f.cell_face_id = {fi, fi};
                cell.face_id[fi] = fid;
            } else {
                auto &f = faces[it->second];
                f.cell_id[1] = cell.id;
                f.cell_face_id[1] = fi;
                cell.face_id[fi] = f.id;
            }
        }
    }
    NFACE = (int)faces.size();
}

void Mesh::update_mesh_params() {
    NNODE = (int)nodes.size();
    NFACE = (int)faces.size();
    NCELL = (int)cells.size();
    NZONE = (int)cell_groups.size();
    NMARK = (int)face_groups.size();
}

void Cell::compute_least_square(Mesh &mesh, int dimension) {
    auto &ls = least_square;
    ls.neighbor_num = (int)neighbors.size();
    ls.dr.resize(ls.neighbor_num);
    ls.weight.resize(ls.neighbor_num);
    double Sxx = 0, Sxy = 0, Sxz = 0, Syy = 0, Syz = 0, Szz = 0;
    for (int i = 0; i < ls.neighbor_num; ++i) {
        Vector dr = mesh.cells[neighbors[i]].position - position;
        double wi = 1.0 / (dr * dr);
        ls.dr[i] = dr;
        ls.weight[i] = wi;
        Sxx += wi * (dr.x * dr.x);
        Sxy += wi * (dr.x * dr.y);
        Sxz += wi * (dr.x * dr.z);
        Syy += wi * (dr.y * dr.y);
        Syz += wi * (dr.y * dr.z);
        Szz += wi * (dr.z * dr.z);
    }
    if (dimension == 2) {
        double FM = Sxx * Syy - Sxy * Sxy;
        ls.Cx = {Syy / FM, -Sxy / FM, 0.0};
        ls.Cy = {-Sxy / FM, Sxx / FM, 0.0};
        ls.Cz = {0.0, 0.0, 0.0};
    } else {
        double FM = -Sxz * Sxz * Syy + 2.0 * Sxy * Sxz * Syz - Sxx * Syz * Syz - Sxy * Sxy * Szz + Sxx * Syy * Szz;
        double a = Sxy * Syz - Sxz * Syy;
        double b = Sxz * Syz - Sxy * Szz;
        double c = Syy * Szz - Syz * Syz;
        double d = Sxx * Szz - Sxz * Sxz;
        double e = Sxy * Sxz - Sxx * Syz;
        double f = Sxx * Syy - Sxy * Sxy;
        ls.Cx = {c / FM, b / FM, a / FM};
        ls.Cy = {b / FM, d / FM, e / FM};
        ls.Cz = {a / FM, e / FM, f / FM};
    }
}

void Mesh::build_geom(double scale) {
    for (auto &n : nodes) n.position *= scale;
    update_mesh_params();
    total_volume = 0.0;
    const int D = dimension();
    min_cell_size = -1.0;
    max_cell_magnitude = -1.0;
    NodeList nl;  // reused: one allocation for all cells and faces
    for (auto &cell : cells) {
        nl.clear();
        for (int it : cell.node_id) nl.push_back(nodes.at(it));
        cell.position = centroid(nl);
        cell.volume = cell_volume(cell.geom_type, nl);
        total_volume += cell.volume;
        double mcs = (D == 2) ? 2.0 * std::sqrt(cell.volume / M_PI)
                              : 2.0 * std::pow((3.0 * cell.volume / (4.0 * M_PI)), 1.0 / 3.0);
        double mcm = cell.position.magnitude();
        if (min_cell_size < 0.0) min_cell_size = mcs;
        else min_cell_size = (mcs < min_cell_size) ? mcs : min_cell_size;
        if (max_cell_magnitude < 0.0) max_cell_magnitude = mcm;
        else max_cell_magnitude = (mcm > max_cell_magnitude) ? mcm : max_cell_magnitude;
    }
    for (auto &f : faces) {
        nl.clear();
        for (int it : f.node_id) {
            nl.push_back(nodes[it]);
            nodes[it].group_id = f.group_id;
        }
        f.position = centroid(nl);
        f.area = face_area(f.geom_type, nl);
        f.normal_vector[0] = face_normal(f.geom_type, cells[f.cell_id[0]].position, f.position, nl);
        f.normal_vector[1] = -f.normal_vector[0];
    }
    for (auto &cell : cells) {
        for (int fid : cell.face_id) {
            auto &f = faces[fid];
            for (int cid : f.cell_id) {
                if (cid == cell.id) continue;
                if (std::find(cell.neighbors.begin(), cell.neighbors.end(), cid) != cell.neighbors.end()) continue;
                cell.neighbors.push_back(cid);
            }
        }
        cell.compute_least_square(*this, D);
    }
}

// Gambit neutral-file reader (mesh_reader.cpp:8-139).  Tokens are
// whitespace-separated; node and cell ids are 1-based in the file.
Mesh load_gambit(const String &file_path, double mesh_scale) {
    StringList lines = Utils::read_lines(file_path);
    const int n = (int)lines.size();
    Mesh mesh;
    auto split = [&](int i) {
        if (i >= n) throw std::invalid_argument("gambit: unexpected end of file " + file_path);
        return Utils::split(lines[i]);
    };
    for (int i = 0; i < n; ++i) {
        StringList d = split(i);
        if (d.empty()) continue;
        if (d[0] == "NUMNP") {
            d = split(++i);
            if (d.size() < 6) throw std::invalid_argument("gambit: bad NUMNP record");
            mesh.NNODE = std::stoi(d[0]);
            mesh.NCELL = std::stoi(d[1]);
            mesh.NZONE = std::stoi(d[2]);
            mesh.NMARK = std::stoi(d[3]);
            mesh.NDFCD = std::stoi(d[4]);
            mesh.NDFVL = std::stoi(d[5]);
            mesh.nodes.reserve(mesh.NNODE);
            mesh.cells.reserve(mesh.NCELL);
            mesh.cell_groups.resize(mesh.NZONE);
            mesh.face_groups.resize(mesh.NMARK + 1);
            continue;
        }
        if (d[0] == "NODAL" && d.size() > 1 && d[1] == "COORDINATES") {
            ++i;
            while (i < n) {
                d = split(i);
                if (!d.empty() && d[0] == "ENDOFSECTION") break;
                if (d.empty()) { ++i; continue; }
                int id = std::stoi(d[0]) - 1;
                double x = 0, y = 0, z = 0;
                if (d.size() >= 3) { x = std::stod(d[1]); y = std::stod(d[2]); }
                if (d.size() >= 4) z = std::stod(d[3]);
                mesh.nodes.emplace_back(id, Vector(x, y, z));
                ++i;
            }
            continue;
        }
        if (d[0] == "ELEMENTS/CELLS") {
            ++i;
            while (i < n) {
                d = split(i);
                if (!d.empty() && d[0] == "ENDOFSECTION") break;
                if (d.size() < 3) throw std::invalid_argument("gambit: bad element record");
                int cid = std::stoi(d[0]) - 1;
                int gt = std::stoi(d[1]);
                int cnt = std::stoi(d[2]);
                List<ObjectId> nl;
                for (size_t j = 3; j < d.size(); ++j) nl.push_back(std::stoi(d[j]) - 1);
                if ((int)nl.size() < cnt) {
                    d = split(++i);
                    for (auto &t : d) nl.push_back(std::stoi(t) - 1);
                }
                for (int nid : nl)
                    if (nid < 0 || nid >= (int)mesh.nodes.size())
                        throw std::invalid_argument("gambit: element references unknown node");
                if ((int)nl.size() < Geom::node_num(gt)) throw std::invalid_argument("gambit: short element");
                mesh.cells.emplace_back(cid, gt, nl);
                ++i;
            }
            mesh.generate_face();
            continue;
        }
        if (d[0] == "ELEMENT" && d.size() > 1 && d[1] == "GROUP") {
            d = split(++i);
            if (d.size() < 2) throw std::invalid_argument("gambit: bad group record");
            int gid = std::stoi(d[1]) - 1;
            d = split(++i);
            mesh.cell_names.push_back(d.at(0));
            i += 2;
            while (i < n) {
                d = split(i);
                if (!d.empty() && d[0] == "ENDOFSECTION") break;
                for (auto &t : d) {
                    int cid = std::stoi(t) - 1;
                    mesh.cells.at(cid).group_id = gid;
                    if (gid >= (int)mesh.cell_groups.size()) mesh.cell_groups.resize(gid + 1);
                    mesh.cell_groups[gid].push_back(cid);
                }
                ++i;
            }
            continue;
        }
        if (d[0] == "BOUNDARY" && d.size() > 1 && d[1] == "CONDITIONS") {
            d = split(++i);
            if (d.size() < 3) throw std::invalid_argument("gambit: bad boundary record");
            String name = d[0];
            int gid = (int)mesh.face_names.size();
            mesh.face_names.push_back(name);
            if (gid >= (int)mesh.face_groups.size()) mesh.face_groups.resize(gid + 1);
            ++i;
            while (i < n) {
                d = split(i);
                if (!d.empty() && d[0] == "ENDOFSECTION") break;
                if (d.size() < 3) throw std::invalid_argument("gambit: bad boundary entry");
                int cid = std::stoi(d[0]) - 1;
                int lf = std::stoi(d[2]) - 1;
                auto &cell = mesh.cells.at(cid);
                mesh.faces.at(cell.face_id.at(lf)).group_id = gid;
                ++i;
            }
            continue;
        }
    }
    for (auto &f : mesh.faces) {
        if (f.group_id >= (int)mesh.face_groups.size()) mesh.face_groups.resize(f.group_id + 1);
        mesh.face_groups[f.group_id].push_back(f.id);
    }
    if (mesh.cells.empty()) throw std::invalid_argument("gambit: no cells in " + file_path);
    mesh.build_geom(mesh_scale);
    return mesh;
}

}  // namespace fvmMesh
}  // namespace MESO
