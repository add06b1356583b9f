// Host mesh layer: the fvmMesh API of meso-lts (include/mesh/object.h).
//
// Same class and member names as the reference so solver code written
// against fvmMesh keeps compiling: Node, Face, Cell, Mesh, LeastSquare,
// Field<Scalar>/Field<Vector>.  Geometry is evaluated with the reference's
// operation order (this file is compiled with -ffp-contract=off) so the
// tables uploaded to the GPU are bit-identical to the reference's.
#pragma once

#include <array>
#include <cmath>
#include <cstdint>
#include <functional>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

namespace MESO {

using String = std::string;
using StringList = std::vector<std::string>;
using ObjectId = int;
using ObjectType = int;
using Scalar = double;
template <class T> using List = std::vector<T>;
template <class T> using Set = std::array<T, 2>;
template <class T> using Dict = std::unordered_map<std::string, T>;

// VSMALL of include/core/math.h:4; the upwind threshold of every solver.
constexpr double VSMALL = 1e-30;

namespace Math {
// 3-vector with the reference's operator semantics (src/core/math/vector.cpp):
// `*` between vectors is the dot product x*x'+y*y'+z*z' evaluated left to
// right, `/` by a scalar multiplies by its reciprocal, `^` is the cross product.
struct Vector {
    double x = 0.0, y = 0.0, z = 0.0;
    Vector() = default;
    Vector(double a, double b, double c) : x(a), y(b), z(c) {}
    double &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    Vector &operator+=(const Vector &o) { x += o.x; y += o.y; z += o.z; return *this; }
    Vector &operator-=(const Vector &o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    Vector &operator*=(double s) { x *= s; y *= s; z *= s; return *this; }
    Vector &operator/=(double s) { double r = 1.0 / s; x *= r; y *= r; z *= r; return *this; }
    Vector operator-() const { return {-x, -y, -z}; }
    Vector operator*(double s) const { return {x * s, y * s, z * s}; }
    Vector operator/(double s) const { double r = 1.0 / s; return {x * r, y * r, z * r}; }
    Vector operator+(const Vector &o) const { return {x + o.x, y + o.y, z + o.z}; }
    Vector operator-(const Vector &o) const { return {x - o.x, y - o.y, z - o.z}; }
    double operator*(const Vector &o) const { return x * o.x + y * o.y + z * o.z; }
    Vector operator^(const Vector &o) const {
        return {y * o.z - z * o.y, z * o.x - x * o.z, x * o.y - y * o.x};
    }
    double magnitude() const { return std::sqrt(x * x + y * y + z * z); }
    Vector normalize() const {
        double m = magnitude();
        if (m == 0.0) return {0.0, 0.0, 0.0};
        return *this / m;
    }
};
inline Vector operator*(double k, const Vector &v) { return {v.x * k, v.y * k, v.z * k}; }
}  // namespace Math

using Vector = Math::Vector;
using Position = Math::Vector;

enum { cell_field_flag, face_field_flag, node_field_flag };

namespace Geom {
constexpr ObjectType Edge = 1, Quad = 2, Tria = 3, Brick = 4, Wedge = 5, Tetra = 6, Pyram = 7;
int face_num(ObjectType t);
int node_num(ObjectType t);
}  // namespace Geom

namespace fvmMesh {
class Mesh;

struct LeastSquare {
    int neighbor_num = 0;
    List<Scalar> weight;
    List<Vector> dr;
    Vector Cx, Cy, Cz;
};

struct Symmetry {
    int id[3] = {0, 0, 0};
};

class Node {
public:
    ObjectId id;
    ObjectId group_id = 0;
    Position position;
    Node(ObjectId i, const Position &p) : id(i), position(p) {}
};

class Face {
public:
    ObjectType geom_type;
    ObjectId id;
    ObjectId group_id = 0;
    Position position;
    Scalar area = 0.0;
    List<ObjectId> node_id;
    Set<ObjectId> cell_id{-1, -1};
    Set<ObjectId> cell_face_id{-1, -1};
    Set<Vector> normal_vector;
    Face(ObjectId i, ObjectType t, List<ObjectId> nodes) : geom_type(t), id(i), node_id(std::move(nodes)) {}
};

class Cell {
public:
    ObjectType geom_type = 0;
    ObjectId id;
    ObjectId group_id = 0;
    Position position;
    Scalar volume = 0.0;
    List<ObjectId> node_id;
    List<ObjectId> face_id;
    List<ObjectId> neighbors;
    LeastSquare least_square;
    Symmetry symmetry;
    explicit Cell(ObjectId i) : id(i) {}
    Cell(ObjectId i, ObjectType t, List<ObjectId> nodes);
    void compute_least_square(Mesh &mesh, int dimension);
};

class Mesh {
public:
    int NNODE = 0, NFACE = 0, NCELL = 0, NZONE = 0, NMARK = 0, NDFCD = 0, NDFVL = 0;
    double total_volume = 0.0;
    List<Node> nodes;
    List<Face> faces;
    List<Cell> cells;
    List<String> cell_names;
    List<List<ObjectId>> cell_groups;
    List<String> face_names = {"fluid-interior"};
    List<List<ObjectId>> face_groups;
    double min_cell_size = 0.0;
    double max_cell_magnitude = 0.0;

    int dimension() const { return NDFVL; }
    void generate_face();
    void update_mesh_params();
    void build_geom(double scale_ratio = 1.0);
};

// Gambit neutral file -> Mesh with geometry (src/mesh/mesh.cpp:4-11).
Mesh load_gambit(const String &file_path, double mesh_scale = 1.0);
}  // namespace fvmMesh

// Mesh-bound array (include/mesh/object.h:42-75).
template <class T>
class Field {
protected:
    fvmMesh::Mesh *mesh_ptr = nullptr;

public:
    int len = 0;
    ObjectType flag = cell_field_flag;
    std::vector<T> values;
    Field() = default;
    Field(fvmMesh::Mesh &mesh, int f) : mesh_ptr(&mesh), flag(f) {
        len = f == cell_field_flag ? mesh.NCELL : (f == face_field_flag ? mesh.NFACE : mesh.NNODE);
        values.assign(len, T());
    }
    fvmMesh::Mesh *get_mesh() const { return mesh_ptr; }
    T &operator[](int i) { return values[i]; }
    const T &operator[](int i) const { return values[i]; }
    void set_zero() { std::fill(values.begin(), values.end(), T()); }
    void MeshCellValueToField(const std::function<T(fvmMesh::Cell &)> &func) {
        for (int i = 0; i < len; ++i) values[i] = func(mesh_ptr->cells[i]);
    }
    Field<Scalar> heft(int id) const;     // component `id` of a vector field
    void output(const String &file) const;  // 18-digit text, one entry per line
};

namespace Utils {
StringList split(const String &s);
StringList read_lines(const String &file);  // non-empty lines, CR/LF stripped
template <class T> List<T> read_np_file(const String &file);
}  // namespace Utils

template <class T> void read_np_data(const String &file, Field<T> &field);

}  // namespace MESO
