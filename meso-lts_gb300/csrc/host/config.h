// Case-file layer: Config / Patch / Mark / Group of meso-lts
// (include/solver/config.h:38-114), with the same parsing rules and the same
// silent defaults, plus the DVS generators (src/solver/dvs/dvs_generator.cpp).
#pragma once

#include "mesh.h"

namespace MESO::Solver {

enum BoundaryType {
    fluid_interior,
    farfield_inlet,
    pressure_inlet,
    freestream_inlet,
    farfield_outlet,
    pressure_outlet,
    wall,
    slip_wall,
    symmetry,
};

extern const Dict<int> mark_type_map;

namespace PatchType {
constexpr ObjectType zeroGradient = 0, fixedValue = 1, calculated = 2, fromFile = 3, switchType = 4;
}

// One "<name> <patchType> <dataType> <value...>" line set.  Getters of
// missing keys return 0 / zero vector / zeroGradient (patch.cpp:55-85).
class Patch {
    Dict<ObjectType> type;
    Dict<ObjectType> ints;
    Dict<bool> switches = {{"mask", false}};
    Dict<Scalar> scalars;
    Dict<Vector> vectors;
    Dict<List<ObjectType>> ints_list;
    Dict<List<Scalar>> scalars_list;
    Dict<List<Vector>> vectors_list;

public:
    String base_dir;  // fromFile paths resolve against the case directory
    void set_value(StringList &s);
    ObjectType get_type(const String &k) const;
    bool get_switch(const String &k) const;
    ObjectType get_int(const String &k) const;
    Scalar get_scalar(const String &k) const;
    Vector get_vector(const String &k) const;
    ObjectType get_file_int(const String &k, ObjectId id) const;
    Scalar get_file_scalar(const String &k, ObjectId id) const;
    Vector get_file_vector(const String &k, ObjectId id) const;
};

struct Mark {
    String name;
    ObjectId id = 0;
    ObjectType type = fluid_interior;
    String type_name;
    Patch patch;
};

struct Group {
    String name;
    ObjectId id = 0;
    Patch patch;
};

class Config {
    String file_path;

public:
    Dict<String> settings;
    Dict<Group> groups;
    Dict<Mark> marks;
    String base_dir;

    Config() = default;
    explicit Config(const String &file_path);
    void update_config(bool update_patch = true);
    const String &path() const { return file_path; }

    template <class T> T get(const String &key, T default_value, bool print_error = true) const;
    bool has(const String &key) const { return settings.count(key) != 0; }
    const Group &get_cell_group(const fvmMesh::Cell &cell, const fvmMesh::Mesh &mesh) const;
    const Mark &get_face_group(const fvmMesh::Face &face, const fvmMesh::Mesh &mesh) const;
    String resolve(const String &p) const;  // path relative to the case directory
};

}  // namespace MESO::Solver

namespace MESO::DVS {
struct GaussHermiteParams { int dimension; double RT; };
struct HalfRangeGHParams { int dimension; double RT; };
struct NewtonCotesParams { int dimension; };

// The DVS as a Mesh of Cells: position = xi, volume = weight,
// symmetry.id = mirror indices.  tensor_n / axis describe tensor sets.
struct VelocitySet {
    fvmMesh::Mesh mesh;
    int tensor_n = 0;
    List<double> axis;
};

VelocitySet generate_dvs(const String &file, const GaussHermiteParams &p);
VelocitySet generate_dvs(const String &file, const HalfRangeGHParams &p);
VelocitySet generate_dvs(const String &file, const NewtonCotesParams &p);
VelocitySet read_mesh_file(const String &file);  // "Sparse" list
VelocitySet load_gambit_dvs(const String &file);  // unstructured velocity mesh
}  // namespace MESO::DVS
