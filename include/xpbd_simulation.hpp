// xpbd_simulation.hpp -- C++ host of the reference's YAML-configured
// Simulation over the C ABI in xpbd_gpu.h (header-only, C++17, no external
// libraries). It stands in for the reference's host layer around the solver:
//
//   YAML subset reader      yaml-cpp as Config.hpp uses it (include/config/Config.hpp:113-209)
//   gmsh 4.1 ASCII reader   MeshUtils::loadTetMeshFromGmshFile (src/utils/MeshUtils.cpp:92-220)
//   mesh placement          MeshObject::loadAndConfigureMesh (include/simobject/MeshObject.hpp:35-62),
//                           Mesh::resize / massCenter / rotateAbout (src/geometry/Mesh.cpp:224-399)
//   config classes          SimulationConfig.hpp:75-138, ElasticMaterialConfig.hpp:20-50,
//                           XPBDMeshObjectConfig.hpp:62-125, FirstOrderXPBDMeshObjectConfig.hpp:21-59,
//                           RigidPrimitiveConfigs.hpp:26-115, RigidObjectConfig.hpp:18-41
//   Simulation              src/simulation/Simulation.cpp:103-276 (setup, update, _timeStep)
//   rigid primitives        RigidPrimitives.cpp (mass, inertia), RigidObject.cpp:12-14,41-77
//
// Supported objects: XPBDMeshObject, FirstOrderXPBDMeshObject, RigidSphere,
// RigidBox, RigidCylinder (fixed, or free: two-way coupled through the
// solver when it collides, integrated on the host when it does not). Rigid
// meshes and the Virtuoso robot objects throw. There is no graphics: the
// `visualization` key is read and ignored; sim-mode "Visualization" paces
// simulated time to wall-clock time.
#pragma once

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "xpbd_gpu.h"

namespace xpbd_sim {

// ---------------------------------------------------------------------------
// YAML subset: block mappings, block sequences (item mappings on the dash
// line or below it), flow sequences (also over several lines), plain / single-
// / double-quoted scalars, comments. Anchors, aliases, tags, multi-line
// scalars and flow mappings throw.
// ---------------------------------------------------------------------------
struct Node {
    enum Kind { Null, Scalar, Seq, Map } kind = Null;
    std::string text;    // scalar text, quotes removed
    bool quoted = false; // a quoted scalar stays a string
    std::vector<Node> seq;
    std::vector<std::pair<std::string, Node>> map;

    bool is_null() const { return kind == Null; }
    const Node* find(const std::string& key) const {
        if (kind != Map) return nullptr;
        for (const auto& kv : map)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
};

namespace detail {

inline std::string trim(const std::string& s) {
    size_t a = s.find_first_not_of(" \t\r"), b = s.find_last_not_of(" \t\r");
    return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

inline std::string strip_comment(const std::string& line) {
    std::string out;
    char quote = 0;
    for (size_t i = 0; i < line.size(); i++) {
        const char ch = line[i];
        if (quote) {
            out += ch;
            if (ch == quote) quote = 0;
            continue;
        }
        if (ch == '"' || ch == '\'') quote = ch;
        else if (ch == '#' && (i == 0 || line[i - 1] == ' ' || line[i - 1] == '\t')) break;
        out += ch;
    }
    while (!out.empty() && (out.back() == ' ' || out.back() == '\t' || out.back() == '\r')) out.pop_back();
    return out;
}

inline int bracket_depth(const std::string& t) {
    int depth = 0;
    char quote = 0;
    for (char ch : t) {
        if (quote) {
            if (ch == quote) quote = 0;
        } else if (ch == '"' || ch == '\'') {
            quote = ch;
        } else if (ch == '[') {
            depth++;
        } else if (ch == ']') {
            depth--;
        }
    }
    return depth;
}

inline Node scalar_node(const std::string& raw) {
    Node n;
    const std::string t = trim(raw);
    if (t.empty() || t == "~" || t == "null" || t == "Null" || t == "NULL") return n;
    n.kind = Node::Scalar;
    if (t.size() >= 2 && t.front() == t.back() && (t[0] == '"' || t[0] == '\'')) {
        n.text = t.substr(1, t.size() - 2);
        n.quoted = true;
        return n;
    }
    if (t[0] == '&' || t[0] == '*' || t[0] == '!' || t[0] == '|' || t[0] == '>' || t[0] == '{')
        throw std::runtime_error("unsupported YAML construct: " + t);
    n.text = t;
    return n;
}

inline Node value_node(const std::string& raw);

inline Node flow_seq(const std::string& t) {
    Node n;
    n.kind = Node::Seq;
    const std::string inner = t.substr(1, t.size() - 2);
    std::string cur;
    char quote = 0;
    int depth = 0;
    for (char ch : inner) {
        if (quote) {
            cur += ch;
            if (ch == quote) quote = 0;
            continue;
        }
        if (ch == '"' || ch == '\'') quote = ch;
        else if (ch == '[') depth++;
        else if (ch == ']') depth--;
        else if (ch == ',' && depth == 0) {
            n.seq.push_back(value_node(cur));
            cur.clear();
            continue;
        }
        cur += ch;
    }
    if (!trim(cur).empty()) n.seq.push_back(value_node(cur));
    return n;
}

inline Node value_node(const std::string& raw) {
    const std::string t = trim(raw);
    if (!t.empty() && t[0] == '[') {
        if (t.back() != ']') throw std::runtime_error("unterminated flow sequence: " + t);
        return flow_seq(t);
    }
    return scalar_node(t);
}

// `key: value` -> true with (key, value text)
inline bool split_key(const std::string& content, std::string& key, std::string& rest) {
    char quote = 0;
    for (size_t i = 0; i < content.size(); i++) {
        const char ch = content[i];
        if (quote) {
            if (ch == quote) quote = 0;
            continue;
        }
        if (ch == '"' || ch == '\'') quote = ch;
        else if (ch == ':' && (i + 1 == content.size() || content[i + 1] == ' ' || content[i + 1] == '\t')) {
            key = trim(content.substr(0, i));
            if (key.size() >= 2 && key.front() == key.back() && (key[0] == '"' || key[0] == '\''))
                key = key.substr(1, key.size() - 2);
            rest = trim(content.substr(i + 1));
            return true;
        }
    }
    return false;
}

inline bool is_dash(const std::string& c) { return c == "-" || (c.size() >= 2 && c[0] == '-' && c[1] == ' '); }

struct Parser {
    std::vector<std::pair<int, std::string>> lines;  // (indent, content)
    size_t pos = 0;

    Node block() {
        if (pos >= lines.size()) return Node();
        return is_dash(lines[pos].second) ? seq(lines[pos].first) : mapping(lines[pos].first);
    }

    Node seq(int indent) {
        Node out;
        out.kind = Node::Seq;
        while (pos < lines.size()) {
            const int ind = lines[pos].first;
            const std::string content = lines[pos].second;
            if (ind != indent || !is_dash(content)) break;
            const std::string rest = trim(content.substr(1));
            pos++;
            std::string k, r;
            if (rest.empty()) {
                out.seq.push_back(pos < lines.size() && lines[pos].first > indent ? block() : Node());
            } else if (rest[0] != '[' && split_key(rest, k, r)) {
                // a mapping starting on the dash line: its keys align with rest
                const int key_indent = indent + (int)(content.size() - rest.size());
                lines.insert(lines.begin() + (long)pos, {key_indent, rest});
                out.seq.push_back(mapping(key_indent));
            } else {
                out.seq.push_back(value_node(rest));
            }
        }
        return out;
    }

    Node mapping(int indent) {
        Node out;
        out.kind = Node::Map;
        while (pos < lines.size()) {
            const int ind = lines[pos].first;
            const std::string content = lines[pos].second;
            if (ind < indent) break;
            if (ind > indent) throw std::runtime_error("bad indentation at '" + content + "'");
            std::string key, rest;
            if (!split_key(content, key, rest)) throw std::runtime_error("expected 'key: value', got '" + content + "'");
            pos++;
            if (!rest.empty()) {
                out.map.push_back({key, value_node(rest)});
            } else if (pos < lines.size() &&
                       (lines[pos].first > indent || (lines[pos].first == indent && is_dash(lines[pos].second)))) {
                out.map.push_back({key, block()});
            } else {
                out.map.push_back({key, Node()});
            }
        }
        return out;
    }
};

}  // namespace detail

inline Node parse_yaml(const std::string& text) {
    detail::Parser p;
    std::istringstream in(text);
    std::string raw;
    while (std::getline(in, raw)) {
        size_t lead = 0;
        while (lead < raw.size() && (raw[lead] == ' ' || raw[lead] == '\t')) {
            if (raw[lead] == '\t') throw std::runtime_error("tabs in indentation");
            lead++;
        }
        const std::string s = detail::strip_comment(raw);
        const std::string t = detail::trim(s);
        if (t == "---" || t == "..." || t.empty()) continue;
        size_t ind = 0;
        while (ind < s.size() && s[ind] == ' ') ind++;
        // a flow sequence may continue over several lines: join until balanced
        if (!p.lines.empty() && detail::bracket_depth(p.lines.back().second) > 0)
            p.lines.back().second += " " + t;
        else
            p.lines.push_back({(int)ind, t});
    }
    Node root = p.block();
    if (p.pos != p.lines.size()) throw std::runtime_error("unparsed content at '" + p.lines[p.pos].second + "'");
    return root;
}

inline Node load_yaml(const std::string& path) {
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    return parse_yaml(ss.str());
}

// scalar conversions as yaml-cpp's as<T> for the reference's parameter types
inline bool scalar_bool(const Node& n) {
    std::string l = n.text;
    std::transform(l.begin(), l.end(), l.begin(), [](unsigned char c) { return (char)std::tolower(c); });
    if (l == "true" || l == "yes" || l == "on") return true;
    if (l == "false" || l == "no" || l == "off") return false;
    throw std::runtime_error("not a boolean: " + n.text);
}
inline double scalar_double(const Node& n) {
    std::string l = n.text;
    std::transform(l.begin(), l.end(), l.begin(), [](unsigned char c) { return (char)std::tolower(c); });
    if (l == ".inf" || l == "inf" || l == "+.inf" || l == "+inf") return HUGE_VAL;
    if (l == "-.inf" || l == "-inf") return -HUGE_VAL;
    char* end = nullptr;
    const double v = std::strtod(n.text.c_str(), &end);
    if (n.text.empty() || *end) throw std::runtime_error("not a number: " + n.text);
    return v;
}

// ---------------------------------------------------------------------------
// Tet meshes
// ---------------------------------------------------------------------------
struct TetMesh {
    std::vector<double> X;        // 3V, (x0, y0, z0, x1, ...) = the ABI's 3 x V column-major
    std::vector<int32_t> tets;    // 4T
    std::vector<int32_t> faces;   // 3F
    int64_t V() const { return (int64_t)X.size() / 3; }
    int64_t T() const { return (int64_t)tets.size() / 4; }
    int64_t F() const { return (int64_t)faces.size() / 3; }
};

// gmsh 4.1 ASCII: the entities' nodes in (dimension, tag) order, tetrahedra
// (type 4) and triangles (type 2), 1-based node tags to 0-based indices
// (MeshUtils.cpp:92-220 goes over gmsh::model::getEntities in that order).
inline TetMesh read_msh(const std::string& path) {
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open " + path);
    std::vector<std::string> tok;
    std::string w;
    while (f >> w) tok.push_back(w);
    size_t i = 0;
    auto section = [&](const char* name) {
        while (i < tok.size() && tok[i] != name) i++;
        if (i == tok.size()) throw std::runtime_error(std::string(name) + " section missing");
        i++;
    };
    auto ll = [&](size_t k) { return std::stoll(tok.at(k)); };
    section("$MeshFormat");
    if (tok.at(i).rfind("4.", 0) != 0) throw std::runtime_error("gmsh format " + tok[i] + ": only 4.x ASCII");
    if (tok.at(i + 1) != "0") throw std::runtime_error("binary gmsh files are not supported");
    section("$Nodes");
    const long long n_blocks = ll(i), n_nodes = ll(i + 1);
    i += 4;
    struct NB {
        int dim, tag;
        std::vector<double> xyz;
    };
    std::vector<NB> nbs;
    for (long long b = 0; b < n_blocks; b++) {
        const int dim = (int)ll(i), etag = (int)ll(i + 1), param = (int)ll(i + 2);
        const long long n = ll(i + 3);
        i += 4 + (size_t)n;  // skip node tags
        const int per = 3 + (param ? dim : 0);
        NB nb{dim, etag, {}};
        nb.xyz.reserve(3 * n);
        for (long long k = 0; k < n; k++) {
            for (int c = 0; c < 3; c++) nb.xyz.push_back(std::stod(tok.at(i + (size_t)(k * per + c))));
        }
        i += (size_t)(n * per);
        nbs.push_back(std::move(nb));
    }
    section("$Elements");
    const long long n_eb = ll(i);
    i += 4;
    const std::map<int, int> nper = {{1, 2}, {2, 3}, {3, 4}, {4, 4}, {5, 8}, {6, 6}, {7, 5}, {8, 3},
                                     {9, 6}, {10, 9}, {11, 10}, {15, 1}};
    struct EB {
        int dim, tag, type;
        std::vector<int32_t> rows;
    };
    std::vector<EB> ebs;
    for (long long b = 0; b < n_eb; b++) {
        const int dim = (int)ll(i), etag = (int)ll(i + 1), etype = (int)ll(i + 2);
        const long long n = ll(i + 3);
        i += 4;
        auto it = nper.find(etype);
        if (it == nper.end()) throw std::runtime_error("unsupported gmsh element type " + std::to_string(etype));
        const int k = it->second;
        EB eb{dim, etag, etype, {}};
        for (long long e = 0; e < n; e++)
            for (int c = 0; c < k; c++) eb.rows.push_back((int32_t)(ll(i + (size_t)(e * (k + 1) + 1 + c)) - 1));
        i += (size_t)(n * (k + 1));
        ebs.push_back(std::move(eb));
    }
    std::vector<size_t> order(nbs.size());
    for (size_t b = 0; b < order.size(); b++) order[b] = b;
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
        return std::make_pair(nbs[a].dim, nbs[a].tag) < std::make_pair(nbs[b].dim, nbs[b].tag);
    });
    TetMesh m;
    for (size_t b : order) m.X.insert(m.X.end(), nbs[b].xyz.begin(), nbs[b].xyz.end());
    std::vector<size_t> eorder(ebs.size());
    for (size_t b = 0; b < eorder.size(); b++) eorder[b] = b;
    std::stable_sort(eorder.begin(), eorder.end(), [&](size_t a, size_t b) {
        return std::make_pair(ebs[a].dim, ebs[a].tag) < std::make_pair(ebs[b].dim, ebs[b].tag);
    });
    for (size_t b : eorder) {
        if (ebs[b].type == 4) m.tets.insert(m.tets.end(), ebs[b].rows.begin(), ebs[b].rows.end());
        else if (ebs[b].type == 2) m.faces.insert(m.faces.end(), ebs[b].rows.begin(), ebs[b].rows.end());
    }
    if (m.V() != n_nodes) throw std::runtime_error("node count mismatch");
    for (const auto* a : {&m.tets, &m.faces})
        for (int32_t v : *a)
            if (v < 0 || v >= m.V()) throw std::runtime_error("element references a node outside the node list");
    return m;
}

// Surface centre of mass (Mesh::massCenter: origin-apex tets of the faces).
inline std::array<double, 3> mass_center(const std::vector<double>& X, const std::vector<int32_t>& faces) {
    double cm[3] = {0, 0, 0}, vol = 0;
    for (size_t f = 0; f < faces.size(); f += 3) {
        const double* a = &X[3 * faces[f]];
        const double* b = &X[3 * faces[f + 1]];
        const double* c = &X[3 * faces[f + 2]];
        const double cr[3] = {b[1] * c[2] - b[2] * c[1], b[2] * c[0] - b[0] * c[2], b[0] * c[1] - b[1] * c[0]};
        const double v = (a[0] * cr[0] + a[1] * cr[1] + a[2] * cr[2]) / 6.0;
        for (int k = 0; k < 3; k++) cm[k] += 0.25 * (a[k] + b[k] + c[k]) * v;
        vol += v;
    }
    return {cm[0] / vol, cm[1] / vol, cm[2] / vol};
}

// MeshObject::loadAndConfigureMesh: optional resize to max-size, optional
// per-axis size, surface centre of mass to `position`, rotation about
// `position` by x, y, z angles in degrees (x first, the "123" matrix).
inline void place(TetMesh& m, const std::array<double, 3>& position, const std::array<double, 3>& rotation_deg,
                  double max_size, const std::array<double, 3>* size) {
    const int64_t V = m.V();
    auto extent = [&]() {
        std::array<double, 3> lo{HUGE_VAL, HUGE_VAL, HUGE_VAL}, hi{-HUGE_VAL, -HUGE_VAL, -HUGE_VAL};
        for (int64_t v = 0; v < V; v++)
            for (int k = 0; k < 3; k++) {
                lo[k] = std::min(lo[k], m.X[3 * v + k]);
                hi[k] = std::max(hi[k], m.X[3 * v + k]);
            }
        return std::array<double, 3>{hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
    };
    if (max_size > 0) {
        const auto e = extent();
        const double s = max_size / std::max(e[0], std::max(e[1], e[2]));
        for (auto& x : m.X) x *= s;
    }
    if (size) {
        const auto e = extent();
        for (int64_t v = 0; v < V; v++)
            for (int k = 0; k < 3; k++)
                if (e[k] != 0) m.X[3 * v + k] *= (*size)[k] / e[k];
    }
    std::array<double, 3> shift = position;
    if (!m.faces.empty()) {
        const auto cm = mass_center(m.X, m.faces);
        for (int k = 0; k < 3; k++) shift[k] = -cm[k] + position[k];
    }
    for (int64_t v = 0; v < V; v++)
        for (int k = 0; k < 3; k++) m.X[3 * v + k] += shift[k];
    const double pi = 3.14159265358979323846;
    const double x = rotation_deg[0] * pi / 180.0, y = rotation_deg[1] * pi / 180.0, z = rotation_deg[2] * pi / 180.0;
    const double cx = std::cos(x), sx = std::sin(x), cy = std::cos(y), sy = std::sin(y), cz = std::cos(z),
                 sz = std::sin(z);
    const double R[3][3] = {{cy * cz, sx * sy * cz - cx * sz, cx * sy * cz + sx * sz},
                            {cy * sz, sx * sy * sz + cx * cz, cx * sy * sz - sx * cz},
                            {-sy, sx * cy, cx * cy}};
    for (int64_t v = 0; v < V; v++) {
        double d[3];
        for (int k = 0; k < 3; k++) d[k] = m.X[3 * v + k] - position[k];
        for (int r = 0; r < 3; r++) m.X[3 * v + r] = R[r][0] * d[0] + R[r][1] * d[1] + R[r][2] * d[2] + position[r];
    }
}

// ---------------------------------------------------------------------------
// Config classes, with the reference's defaults
// ---------------------------------------------------------------------------
using Vec3 = std::array<double, 3>;

namespace detail {
inline const Node* get(const Node& n, const char* key) {
    const Node* v = n.find(key);
    return (v && !v->is_null()) ? v : nullptr;
}
inline double num(const Node& n, const char* key, double def) {
    const Node* v = get(n, key);
    return v ? scalar_double(*v) : def;
}
inline bool boolean(const Node& n, const char* key, bool def) {
    const Node* v = get(n, key);
    return v ? scalar_bool(*v) : def;
}
inline std::string str(const Node& n, const char* key, const std::string& def) {
    const Node* v = get(n, key);
    return v ? v->text : def;
}
inline Vec3 vec3(const Node& n, const char* key, Vec3 def) {
    const Node* v = get(n, key);
    if (!v) return def;
    if (v->kind != Node::Seq || v->seq.size() != 3) throw std::runtime_error(std::string(key) + ": expected a 3-vector");
    return {scalar_double(v->seq[0]), scalar_double(v->seq[1]), scalar_double(v->seq[2])};
}
inline int option(const Node& n, const char* key, const std::map<std::string, int>& options, const char* def) {
    const std::string v = str(n, key, def);
    auto it = options.find(v);
    if (it == options.end()) throw std::runtime_error(std::string(key) + ": '" + v + "' is not an option");
    return it->second;
}
}  // namespace detail

struct ElasticMaterialConfig {  // ElasticMaterialConfig.hpp:20-50
    std::string name;
    double density = 1000.0, E = 3e6, nu = 0.499, mu_s = 0.5, mu_k = 0.2;
};

enum class ObjectType { XPBD, FirstOrderXPBD, RigidSphere, RigidBox, RigidCylinder };

struct ObjectConfig {
    ObjectType type = ObjectType::XPBD;
    std::string name;
    bool collisions = false, graphics_only = false;
    Vec3 position{0, 0, 0}, velocity{0, 0, 0}, rotation{0, 0, 0};
    // XPBD mesh objects (XPBDMeshObjectConfig.hpp:62-125)
    std::string filename, element_classes_filename;
    double max_size = -1;  // < 0: not given
    bool has_size = false;
    Vec3 size{1, 1, 1};    // also RigidBox's size
    std::vector<std::string> materials;
    bool self_collisions = false;
    int num_solver_iters = 1, num_local_collision_iters = 0;
    int solver_type = XPBD_SOLVER_GAUSS_SEIDEL, constraint_type = XPBD_CONSTRAINT_COMBINED,
        residual_policy = XPBD_RESIDUAL_NEVER;
    double damping_multiplier = 1.0;  // FirstOrderXPBDMeshObjectConfig.hpp:21-59
    bool adjust_damping_to_material = false;
    // rigid primitives (RigidPrimitiveConfigs.hpp:26-115, RigidObjectConfig.hpp:18-41)
    double radius = 1.0, height = 1.0, density = 1000.0;
    bool fixed = false;
    Vec3 angular_velocity{0, 0, 0};

    bool rigid() const { return type != ObjectType::XPBD && type != ObjectType::FirstOrderXPBD; }
};

struct SimulationConfig {  // SimulationConfig.hpp:75-138
    std::string name, description;
    double time_step = 1e-3, end_time = 10.0, g_accel = 9.81, fps = 30.0, collision_rate = 100.0;
    std::string sim_mode = "Visualization", visualization = "VTK";
    std::vector<ElasticMaterialConfig> materials;
    std::vector<ObjectConfig> objects;
};

inline SimulationConfig parse_config(const Node& root) {
    using namespace detail;
    SimulationConfig c;
    c.name = str(root, "name", "");
    c.description = str(root, "description", "");
    c.time_step = num(root, "time-step", 1e-3);
    c.end_time = num(root, "end-time", 10.0);
    c.g_accel = num(root, "g-accel", 9.81);
    c.fps = num(root, "fps", 30.0);
    c.collision_rate = num(root, "collision-rate", 100.0);
    c.sim_mode = str(root, "sim-mode", "Visualization");
    if (c.sim_mode != "Visualization" && c.sim_mode != "AFAP" && c.sim_mode != "Frame-by-frame")
        throw std::runtime_error("sim-mode: '" + c.sim_mode + "' is not an option");
    c.visualization = str(root, "visualization", "VTK");
    if (c.visualization != "None" && c.visualization != "Easy3D" && c.visualization != "VTK")
        throw std::runtime_error("visualization: '" + c.visualization + "' is not an option");
    if (const Node* objs = get(root, "objects")) {
        for (const Node& on : objs->seq) {
            const Node* t = get(on, "type");
            if (!t) throw std::runtime_error("Type of object is needed!");
            ObjectConfig o;
            const std::string type = t->text;
            if (type == "XPBDMeshObject") o.type = ObjectType::XPBD;
            else if (type == "FirstOrderXPBDMeshObject") o.type = ObjectType::FirstOrderXPBD;
            else if (type == "RigidSphere") o.type = ObjectType::RigidSphere;
            else if (type == "RigidBox") o.type = ObjectType::RigidBox;
            else if (type == "RigidCylinder") o.type = ObjectType::RigidCylinder;
            else if (type == "RigidMeshObject" || type == "VirtuosoArm" || type == "VirtuosoRobot")
                throw std::runtime_error("object type '" + type + "' is not provided by the GB300 solver");
            else
                throw std::runtime_error("Unknown type of object! '" + type + "' is not a type of simulation object.");
            o.name = str(on, "name", "");
            o.collisions = boolean(on, "collisions", false);
            o.graphics_only = boolean(on, "graphics-only", false);
            o.position = vec3(on, "position", {0, 0, 0});
            o.velocity = vec3(on, "velocity", {0, 0, 0});
            o.rotation = vec3(on, "rotation", {0, 0, 0});
            if (o.rigid()) {
                o.radius = num(on, "radius", 1.0);
                o.density = num(on, "density", 1000.0);
                o.fixed = boolean(on, "fixed", false);
                o.angular_velocity = vec3(on, "angular-velocity", {0, 0, 0});
                if (o.type == ObjectType::RigidBox) o.size = vec3(on, "size", {1, 1, 1});
                if (o.type == ObjectType::RigidCylinder) o.height = num(on, "height", 1.0);
            } else {
                o.filename = str(on, "filename", "");
                if (const Node* ms = get(on, "materials"))
                    for (const Node& m : ms->seq) o.materials.push_back(m.text);
                o.element_classes_filename = str(on, "element-classes-filename", "");
                o.self_collisions = boolean(on, "self-collisions", false);
                o.num_solver_iters = (int)num(on, "num-solver-iters", 1);
                o.num_local_collision_iters = (int)num(on, "num-local-collision-iters", 0);
                o.solver_type = option(on, "solver-type",
                                       {{"Gauss-Seidel", XPBD_SOLVER_GAUSS_SEIDEL}, {"Jacobi", XPBD_SOLVER_JACOBI},
                                        {"Parallel-Jacobi", XPBD_SOLVER_JACOBI}},
                                       "Gauss-Seidel");
                o.constraint_type = option(on, "constraint-type",
                                           {{"Stable-Neohookean", XPBD_CONSTRAINT_SEPARATE},
                                            {"Stable-Neohookean-Combined", XPBD_CONSTRAINT_COMBINED}},
                                           "Stable-Neohookean-Combined");
                o.residual_policy = option(on, "residual-policy",
                                           {{"Never", XPBD_RESIDUAL_NEVER},
                                            {"Every-Substep", XPBD_RESIDUAL_EVERY_SUBSTEP},
                                            {"Every-Iteration", XPBD_RESIDUAL_EVERY_ITERATION}},
                                           "Never");
                if (o.type == ObjectType::FirstOrderXPBD) {
                    o.damping_multiplier = num(on, "damping-multiplier", 1.0);
                    o.adjust_damping_to_material = boolean(on, "adjust-damping-to-material", false);
                }
                o.max_size = num(on, "max-size", -1.0);
                if (get(on, "size")) {
                    o.has_size = true;
                    o.size = vec3(on, "size", {1, 1, 1});
                }
            }
            c.objects.push_back(o);
        }
    }
    if (const Node* ms = get(root, "materials")) {
        for (const Node& mn : ms->seq) {
            ElasticMaterialConfig m;
            m.name = str(mn, "name", "");
            m.density = num(mn, "density", 1000.0);
            m.E = num(mn, "E", 3e6);
            m.nu = num(mn, "nu", 0.499);
            m.mu_s = num(mn, "mu-s", 0.5);
            m.mu_k = num(mn, "mu-k", 0.2);
            c.materials.push_back(m);
        }
    }
    return c;
}

// ---------------------------------------------------------------------------
// Rigid primitives
// ---------------------------------------------------------------------------
using Quat = std::array<double, 4>;  // (x, y, z, w)

// eulXYZ2Quat (src/utils/GeometryUtils.cpp:104-112) with the rotation in
// degrees turned to radians by RigidObject's factor 3.1415/180 (RigidObject.cpp:12-14)
inline Quat rigid_quat(const Vec3& deg) {
    const double f = 3.1415 / 180.0;
    const double hx = 0.5 * deg[0] * f, hy = 0.5 * deg[1] * f, hz = 0.5 * deg[2] * f;
    const double cx = std::cos(hx), sx = std::sin(hx), cy = std::cos(hy), sy = std::sin(hy), cz = std::cos(hz),
                 sz = std::sin(hz);
    return {sx * cy * cz - cx * sy * sz, cx * sy * cz + sx * cy * sz, cx * cy * sz - sx * sy * cz,
            cx * cy * cz + sx * sy * sz};
}

// mass and diagonal inertia (RigidPrimitives.cpp, pi as 3.1415)
inline void mass_inertia(const ObjectConfig& o, double& m, Vec3& I) {
    if (o.type == ObjectType::RigidBox) {
        const double sx = o.size[0], sy = o.size[1], sz = o.size[2];
        m = sx * sy * sz * o.density;
        I = {1.0 / 12.0 * m * (sy * sy + sz * sz), 1.0 / 12.0 * m * (sx * sx + sz * sz),
             1.0 / 12.0 * m * (sx * sx + sy * sy)};
    } else if (o.type == ObjectType::RigidCylinder) {
        const double r = o.radius, h = o.height;
        m = 3.1415 * r * r * h * o.density;
        I = {1.0 / 12.0 * m * (3 * r * r + h * h), 1.0 / 12.0 * m * (3 * r * r + h * h), 1.0 / 2.0 * m * r * r};
    } else {
        const double r = o.radius;
        m = 4.0 / 3.0 * 3.1415 * r * r * r * o.density;
        const double i = 2.0 / 5.0 * m * r * r;
        I = {i, i, i};
    }
}

// RigidObject::update / velocityUpdate (RigidObject.cpp:41-77) for a free
// body that collides with nothing (the solver integrates colliding ones)
struct FreeBody {
    Vec3 p, v, w, I;
    Quat q, q_prev;
    Vec3 p_prev;
    double m;

    static Quat mult(const Quat& a, const Quat& b) {
        return {a[3] * b[0] + a[0] * b[3] + a[1] * b[2] - a[2] * b[1],
                a[3] * b[1] + a[1] * b[3] + a[2] * b[0] - a[0] * b[2],
                a[3] * b[2] + a[2] * b[3] + a[0] * b[1] - a[1] * b[0],
                a[3] * b[3] - a[0] * b[0] - a[1] * b[1] - a[2] * b[2]};
    }
    static Quat inv(const Quat& q) {
        const double n = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
        return {-q[0] / n, -q[1] / n, -q[2] / n, q[3] / n};
    }
    static Vec3 rot(const Vec3& v, const Quat& q) {
        const double ud = q[0] * v[0] + q[1] * v[1] + q[2] * v[2];
        const double s = 2 * q[3] * q[3] - 1;
        const Vec3 c = {q[1] * v[2] - q[2] * v[1], q[2] * v[0] - q[0] * v[2], q[0] * v[1] - q[1] * v[0]};
        return {2 * ud * q[0] + s * v[0] + 2 * q[3] * c[0], 2 * ud * q[1] + s * v[1] + 2 * q[3] * c[1],
                2 * ud * q[2] + s * v[2] + 2 * q[3] * c[2]};
    }
    void update(double dt, double g) {
        v[2] += dt * (-m * g) / m;
        for (int k = 0; k < 3; k++) p[k] += dt * v[k];
        Vec3 wb = rot(w, inv(q));
        const Vec3 Iw = {I[0] * wb[0], I[1] * wb[1], I[2] * wb[2]};
        const Vec3 c = {wb[1] * Iw[2] - wb[2] * Iw[1], wb[2] * Iw[0] - wb[0] * Iw[2], wb[0] * Iw[1] - wb[1] * Iw[0]};
        for (int k = 0; k < 3; k++) wb[k] += dt * (1.0 / I[k]) * (0.0 - c[k]);
        w = rot(wb, q);
        const Quat dq = mult({w[0], w[1], w[2], 0.0}, q);
        for (int k = 0; k < 4; k++) q[k] += 0.5 * dt * dq[k];
        const double n = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
        for (auto& e : q) e /= n;
    }
    void velocity_update(double dt) {
        for (int k = 0; k < 3; k++) v[k] = (p[k] - p_prev[k]) / dt;
        const Quat dq = mult(q, inv(q_prev));
        const double sgn = dq[3] < 0 ? -1.0 : 1.0;
        for (int k = 0; k < 3; k++) w[k] = 2 / dt * dq[k] * sgn;
        p_prev = p;
        q_prev = q;
    }
};

// ---------------------------------------------------------------------------
// Simulation
// ---------------------------------------------------------------------------
inline std::vector<int64_t> read_element_classes(const std::string& path) {
    // FileUtils::readVectorFromFile<int>: one integer per line, up to the
    // first line that does not start with one
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open " + path);
    std::vector<int64_t> out;
    std::string line;
    while (std::getline(f, line)) {
        std::istringstream ss(line);
        long long v;
        if (!(ss >> v)) break;
        out.push_back(v);
    }
    return out;
}

inline void check(int st, xpbd_ctx* c, const char* what) {
    if (st != XPBD_OK)
        throw std::runtime_error(std::string(what) + ": " + (c ? xpbd_last_error(c) : xpbd_status_string(st)));
}

class Simulation {
   public:
    struct Object {
        ObjectConfig cfg;
        TetMesh mesh;
        xpbd_ctx* ctx = nullptr;
    };
    struct Rigid {
        ObjectConfig cfg;
        int kind;
        Vec3 position, dims;
        Quat quat;
        double mass = 0;
        Vec3 inertia{0, 0, 0};
        std::unique_ptr<FreeBody> host_body;  // free and colliding with nothing
    };

    // path: a YAML file; relative mesh paths resolve against its directory
    explicit Simulation(const std::string& path) {
        cfg_ = parse_config(load_yaml(path));
        const size_t slash = path.find_last_of('/');
        base_dir_ = slash == std::string::npos ? "." : path.substr(0, slash);
    }
    Simulation(const SimulationConfig& cfg, const std::string& base_dir) : cfg_(cfg), base_dir_(base_dir) {}
    Simulation(const Simulation&) = delete;
    Simulation& operator=(const Simulation&) = delete;
    ~Simulation() {
        for (auto& o : objects_)
            if (o.ctx) xpbd_destroy(o.ctx);
    }

    const SimulationConfig& config() const { return cfg_; }
    double time() const { return time_; }
    std::vector<Object>& objects() { return objects_; }
    std::vector<Rigid>& rigids() { return rigids_; }

    // Simulation::setup (Simulation.cpp:103-137): objects from their configs
    void setup() {
        if (setup_) throw std::runtime_error("setup() called twice");
        setup_ = true;
        for (const ObjectConfig& oc : cfg_.objects) {
            if (oc.graphics_only) continue;
            if (oc.rigid()) {
                Rigid r;
                r.cfg = oc;
                r.position = oc.position;
                r.quat = rigid_quat(oc.rotation);
                if (oc.type == ObjectType::RigidBox) {
                    r.kind = XPBD_SDF_BOX;
                    r.dims = oc.size;
                } else if (oc.type == ObjectType::RigidCylinder) {
                    r.kind = XPBD_SDF_CYLINDER;
                    r.dims = {oc.radius, oc.height, 0.0};
                } else {
                    r.kind = XPBD_SDF_SPHERE;
                    r.dims = {oc.radius, 0.0, 0.0};
                }
                if (!oc.fixed) {
                    mass_inertia(oc, r.mass, r.inertia);
                    if (!oc.collisions) {
                        r.host_body.reset(new FreeBody{r.position, oc.velocity, oc.angular_velocity, r.inertia,
                                                       r.quat, r.quat, r.position, r.mass});
                    }
                }
                rigids_.push_back(std::move(r));
            } else {
                add_object(oc);
            }
        }
        int colliding = 0;
        for (auto& o : objects_) colliding += o.cfg.collisions;
        bool free_colliding = false;
        for (auto& r : rigids_) free_colliding |= !r.cfg.fixed && r.cfg.collisions;
        if (colliding > 1 && free_colliding)
            throw std::runtime_error("a free rigid body colliding with more than one XPBD object is not provided");
        push_rigids(false);
    }

    // Simulation::_timeStep (Simulation.cpp:197-276): every object's step
    // (detection on the shared cadence, update, velocity update), then the
    // free bodies that collide with nothing
    void time_step() {
        for (auto& o : objects_) check(xpbd_step(o.ctx, 1), o.ctx, "xpbd_step");
        for (auto& r : rigids_)
            if (r.host_body) {
                r.host_body->update(cfg_.time_step, cfg_.g_accel);
                r.host_body->velocity_update(cfg_.time_step);
            }
        time_ += cfg_.time_step;
    }

    // Simulation::update (Simulation.cpp:139-195): steps until end-time (or
    // max_steps); "Visualization" keeps simulated time behind wall-clock time
    int update(int max_steps = -1) {
        const auto start = std::chrono::steady_clock::now();
        int n = 0;
        while (time_ < cfg_.end_time && (max_steps < 0 || n < max_steps)) {
            if (cfg_.sim_mode == "Visualization") {
                const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
                if (time_ > wall) std::this_thread::sleep_for(std::chrono::duration<double>(time_ - wall));
            }
            time_step();
            n++;
        }
        for (auto& o : objects_) check(xpbd_synchronize(o.ctx), o.ctx, "xpbd_synchronize");
        return n;
    }

    // the object's current positions (3V, the ABI layout)
    std::vector<double> positions(const std::string& name) {
        for (auto& o : objects_)
            if (o.cfg.name == name) {
                std::vector<double> x(o.mesh.X.size());
                check(xpbd_get_positions(o.ctx, x.data()), o.ctx, "xpbd_get_positions");
                return x;
            }
        throw std::runtime_error("no object named " + name);
    }

    // kinematic motion of a fixed rigid object between steps
    void move_rigid(const std::string& name, const Vec3& position, const Vec3* rotation_deg = nullptr) {
        for (auto& r : rigids_)
            if (r.cfg.name == name) {
                if (!r.cfg.fixed) throw std::runtime_error("rigid object " + name + " is free: the solver moves it");
                r.position = position;
                if (rotation_deg) r.quat = rigid_quat(*rotation_deg);
                push_rigids(true);
                return;
            }
        throw std::runtime_error("no rigid object named " + name);
    }

   private:
    const ElasticMaterialConfig& material(const std::string& name) const {
        for (const auto& m : cfg_.materials)
            if (m.name == name) return m;
        throw std::runtime_error("material '" + name + "' is not defined");
    }

    std::string resolve(const std::string& p) const { return (!p.empty() && p[0] == '/') ? p : base_dir_ + "/" + p; }

    void add_object(const ObjectConfig& oc) {
        Object o;
        o.cfg = oc;
        o.mesh = read_msh(resolve(oc.filename));
        place(o.mesh, oc.position, oc.rotation, oc.max_size, oc.has_size ? &oc.size : nullptr);
        const int64_t T = o.mesh.T();
        std::vector<ElasticMaterialConfig> mats;
        for (const auto& name : oc.materials) mats.push_back(material(name));
        if (mats.empty()) mats.push_back(ElasticMaterialConfig{});
        std::vector<int64_t> cls(T, 0);
        if (!oc.element_classes_filename.empty()) {
            cls = read_element_classes(resolve(oc.element_classes_filename));
            if ((int64_t)cls.size() != T)
                throw std::runtime_error("Element classes file has a different number of elements than the mesh!");
        }
        std::vector<double> E(T), nu(T), rho(T);
        for (int64_t t = 0; t < T; t++) {
            // classes past the material list take the last material (XPBDMeshObject.cpp:289-297)
            const auto& m = mats[(size_t)std::min<int64_t>(cls[t], (int64_t)mats.size() - 1)];
            E[t] = m.E;
            nu[t] = m.nu;
            rho[t] = m.density;
        }
        xpbd_params p;
        xpbd_default_params(&p);
        p.dt = cfg_.time_step;
        p.g_accel = cfg_.g_accel;
        p.collision_rate = cfg_.collision_rate;
        p.num_iters = oc.num_solver_iters;
        p.solver_type = oc.solver_type;
        p.constraint_type = oc.constraint_type;
        p.residual_policy = oc.residual_policy;
        p.num_local_collision_iters = oc.num_local_collision_iters;
        p.first_order = oc.type == ObjectType::FirstOrderXPBD ? 1 : 0;
        p.damping_multiplier = oc.damping_multiplier;
        p.adjust_damping_to_material = oc.adjust_damping_to_material ? 1 : 0;
        p.self_collisions = oc.self_collisions ? 1 : 0;
        const bool faces = oc.collisions && o.mesh.F() > 0;
        xpbd_mesh_desc d{o.mesh.V(), T, faces ? o.mesh.F() : 0, o.mesh.X.data(), o.mesh.tets.data(),
                         faces ? o.mesh.faces.data() : nullptr, E.data(), nu.data(), rho.data()};
        check(xpbd_create(&d, &p, &o.ctx), nullptr, "xpbd_create");
        if (oc.velocity[0] != 0 || oc.velocity[1] != 0 || oc.velocity[2] != 0) {
            std::vector<double> v(o.mesh.X.size());
            for (size_t i = 0; i < v.size(); i++) v[i] = oc.velocity[i % 3];
            check(xpbd_set_velocities(o.ctx, v.data()), o.ctx, "xpbd_set_velocities");
        }
        objects_.push_back(std::move(o));
    }

    // the colliding rigid objects as the solver's SDF table; setting the SDFs
    // drops the free bodies, so their live state is carried over
    void push_rigids(bool carry_state) {
        std::vector<Rigid*> live;
        for (auto& r : rigids_)
            if (r.cfg.collisions) live.push_back(&r);
        if (live.empty()) return;
        for (auto& o : objects_) {
            if (!o.cfg.collisions) continue;
            std::vector<std::array<double, 13>> state(live.size());
            if (carry_state)
                for (size_t s = 0; s < live.size(); s++)
                    if (!live[s]->cfg.fixed)
                        check(xpbd_get_rigid_body(o.ctx, 0, (int)s, state[s].data()), o.ctx, "xpbd_get_rigid_body");
            std::vector<int32_t> kind;
            std::vector<double> pos, quat, dims;
            for (size_t s = 0; s < live.size(); s++) {
                Rigid* r = live[s];
                if (carry_state && !r->cfg.fixed) {
                    r->position = {state[s][0], state[s][1], state[s][2]};
                    r->quat = {state[s][3], state[s][4], state[s][5], state[s][6]};
                    r->cfg.velocity = {state[s][7], state[s][8], state[s][9]};
                    r->cfg.angular_velocity = {state[s][10], state[s][11], state[s][12]};
                }
                kind.push_back(r->kind);
                pos.insert(pos.end(), r->position.begin(), r->position.end());
                quat.insert(quat.end(), r->quat.begin(), r->quat.end());
                dims.insert(dims.end(), r->dims.begin(), r->dims.end());
            }
            check(xpbd_set_sdfs(o.ctx, (int)live.size(), kind.data(), pos.data(), quat.data(), dims.data()), o.ctx,
                  "xpbd_set_sdfs");
            for (size_t s = 0; s < live.size(); s++) {
                Rigid* r = live[s];
                if (!r->cfg.fixed)
                    check(xpbd_set_rigid_body(o.ctx, 0, (int)s, r->mass, r->inertia.data(), r->cfg.velocity.data(),
                                              r->cfg.angular_velocity.data()),
                          o.ctx, "xpbd_set_rigid_body");
            }
        }
    }

    SimulationConfig cfg_;
    std::string base_dir_;
    std::vector<Object> objects_;
    std::vector<Rigid> rigids_;
    double time_ = 0.0;
    bool setup_ = false;
};

}  // namespace xpbd_sim
