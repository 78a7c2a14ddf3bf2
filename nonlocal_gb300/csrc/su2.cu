// SU2 mesh files, read the way the reference's parser reads them
// (libraries/mesh/mesh_2d/su2_parser.hpp:74-195).
//
// The reference stores every element line as a string in a std::unordered_set
// and every marker in a std::unordered_map keyed by its name, and numbers the
// elements in the iteration order of those containers.  Element and group
// order therefore depend on the standard library's hashed containers, and a
// caller that wants the reference's element numbering for a file has to run
// the same container operations in the same sequence: the same keys
// (trimmed lines, the 2D block's trailing element index removed), the same
// bucket hints, insertions, erasures and moves.  That is what this reader
// does; the rest (node order, local node order per element type) follows the
// file format.  Host code only.
#include "../../include/nlgpu.h"

#include <cctype>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

struct nlgpu_su2 {
    struct Group {
        std::string name;
        int dimension = 0;
        int64_t first = 0, count = 0;
    };
    std::vector<double> nodes;                  // [n][2]
    std::vector<int> type;                      // VTK number of each element
    std::vector<std::vector<int64_t>> elements; // local node order; 2D elements first
    int64_t elements_2d = 0;
    std::vector<Group> groups;                  // in the container's group order
};

namespace {

using Lines = std::unordered_set<std::string>;

// VTK element numbers (vtk_elements_set.hpp:7-15) and the local position of
// each node listed in the file (su2_parser.hpp:55-68)
const std::vector<int>* file_to_local(int vtk) {
    static const std::vector<int> linear{0, 1}, quadratic{0, 2, 1}, triangle{0, 1, 2},
        quadratic_triangle{0, 1, 2, 3, 4, 5}, bilinear{0, 1, 2, 3}, serendipity{0, 2, 4, 6, 1, 3, 5, 7},
        lagrange{2, 0, 6, 8, 1, 3, 7, 5, 4};
    switch (vtk) {
        case 3: return &linear;
        case 21: return &quadratic;
        case 5: return &triangle;
        case 22: return &quadratic_triangle;
        case 9: return &bilinear;
        case 23: return &serendipity;
        case 28: return &lagrange;
        default: return nullptr;
    }
}

bool is_2d(int vtk) { return vtk == 5 || vtk == 22 || vtk == 9 || vtk == 23 || vtk == 28; }

void parse_element(const std::string& line, int& vtk, std::vector<int64_t>& nodes) {
    std::stringstream s{line};
    size_t type = 0;
    s >> type;
    const std::vector<int>* order = file_to_local(int(type));
    if (!order) throw std::domain_error{"Unknown element type."};
    vtk = int(type);
    nodes.assign(order->size(), 0);
    for (const int local : *order) s >> nodes[size_t(local)];
    if (!s) throw std::runtime_error{"element line too short: " + line};
}

// count element lines, trailing whitespace trimmed, and for the 2D block the
// element index after the last space dropped
Lines read_lines(std::istream& f, size_t count, bool drop_index) {
    Lines lines(count);
    std::string line;
    for (size_t k = 0; k < count; ++k) {
        if (!std::getline(f, line)) throw std::runtime_error{"file ends inside an element block"};
        while (!line.empty() && std::isspace(static_cast<unsigned char>(line.back()))) line.pop_back();
        if (drop_index) {
            const size_t cut = line.rfind(' ');
            if (cut == std::string::npos) throw std::runtime_error{"element line without an index: " + line};
            line.resize(cut);
        }
        lines.emplace(std::move(line));
    }
    return lines;
}

bool group_is_2d(const Lines& group) {
    if (group.empty()) throw std::runtime_error{"empty marker"};
    int vtk = 0;
    std::vector<int64_t> nodes;
    parse_element(*group.begin(), vtk, nodes);   // the first element decides, as in the reference
    return is_2d(vtk);
}

void read(const char* path, nlgpu_su2& m) {
    std::ifstream f{path};
    if (!f) throw std::runtime_error{std::string{"cannot open "} + path};
    std::string tag;
    size_t count = 0;
    f >> tag >> tag >> tag >> count;             // NDIME= 2  NELEM= count
    std::getline(f, tag);
    Lines elements_2d = read_lines(f, count, true);
    m.elements_2d = int64_t(elements_2d.size());
    size_t n_nodes = 0;
    f >> tag >> n_nodes;                          // NPOIN= n
    m.nodes.resize(2 * n_nodes);
    for (size_t i = 0; i < n_nodes; ++i) f >> m.nodes[2 * i] >> m.nodes[2 * i + 1] >> tag;
    if (!f) throw std::runtime_error{"cannot read the node block"};
    size_t n_markers = 0;
    f >> tag >> n_markers;                        // NMARK= k
    std::unordered_map<std::string, Lines> groups;
    for (size_t g = 0; g < n_markers; ++g) {
        std::string name;
        size_t elements = 0;
        f >> tag >> name >> tag >> elements;      // MARKER_TAG= name  MARKER_ELEMS= count
        std::getline(f, tag);
        groups[name] = read_lines(f, elements, false);
    }
    if (groups.contains("DEFAULT"))
        throw std::domain_error{"The group name cannot be named \"DEFAULT\", as it is a reserved group name."};
    for (const auto& [name, lines] : groups)
        if (group_is_2d(lines))
            for (const std::string& line : lines)
                if (const auto it = elements_2d.find(line); it != elements_2d.end()) elements_2d.erase(it);
    if (!elements_2d.empty()) groups["DEFAULT"] = std::move(elements_2d);

    size_t total = 0;
    for (const auto& g : groups) total += g.second.size();
    m.elements.resize(total);
    m.type.resize(total);
    int64_t next_2d = 0, next_1d = m.elements_2d;
    for (const auto& [name, lines] : groups) {
        const bool two = group_is_2d(lines);
        int64_t& next = two ? next_2d : next_1d;
        if (next + int64_t(lines.size()) > int64_t(total))
            throw std::runtime_error{"marker elements are not among the listed elements"};
        m.groups.push_back({name, two ? 2 : 1, next, int64_t(lines.size())});
        for (const std::string& line : lines) {
            parse_element(line, m.type[size_t(next)], m.elements[size_t(next)]);
            ++next;
        }
    }
    for (const auto& e : m.elements)
        for (const int64_t v : e)
            if (v < 0 || v >= int64_t(n_nodes)) throw std::runtime_error{"element node out of range"};
}

thread_local std::string g_su2_error;

}  // namespace

extern "C" {

int nlgpu_su2_read(const char* path, nlgpu_su2** mesh) {
    if (!path || !mesh) return NLGPU_ERR_ARG;
    *mesh = nullptr;
    auto* m = new (std::nothrow) nlgpu_su2;
    if (!m) return NLGPU_ERR_OUT_OF_MEMORY;
    try {
        read(path, *m);
    } catch (const std::exception& e) {
        g_su2_error = e.what();
        delete m;
        return NLGPU_ERR_ARG;
    }
    *mesh = m;
    return NLGPU_OK;
}

int nlgpu_su2_free(nlgpu_su2* mesh) {
    delete mesh;
    return NLGPU_OK;
}

const char* nlgpu_su2_last_error(void) { return g_su2_error.c_str(); }

int nlgpu_su2_info(const nlgpu_su2* m, int64_t* n_nodes, int64_t* n_elements_2d, int* nodes_per_element,
                   int* element_type, int* n_groups) {
    if (!m) return NLGPU_ERR_ARG;
    int vtk = m->elements_2d ? m->type[0] : 0;
    for (int64_t e = 0; e < m->elements_2d; ++e)
        if (m->type[size_t(e)] != vtk) vtk = -1;
    if (n_nodes) *n_nodes = int64_t(m->nodes.size() / 2);
    if (n_elements_2d) *n_elements_2d = m->elements_2d;
    if (nodes_per_element) *nodes_per_element = vtk > 0 ? int(file_to_local(vtk)->size()) : 0;
    if (element_type) *element_type = vtk == 9 ? NLGPU_BILINEAR : vtk == 23 ? NLGPU_QUADRATIC_SERENDIPITY : -1;
    if (n_groups) *n_groups = int(m->groups.size());
    return NLGPU_OK;
}

int nlgpu_su2_nodes(const nlgpu_su2* m, double* nodes) {
    if (!m || !nodes) return NLGPU_ERR_ARG;
    std::memcpy(nodes, m->nodes.data(), m->nodes.size() * sizeof(double));
    return NLGPU_OK;
}

int nlgpu_su2_elements_2d(const nlgpu_su2* m, int64_t* elements) {
    if (!m || !elements) return NLGPU_ERR_ARG;
    size_t k = 0;
    for (int64_t e = 0; e < m->elements_2d; ++e) {
        const auto& el = m->elements[size_t(e)];
        if (el.size() != m->elements[0].size()) return NLGPU_ERR_UNSUPPORTED;
        for (const int64_t v : el) elements[k++] = v;
    }
    return NLGPU_OK;
}

int nlgpu_su2_group(const nlgpu_su2* m, int g, char* name, int64_t name_capacity, int* dimension, int64_t* first,
                    int64_t* count, int* nodes_per_element, int64_t* nodes) {
    if (!m || g < 0 || g >= int(m->groups.size())) return NLGPU_ERR_ARG;
    const nlgpu_su2::Group& grp = m->groups[size_t(g)];
    if (name) {
        if (name_capacity < int64_t(grp.name.size()) + 1) return NLGPU_ERR_ARG;
        std::memcpy(name, grp.name.c_str(), grp.name.size() + 1);
    }
    if (dimension) *dimension = grp.dimension;
    if (first) *first = grp.first;
    if (count) *count = grp.count;
    const size_t nen = grp.count ? m->elements[size_t(grp.first)].size() : 0;
    if (nodes_per_element) *nodes_per_element = int(nen);
    if (nodes) {
        size_t k = 0;
        for (int64_t e = grp.first; e < grp.first + grp.count; ++e) {
            const auto& el = m->elements[size_t(e)];
            if (el.size() != nen) return NLGPU_ERR_UNSUPPORTED;
            for (const int64_t v : el) nodes[k++] = v;
        }
    }
    return NLGPU_OK;
}

}  // extern "C"
