// io.cpp -- readers of the StaticBTESolver input formats.
//   BTEMesh: COMSOL .mphtxt (reference behaviour: src/BTEMesh.cpp:7-130) and the
//            uniform 1D mesh (src/BTEMesh.cpp:132-147);
//   BTEBand: "vg tau Ctot Lr" per line until a line of length <= 1 (src/BTEBand.cpp:8-26);
//   BTEBoundaryCondition: count, two skipped lines, "entity type T" rows
//            (src/BTEBoundaryCondition.cpp:7-23).
#include <cstdlib>
#include <sstream>
#include <string>

#include "../../include/StaticBTESolver/BTEBand.h"
#include "../../include/StaticBTESolver/BTEBoundaryCondition.h"
#include "../../include/StaticBTESolver/BTEMesh.h"

namespace {

// Line-oriented cursor over the whole file.
struct Lines {
    std::vector<std::string> v;
    size_t i = 0;
    bool find(const std::string& exact) {
        while (i < v.size()) {
            std::string s = v[i++];
            if (!s.empty() && s.back() == '\r') s.pop_back();
            if (s == exact) return true;
        }
        return false;
    }
    // next line whose comment part is "# <tag>"; returns its leading integer
    long next_tagged(const std::string& tag) {
        while (i < v.size()) {
            const std::string& s = v[i++];
            if (s.find(tag) != std::string::npos) return std::strtol(s.c_str(), nullptr, 10);
        }
        return -1;
    }
};

// Read `count` whitespace-separated numbers starting at the cursor.
template <typename T>
bool read_numbers(Lines& L, size_t count, std::vector<T>& out) {
    out.clear();
    out.reserve(count);
    while (out.size() < count && L.i < L.v.size()) {
        std::istringstream ss(L.v[L.i++]);
        T x;
        while (out.size() < count && ss >> x) out.push_back(x);
    }
    return out.size() == count;
}

}  // namespace

BTEMesh::BTEMesh(std::ifstream& in, double Lx, double Ly, double Lz) : L_x(Lx), L_y(Ly), L_z(Lz) {
    if (!in.is_open()) {
        std::cout << "DEBUG: file not open" << std::endl;
        std::exit(1);
    }
    Lines L;
    for (std::string s; std::getline(in, s);) L.v.push_back(s);
    if (!L.find("4 Mesh # class")) return;
    dim = (int)L.next_tagged("# sdim");
    const long npts = L.next_tagged("# number of mesh points");
    L.find("# Mesh point coordinates");
    std::vector<double> xyz;
    read_numbers(L, (size_t)npts * dim, xyz);
    meshPts.reserve(npts);
    for (long p = 0; p < npts; ++p) {
        auto pt = std::make_shared<staticbtesolver::Point>();
        pt->x = xyz[(size_t)p * dim] * L_x;
        if (dim >= 2) pt->y = xyz[(size_t)p * dim + 1] * L_y;
        if (dim == 3) pt->z = xyz[(size_t)p * dim + 2] * L_z;
        meshPts.push_back(pt);
    }
    // element sections: "3 <name> # type name" ... "# Elements" ... "# Geometric entity indices"
    auto section = [&](const std::string& name, int nodes, std::vector<int>& conn, std::vector<int>* ent) -> long {
        const size_t save = L.i;
        if (!L.find("3 " + name + " # type name")) { L.i = save; return -1; }
        L.next_tagged("# number of nodes per element");
        const long n = L.next_tagged("# number of elements");
        L.find("# Elements");
        read_numbers(L, (size_t)n * nodes, conn);
        if (ent) {
            L.next_tagged("# number of geometric entity indices");
            L.find("# Geometric entity indices");
            read_numbers(L, (size_t)n, *ent);
        }
        return n;
    };
    std::vector<int> conn, ent;
    long n1 = section("edg", 2, conn, &ent);
    for (long k = 0; k < n1; ++k)
        elements1D.push_back(std::make_shared<staticbtesolver::Segment>(conn[2 * k], conn[2 * k + 1], ent[k]));
    if (dim == 1) return;
    // Triangle entity indices are kept only for 3D meshes, as in the reference
    // (in 2D the triangles are the cells and their entity is left at 0).
    long n2 = section("tri", 3, conn, dim == 3 ? &ent : nullptr);
    for (long k = 0; k < n2; ++k)
        elements2D.push_back(std::make_shared<staticbtesolver::Triangle>(conn[3 * k], conn[3 * k + 1],
                                                                         conn[3 * k + 2], dim == 3 ? ent[k] : 0));
    if (dim == 2) return;
    long n3 = section("tet", 4, conn, nullptr);
    for (long k = 0; k < n3; ++k)
        elements3D.push_back(std::make_shared<staticbtesolver::Tetrahedron>(conn[4 * k], conn[4 * k + 1],
                                                                            conn[4 * k + 2], conn[4 * k + 3]));
}

BTEMesh::BTEMesh(int N_cell, double Lx) : dim(1), L_x(Lx), L_y(0), L_z(0) {
    for (int i = 0; i <= N_cell; ++i) meshPts.push_back(std::make_shared<staticbtesolver::Point>(Lx / N_cell * i));
    for (int i = 0; i < N_cell; ++i) elements1D.push_back(std::make_shared<staticbtesolver::Segment>(i, i + 1));
}

BTEBand::BTEBand(std::ifstream& in) {
    if (!in.is_open()) {
        std::cout << "DEBUG: file not open" << std::endl;
        std::exit(1);
    }
    for (std::string line; std::getline(in, line);) {
        if (line.length() <= 1) break;
        std::istringstream ss(line);
        Band b;
        ss >> b.group_velocity >> b.relaxation_time >> b.Ctot >> b.Lr;
        bands.push_back(b);
    }
}

std::ostream& operator<<(std::ostream& os, const BTEBand& band) {
    for (const auto& b : band) os << b << std::endl;
    return os;
}

BTEBoundaryCondition::BTEBoundaryCondition(std::ifstream& in) {
    if (!in.is_open()) {
        std::cout << "DEBUG: file not open" << std::endl;
        std::exit(1);
    }
    int num = 0;
    in >> num;
    std::string skip;
    for (int k = 0; k < 3; ++k) std::getline(in, skip);
    for (int k = 0; k < num; ++k) {
        staticbtesolver::BoundaryCondition bc;
        int entity = 0;
        in >> entity >> bc.type >> bc.temperature;
        bc.index = -entity - 1;
        boundaryConditions.push_back(bc);
    }
}

std::ostream& operator<<(std::ostream& os, const BTEBoundaryCondition& bcs) {
    for (const auto& b : bcs) os << b << std::endl;
    return os;
}
