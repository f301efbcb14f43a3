// oracle/bte_oracle.cpp -- TEST INFRASTRUCTURE ONLY (the oracle).
//
// CPU restatement of the reference's DOM-FVM phonon BTE source iteration.  See
// oracle/bte_oracle.h for what it is used for and how it is pinned.  All
// arithmetic is FP64 with int32 indices, in the reference's evaluation order
// where that order is visible in the source.
#include "bte_oracle.h"
#include "krylov.h"

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const double kPi = M_PI;

struct V3 {
    double x = 0, y = 0, z = 0;
};
inline V3 sub(const V3& a, const V3& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline double dotp(const V3& a, const V3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(const V3& p1, const V3& p2) {  // includes/StaticBTESolver/utility.h:19-21
    return {p1.y * p2.z - p2.y * p1.z, p2.x * p1.z - p1.x * p2.z, p1.x * p2.y - p2.x * p1.y};
}
inline double len(const V3& a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }

struct Mesh {
    int dim = 0;
    double Lx = 0, Ly = 0, Lz = 0;
    std::vector<V3> pts;
    std::vector<std::array<int, 2>> seg;
    std::vector<int> seg_ent;
    std::vector<std::array<int, 3>> tri;
    std::vector<int> tri_ent;
    std::vector<std::array<int, 4>> tet;
};

struct Band {
    double vg, tau, C, Lr;
};
struct BC {
    int index;  // -(entity)-1, src/BTEBoundaryCondition.cpp:21
    int type;
    double T;
};

int leading_int(const std::string& line) { return std::atoi(line.c_str()); }

// src/BTEMesh.cpp:7-130 (COMSOL .mphtxt, sections located by their literal
// "# type name" lines; coordinates scaled by L_x/L_y/L_z).
bool read_mphtxt(const std::string& path, double Lx, double Ly, double Lz, Mesh& m) {
    std::ifstream in(path);
    if (!in.is_open()) return false;
    m.Lx = Lx; m.Ly = Ly; m.Lz = Lz;
    std::string line;
    while (std::getline(in, line) && line != "4 Mesh # class") {}
    std::getline(in, line);  // "4 # version"
    std::getline(in, line);
    m.dim = leading_int(line);
    std::getline(in, line);
    int npts = leading_int(line);
    while (std::getline(in, line) && line != "# Mesh point coordinates") {}
    m.pts.resize(npts);
    for (int i = 0; i < npts; ++i) {
        V3 p;
        if (m.dim == 3) { in >> p.x >> p.y >> p.z; p.x *= Lx; p.y *= Ly; p.z *= Lz; }
        else if (m.dim == 2) { in >> p.x >> p.y; p.x *= Lx; p.y *= Ly; }
        else { in >> p.x; p.x *= Lx; }
        m.pts[i] = p;
    }
    auto read_section = [&](const char* name, int nodes, std::vector<int>& conn, std::vector<int>* ent) {
        while (std::getline(in, line) && line != name) {}
        for (int i = 0; i < 4; ++i) std::getline(in, line);
        int n = leading_int(line);
        std::getline(in, line);
        conn.resize((size_t)n * nodes);
        for (size_t i = 0; i < conn.size(); ++i) in >> conn[i];
        if (ent) {
            for (int i = 0; i < 4; ++i) std::getline(in, line);
            ent->resize(n);
            for (int i = 0; i < n; ++i) in >> (*ent)[i];
        }
        return n;
    };
    std::vector<int> c;
    int n1 = read_section("3 edg # type name", 2, c, &m.seg_ent);
    m.seg.resize(n1);
    for (int i = 0; i < n1; ++i) m.seg[i] = {c[2 * i], c[2 * i + 1]};
    if (m.dim == 1) return true;
    // Triangle entity indices are read only for 3D meshes (:221-246).
    int n2 = read_section("3 tri # type name", 3, c, m.dim == 3 ? &m.tri_ent : nullptr);
    m.tri.resize(n2);
    for (int i = 0; i < n2; ++i) m.tri[i] = {c[3 * i], c[3 * i + 1], c[3 * i + 2]};
    if (m.dim == 2) { m.tri_ent.assign(n2, 0); return true; }
    int n3 = read_section("3 tet # type name", 4, c, nullptr);
    m.tet.resize(n3);
    for (int i = 0; i < n3; ++i) m.tet[i] = {c[4 * i], c[4 * i + 1], c[4 * i + 2], c[4 * i + 3]};
    return true;
}

// src/BTEMesh.cpp:132-147
void make_1d(int N, double Lx, Mesh& m) {
    m.dim = 1; m.Lx = Lx;
    m.pts.resize(N + 1);
    for (int i = 0; i <= N; ++i) m.pts[i].x = Lx / N * i;
    m.seg.resize(N);
    m.seg_ent.assign(N, 0);
    for (int i = 0; i < N; ++i) m.seg[i] = {i, i + 1};
}

// src/BTEBand.cpp:8-26: one band per line, stop at the first line of length <= 1.
bool read_bands(const std::string& path, std::vector<Band>& bands) {
    std::ifstream in(path);
    if (!in.is_open()) return false;
    std::string line;
    while (std::getline(in, line)) {
        if (line.length() <= 1) break;
        std::stringstream ss(line);
        Band b{0, 0, 0, 0};
        ss >> b.vg >> b.tau >> b.C >> b.Lr;
        bands.push_back(b);
    }
    return true;
}

// src/BTEBoundaryCondition.cpp:7-23
bool read_bcs(const std::string& path, std::vector<BC>& bcs) {
    std::ifstream in(path);
    if (!in.is_open()) return false;
    int num = 0;
    std::string line;
    in >> num;
    for (int i = 0; i < 3; ++i) std::getline(in, line);
    for (int i = 0; i < num; ++i) {
        int idx, type;
        double T;
        in >> idx >> type >> T;
        bcs.push_back({-idx - 1, type, T});
    }
    return true;
}

// src/utility.cpp:69-113: Gauss-Legendre nodes by simultaneous Newton
// iteration on P_n (the update uses (n+1)/n times the derivative, which the
// weight formula compensates for), stopped when no node moves by more than 2^-52.
// Returns interleaved (node, weight) on [a, b].
std::vector<double> gauss_legendre(double a, double b, int n) {
    const int N = n - 1, N1 = n, N2 = n + 1;
    std::vector<double> y(N1), y0(N1, 2.0), Lp(N1);
    std::vector<std::vector<double>> L(N1, std::vector<double>(N2, 0.0));
    for (int i = 0; i < N1; ++i) L[i][0] = 1;
    for (int i = 0; i < N1; ++i) y[i] = std::cos((2 * (N - i) + 1) * kPi / (2 * N + 2));
    auto maxdiff = [&]() {
        double r = 0;
        for (int i = 0; i < N1; ++i) r = std::max(std::fabs(y[i] - y0[i]), r);
        return r;
    };
    const double eps = std::pow(2, -52);
    while (maxdiff() > eps) {
        for (int i = 0; i < N1; ++i) L[i][1] = y[i];
        for (int j = 2; j < N1 + 1; ++j)
            for (int i = 0; i < N1; ++i)
                L[i][j] = ((2 * j - 1) * y[i] * L[i][j - 1] - (j - 1) * L[i][j - 2]) / j;
        for (int i = 0; i < N1; ++i) {
            Lp[i] = (N2) * (L[i][N1 - 1] - y[i] * L[i][N2 - 1]) / (1 - y[i] * y[i]);
            y0[i] = y[i];
            y[i] = y0[i] - L[i][N2 - 1] / Lp[i];
        }
    }
    std::vector<double> g;
    for (int i = 0; i < N1; ++i) {
        g.push_back((a * (1 - y[i]) + b * (1 + y[i])) / 2);
        g.push_back((b - a) / ((1 - y[i] * y[i]) * Lp[i] * Lp[i]) * N2 / N1 * N2 / N1);
    }
    return g;
}

}  // namespace

struct oracle_session {
    Mesh mesh;
    std::vector<Band> bands;
    std::vector<BC> bcs;
    int DM = 3, num_theta = 0, num_phi = 0;
    double T_ref = 0, solid_angle = 4 * kPi, WFACTOR = 0;
    int N_cell = 0, N_dir = 0, N_band = 0, N_face = 0;
    // quadrature
    std::vector<double> omega;
    std::vector<V3> dirs, S;
    // geometry
    std::vector<V3> centroid;
    std::vector<double> volume, area;  // area[c*N_face+f]
    std::vector<V3> normal;            // normal[c*N_face+f]
    std::vector<int> nbr;              // nbr[c*N_face+f]
    // state
    std::vector<double> e_curr, e_prev;      // [b][d][c]
    std::vector<double> Tb, ebar, T;         // Tb,ebar [c][b]; T [c]
    std::vector<double> margins, q, q_band;
    long long solves = 0, inner_iters = 0, unconverged = 0;
    double solve_seconds = 0;

    size_t eidx(int b, int d, int c) const { return ((size_t)b * N_dir + d) * N_cell + c; }
    const V3& n_of(int c, int f) const { return normal[(size_t)c * N_face + f]; }
    double a_of(int c, int f) const { return area[(size_t)c * N_face + f]; }
    int nb_of(int c, int f) const { return nbr[(size_t)c * N_face + f]; }

    // src/StaticBTESolver.cpp:48-94
    void set_param(int dm, int nt, int np, double tref) {
        num_theta = nt; num_phi = np; T_ref = tref; DM = dm;
        solid_angle = 4 * kPi;
        if (mesh.dim == 1) {
            T_ref = 0;
            N_cell = (int)mesh.seg.size();
            if (DM == 3) N_dir = nt * np;
            else if (DM == 2) { N_dir = nt; solid_angle = 2 * kPi; }
            N_face = 2;
        }
        if (mesh.dim == 2) {
            N_cell = (int)mesh.tri.size();
            if (DM == 3) { WFACTOR = 2.0; N_dir = 4 * nt * np; }
            else if (DM == 2) { WFACTOR = 4 * kPi; N_dir = 4 * np; }
            N_face = 3;
        } else if (mesh.dim == 3) {
            N_cell = (int)mesh.tet.size();
            if (DM == 3) { WFACTOR = 1.0; N_dir = 8 * nt * np; }
            else if (DM == 2) { WFACTOR = 2.0; N_dir = 4 * nt * np; }
            N_face = 4;
        }
        N_band = (int)bands.size();
    }

    // src/StaticBTESolver.cpp:373-492
    void quadrature() {
        omega.clear(); dirs.clear(); S.clear();
        if (DM == 2) {
            if (mesh.dim >= 2) {
                double dphi = 0.5 * kPi / num_phi;
                std::vector<double> phi(4 * num_phi, 0);
                phi[0] = 0.5 * dphi;
                for (size_t k = 1; k < phi.size(); ++k) phi[k] = phi[k - 1] + dphi;
                for (size_t k = 0; k < phi.size(); ++k) {
                    double w = WFACTOR / phi.size();
                    omega.push_back(w);
                    S.push_back({w * std::sin(phi[k]), w * std::cos(phi[k]), 0});
                    dirs.push_back({std::sin(phi[k]), std::cos(phi[k]), 0});
                }
            } else {
                std::vector<double> g = gauss_legendre(0, kPi, N_dir);
                WFACTOR = 0;
                for (int d = 0; d < N_dir; ++d) {
                    double ct = std::cos(g[2 * d]);
                    double st = std::pow(1 - ct * ct, 0.5);
                    omega.push_back(g[2 * d + 1] * 2);
                    dirs.push_back({ct, st, 0});
                }
                for (int d = 0; d < N_dir; ++d) WFACTOR += omega[d];
                S.assign(N_dir, V3{});
            }
        } else if (DM == 3) {
            if (mesh.dim >= 2) {
                double dth = 0.5 * kPi / num_theta, dphi = 0.5 * kPi / num_phi;
                std::vector<double> theta(mesh.dim == 2 ? num_theta : 2 * num_theta, 0);
                std::vector<double> phi(4 * num_phi, 0);
                theta[0] = 0.5 * dth;
                phi[0] = 0.5 * dphi;
                for (size_t k = 1; k < phi.size(); ++k) phi[k] = phi[k - 1] + dphi;
                for (size_t k = 1; k < theta.size(); ++k) theta[k] = theta[k - 1] + dth;
                omega.assign(theta.size() * phi.size(), 0);
                S.assign(omega.size(), V3{});
                dirs.assign(omega.size(), V3{});
                for (size_t t = 0; t < theta.size(); ++t)
                    for (size_t p = 0; p < phi.size(); ++p) {
                        size_t nf = p + t * 4 * num_phi;
                        omega[nf] = WFACTOR * 2 * std::sin(theta[t]) * std::sin(0.5 * dth) * dphi;
                        double fac = std::sin(0.5 * dphi) * (dth - std::cos(2 * theta[t]) * std::sin(dth));
                        S[nf] = {WFACTOR * std::sin(phi[p]) * fac, WFACTOR * std::cos(phi[p]) * fac,
                                 WFACTOR * 0.5 * dphi * std::sin(2 * theta[t]) * std::sin(dth)};
                        dirs[nf] = {std::sin(theta[t]) * std::sin(phi[p]),
                                    std::sin(theta[t]) * std::cos(phi[p]), std::cos(theta[t])};
                    }
            } else {
                std::vector<double> g = gauss_legendre(-1, 1, num_theta);
                std::vector<double> gp = gauss_legendre(-kPi, kPi, num_phi);
                omega.assign((size_t)num_theta * num_phi, 0);
                dirs.assign(omega.size(), V3{});
                for (int i = 0; i < num_theta; ++i) {
                    double ct = g[2 * i], st = std::pow(1 - ct * ct, 0.5);
                    for (int j = 0; j < num_phi; ++j) {
                        double cp = gp[2 * j] / kPi, sp = std::pow(1 - cp * cp, 0.5);
                        omega[i * num_phi + j] = g[2 * i + 1] * gp[2 * j + 1];
                        dirs[i * num_phi + j] = {ct, st * cp, st * sp};
                    }
                }
                WFACTOR = 0;
                for (int d = 0; d < N_dir; ++d) WFACTOR += omega[d];
                S.assign(N_dir, V3{});
            }
        }
    }

    // src/StaticBTESolver.cpp:494-688
    void geometry() {
        centroid.assign(N_cell, V3{});
        volume.assign(N_cell, 0);
        area.assign((size_t)N_cell * N_face, 0);
        normal.assign((size_t)N_cell * N_face, V3{});
        nbr.assign((size_t)N_cell * N_face, 0);
        const auto& P = mesh.pts;
        std::vector<std::vector<int>> pt2cell;
        if (mesh.dim == 1) {
            for (int c = 0; c < N_cell; ++c) {
                centroid[c].x = mesh.Lx / N_cell * (c + 0.5);
                volume[c] = mesh.Lx / N_cell;
                area[c * 2] = 1; area[c * 2 + 1] = 1;
                normal[c * 2].x = -1; normal[c * 2 + 1].x = 1;
                nbr[c * 2] = c - 1; nbr[c * 2 + 1] = c + 1;
            }
            nbr[0] = -0 - 1;                    // :609
            nbr[(N_cell - 1) * 2 + 1] = -1 - 1;  // :610
            return;
        }
        pt2cell.resize(P.size());
        if (mesh.dim == 2) {
            for (int c = 0; c < N_cell; ++c) {
                const auto& t = mesh.tri[c];
                const V3 &p1 = P[t[0]], &p2 = P[t[1]], &p3 = P[t[2]];
                centroid[c] = {(p1.x + p2.x + p3.x) / 3, (p1.y + p2.y + p3.y) / 3, 0};
                volume[c] = 0.5 * len(cross(sub(p3, p1), sub(p2, p1)));  // utility.cpp:36-38
                for (int v : t) pt2cell[v].push_back(c);
                for (int e = 0; e < 3; ++e) {
                    const V3& q0 = P[t[e % 3]];
                    const V3& q1 = P[t[(e + 1) % 3]];
                    const V3& q2 = P[t[(e + 2) % 3]];
                    area[c * 3 + e] = len(sub(q1, q2));
                    V3 nrm{q2.y - q1.y, q1.x - q2.x, 0};
                    if (dotp(nrm, sub(q0, q1)) > 0) nrm = sub(V3{}, nrm);
                    double l = len(nrm);
                    normal[c * 3 + e] = {nrm.x / l, nrm.y / l, nrm.z / l};
                }
            }
        } else {
            for (int c = 0; c < N_cell; ++c) {
                const auto& t = mesh.tet[c];
                const V3 &p1 = P[t[0]], &p2 = P[t[1]], &p3 = P[t[2]], &p4 = P[t[3]];
                centroid[c] = {(p1.x + p2.x + p3.x + p4.x) / 4, (p1.y + p2.y + p3.y + p4.y) / 4,
                               (p1.z + p2.z + p3.z + p4.z) / 4};
                V3 a = sub(p1, p4), b = sub(p2, p4), cc = sub(p3, p4);  // utility.cpp:46-50
                double det = a.x * (b.y * cc.z - b.z * cc.y) - b.x * (a.y * cc.z - a.z * cc.y) +
                             cc.x * (a.y * b.z - a.z * b.y);
                volume[c] = 1.0 / 6 * std::fabs(det);
                for (int v : t) pt2cell[v].push_back(c);
                for (int f = 0; f < 4; ++f) {
                    const V3& q0 = P[t[f % 4]];
                    const V3& q1 = P[t[(f + 1) % 4]];
                    const V3& q2 = P[t[(f + 2) % 4]];
                    const V3& q3 = P[t[(f + 3) % 4]];
                    V3 n = cross(sub(q3, q1), sub(q3, q2));  // utility.cpp:40-44
                    area[c * 4 + f] = 0.5 * len(n);
                    if (dotp(n, sub(q0, q1)) > 0) n = sub(V3{}, n);
                    double l = len(n);
                    normal[c * 4 + f] = {n.x / l, n.y / l, n.z / l};
                }
            }
        }
        // Boundary elements keyed by their sorted vertex set; the first element
        // in file order wins, as the reference's linear scan (:632-644, :668-679)
        // stops at the first match.
        std::map<std::vector<int>, int> bnd;
        if (mesh.dim == 2) {
            for (size_t i = 0; i < mesh.seg.size(); ++i) {
                std::vector<int> k{mesh.seg[i][0], mesh.seg[i][1]};
                std::sort(k.begin(), k.end());
                bnd.emplace(k, mesh.seg_ent[i]);
            }
        } else {
            for (size_t i = 0; i < mesh.tri.size(); ++i) {
                std::vector<int> k{mesh.tri[i][0], mesh.tri[i][1], mesh.tri[i][2]};
                std::sort(k.begin(), k.end());
                bnd.emplace(k, mesh.tri_ent[i]);
            }
        }
        const int nv = N_face;  // vertices per cell
        for (int c = 0; c < N_cell; ++c) {
            const int* cv = mesh.dim == 2 ? mesh.tri[c].data() : mesh.tet[c].data();
            for (int f = 0; f < N_face; ++f) {
                std::vector<int> fv;
                for (int k = 1; k < nv; ++k) fv.push_back(cv[(f + k) % nv]);
                for (int o : pt2cell[fv[0]]) {  // :617-630, :655-666
                    if (o == c) continue;
                    const int* ov = mesh.dim == 2 ? mesh.tri[o].data() : mesh.tet[o].data();
                    int hit = 0;
                    for (int i = 0; i < nv; ++i)
                        for (int v : fv)
                            if (ov[i] == v) { ++hit; break; }
                    if (hit >= nv - 1) { nbr[c * N_face + f] = o; break; }
                }
                if (nbr[c * N_face + f] == 0) {  // :631, :667 (0 doubles as "not found")
                    std::vector<int> k = fv;
                    std::sort(k.begin(), k.end());
                    auto it = bnd.find(k);
                    if (it != bnd.end()) nbr[c * N_face + f] = -it->second - 1;
                }
            }
        }
    }

    double g_of(int d, int c, int f) const {  // S.n in 2D/3D, s.n in 1D
        return mesh.dim > 1 ? dotp(S[d], n_of(c, f)) : dotp(dirs[d], n_of(c, f));
    }

    // src/StaticBTESolver.cpp:122-160
    void get_Ke(int b, int d, int* rowptr, int* col, double* val) const {
        const Band& B = bands[b];
        int nz = 0;
        rowptr[0] = 0;
        std::vector<std::pair<int, double>> row;
        for (int c = 0; c < N_cell; ++c) {
            row.clear();
            double diag = 0;
            for (int f = 0; f < N_face; ++f) {
                double temp = B.vg * B.tau * a_of(c, f);
                temp *= g_of(d, c, f);
                if (dotp(dirs[d], n_of(c, f)) >= 0) diag += temp;
                else if (nb_of(c, f) >= 0) row.emplace_back(nb_of(c, f), temp);
            }
            diag += mesh.dim > 1 ? volume[c] * omega[d] : volume[c];
            row.emplace_back(c, diag);
            std::sort(row.begin(), row.end());
            for (auto& p : row) { col[nz] = p.first; val[nz] = p.second; ++nz; }
            rowptr[c + 1] = nz;
        }
    }

    // src/StaticBTESolver.cpp:162-269
    void get_Re(int b, int d, const double* ep, const double* eb, double* Re) const {
        const Band& B = bands[b];
        for (int c = 0; c < N_cell; ++c) {
            double r = 0;
            for (int f = 0; f < N_face; ++f) {
                const V3& n = n_of(c, f);
                if (dotp(dirs[d], n) >= 0) continue;
                double a_f = B.vg * B.tau * a_of(c, f);
                a_f *= g_of(d, c, f);
                for (const BC& bc : bcs) {
                    if (nb_of(c, f) != bc.index) continue;
                    if (bc.type == 1) {
                        r -= B.C / solid_angle * (bc.T - T_ref) * a_f;
                    } else if (bc.type == 2) {
                        double es = 0, wsum = 0;
                        for (int di = 0; di < N_dir; ++di) {
                            if (dotp(dirs[di], n) > 0) {
                                double e = ep[eidx(b, di, c)];
                                if (mesh.dim == 3) {
                                    es += e * dotp(S[di], n) * omega[di];
                                    wsum += dotp(S[di], n) * omega[di];
                                } else if (mesh.dim == 2) {
                                    es += e * dotp(S[di], n);
                                    wsum += dotp(S[di], n);
                                } else {
                                    es += e * dotp(dirs[di], n) * omega[di];
                                }
                            }
                        }
                        es = mesh.dim != 1 ? es / wsum : es / kPi;
                        r -= es * a_f;
                    } else if (bc.type == 31) {
                        int it = d / (4 * num_phi), ip = d % (4 * num_phi);
                        if (mesh.dim == 2) ip = ip >= 2 * num_phi ? 6 * num_phi - ip - 1 : 2 * num_phi - ip - 1;
                        else if (mesh.dim == 3) ip = 4 * num_phi - ip - 1;
                        else { std::fprintf(stderr, "type 31 in 1D\n"); std::exit(1); }
                        r -= ep[eidx(b, it * 4 * num_phi + ip, c)] * a_f;
                    } else if (bc.type == 32) {
                        int it = d / (4 * num_phi), ip = d % (4 * num_phi);
                        if (mesh.dim == 2) {
                            ip = 4 * num_phi - ip - 1;
                            r -= ep[eidx(b, it * 4 * num_phi + ip, c)] * a_f;
                        } else if (mesh.dim == 3) {
                            int ix = ip / (2 * num_phi), isx = 2 * num_phi - ip % (2 * num_phi) - 1;
                            r -= ep[eidx(b, it * 4 * num_phi + isx + ix * 2 * num_phi, c)] * a_f;
                        } else { std::fprintf(stderr, "type 32 in 1D\n"); std::exit(1); }
                    } else if (bc.type == 33) {
                        if (mesh.dim < 3) { std::fprintf(stderr, "type 33 below 3D\n"); std::exit(1); }
                        int iz = 2 * num_phi - d / (4 * num_phi) - 1, isz = d % (4 * num_phi);
                        r -= ep[eidx(b, isz + iz * 4 * num_phi, c)] * a_f;
                    } else {
                        std::fprintf(stderr, "unsupported boundary type %d\n", bc.type);
                        std::exit(1);
                    }
                }
            }
            // Re starts at zero (new double[N_cell]() at :738) and accumulates.
            if (mesh.dim != 1) r += eb[(size_t)c * N_band + b] * volume[c] * omega[d];
            else r += eb[(size_t)c * N_band + b] * volume[c];
            Re[c] = r;
        }
    }

    // src/StaticBTESolver.cpp:96-120
    void reductions() {
        for (int b = 0; b < N_band; ++b)
            for (int c = 0; c < N_cell; ++c) {
                double e0 = 0;
                for (int d = 0; d < N_dir; ++d) e0 += e_curr[eidx(b, d, c)] * omega[d];
                Tb[(size_t)c * N_band + b] = e0 / bands[b].C + T_ref;
            }
        for (int c = 0; c < N_cell; ++c) {
            double rr = 0, rn = 0;
            for (int b = 0; b < N_band; ++b) {
                rr += bands[b].Lr * Tb[(size_t)c * N_band + b];
                rn += bands[b].Lr;
            }
            T[c] = rr / rn;
        }
        for (int c = 0; c < N_cell; ++c)
            for (int b = 0; b < N_band; ++b)
                ebar[(size_t)c * N_band + b] = bands[b].C / solid_angle * (T[c] - T_ref);
    }

    // src/StaticBTESolver.cpp:311-321
    double margin() const {
        double m = 0;
        for (size_t i = 0; i < e_curr.size(); ++i) m += std::pow(e_curr[i] - e_prev[i], 2);
        return m / N_band / N_cell;
    }

    // src/StaticBTESolver.cpp:323-370
    void heat_flux() {
        int nbc = (int)bcs.size();
        q.assign(nbc, 0);
        q_band.assign((size_t)nbc * N_band, 0);
        for (int i = 0; i < nbc; ++i) {
            for (int b = 0; b < N_band; ++b) {
                double length = 0, heat = 0;
                for (int c = 0; c < N_cell; ++c)
                    for (int f = 0; f < N_face; ++f) {
                        if (nb_of(c, f) != bcs[i].index) continue;
                        const V3& n = n_of(c, f);
                        for (int d = 0; d < N_dir; ++d) {
                            double e = e_curr[eidx(b, d, c)];
                            if (DM == 3 && mesh.dim == 3) heat += e * dotp(dirs[d], n) * a_of(c, f) * omega[d];
                            else if (mesh.dim == 1) heat += e * dotp(dirs[d], n) * omega[d];
                            else heat += e * dotp(S[d], n) * a_of(c, f);
                        }
                        length += a_of(c, f);
                    }
                double qb = mesh.dim != 1 ? heat / length * bands[b].vg : heat * bands[b].vg;
                q_band[(size_t)i * N_band + b] = qb;
                q[i] += qb;
            }
        }
    }
};

extern "C" {

oracle_session* oracle_open(const char* geo, const char* bc_file, const char* band_file, int DM,
                            int num_theta, int num_phi, double T_ref, double L_x, double L_y,
                            double L_z) {
    auto* s = new oracle_session;
    std::string g(geo);
    bool ok;
    if (g.find('.') == std::string::npos) { make_1d(std::atoi(geo), L_x, s->mesh); ok = true; }
    else ok = read_mphtxt(g, L_x, L_y, L_z, s->mesh);
    ok = ok && read_bands(band_file, s->bands) && read_bcs(bc_file, s->bcs);
    if (!ok) { delete s; return nullptr; }
    s->set_param(DM, num_theta, num_phi, T_ref);
    s->quadrature();
    s->geometry();
    return s;
}

void oracle_close(oracle_session* s) { delete s; }

void oracle_counts(const oracle_session* s, int* c) {
    c[0] = s->N_cell; c[1] = s->N_dir; c[2] = s->N_band; c[3] = s->N_face;
    c[4] = (int)s->bcs.size(); c[5] = s->mesh.dim;
}

void oracle_quadrature(const oracle_session* s, double* dirs, double* S, double* omega, double* sc) {
    for (int d = 0; d < s->N_dir; ++d) {
        dirs[3 * d] = s->dirs[d].x; dirs[3 * d + 1] = s->dirs[d].y; dirs[3 * d + 2] = s->dirs[d].z;
        S[3 * d] = s->S[d].x; S[3 * d + 1] = s->S[d].y; S[3 * d + 2] = s->S[d].z;
        omega[d] = s->omega[d];
    }
    sc[0] = s->solid_angle; sc[1] = s->WFACTOR; sc[2] = s->T_ref;
}

void oracle_geometry(const oracle_session* s, double* volume, double* centroid, double* area,
                     double* normal, int* nbr) {
    for (int c = 0; c < s->N_cell; ++c) {
        volume[c] = s->volume[c];
        centroid[3 * c] = s->centroid[c].x; centroid[3 * c + 1] = s->centroid[c].y;
        centroid[3 * c + 2] = s->centroid[c].z;
    }
    size_t nf = (size_t)s->N_cell * s->N_face;
    for (size_t i = 0; i < nf; ++i) {
        area[i] = s->area[i];
        normal[3 * i] = s->normal[i].x; normal[3 * i + 1] = s->normal[i].y; normal[3 * i + 2] = s->normal[i].z;
        nbr[i] = s->nbr[i];
    }
}

// src/StaticBTESolver.cpp:690-808
int oracle_run(oracle_session* s, int max_iter, double outer_tol, int inner, double inner_tol,
               int threads, long long max_systems) {
    const int NC = s->N_cell, NF = s->N_face;
    const size_t ne = (size_t)s->N_band * s->N_dir * NC;
    s->e_curr.assign(ne, 0.0);
    s->e_prev.assign(ne, 0.0);
    s->Tb.assign((size_t)NC * s->N_band, 0.0);
    s->ebar.assign((size_t)NC * s->N_band, 0.0);  // cell_band_density starts at zero (:92)
    s->T.assign(NC, 0.0);
    s->margins.clear();
    s->solves = s->inner_iters = s->unconverged = 0;
    s->solve_seconds = 0;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    const int nsys = s->N_band * s->N_dir;
    long long done_systems = 0;
    int it = 0;
    for (; it < max_iter; ++it) {
        std::swap(s->e_prev, s->e_curr);
        std::fill(s->e_curr.begin(), s->e_curr.end(), 0.0);
        long long budget = max_systems > 0 ? std::max(0LL, max_systems - done_systems) : nsys;
        int todo = (int)std::min<long long>(nsys, budget);
        long long iters = 0, unconv = 0;
        auto t0 = std::chrono::steady_clock::now();
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : iters, unconv)
        for (int k = 0; k < todo; ++k) {
            int b = k / s->N_dir, d = k % s->N_dir;
            std::vector<int> rowptr(NC + 1), col((size_t)NF * NC + 1);
            std::vector<double> val((size_t)NF * NC + 1), Re(NC);
            s->get_Ke(b, d, rowptr.data(), col.data(), val.data());
            s->get_Re(b, d, s->e_prev.data(), s->ebar.data(), Re.data());
            oracle::Csr A;
            A.n = NC;
            A.rowptr = rowptr;
            A.col.assign(col.begin(), col.begin() + rowptr[NC]);
            A.val.assign(val.begin(), val.begin() + rowptr[NC]);
            double* x = &s->e_curr[s->eidx(b, d, 0)];
            oracle::KrylovResult r = inner == ORACLE_INNER_BICGSTAB
                                         ? oracle::bicgstab_jacobi(A, Re.data(), x, inner_tol, 1000)
                                         : oracle::gmres_ilu0(A, Re.data(), x, inner_tol, 1e-50, 1e5, 1000);
            iters += r.iterations;
            if (!r.converged) ++unconv;
        }
        s->solve_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        s->solves += todo;
        s->inner_iters += iters;
        s->unconverged += unconv;
        done_systems += todo;
        s->reductions();
        double m = s->margin();
        s->margins.push_back(m);
        if (max_systems > 0 && done_systems >= max_systems) { ++it; break; }
        if (m <= outer_tol) { ++it; break; }
    }
    s->heat_flux();
    return it;
}

// One outer iteration (the loop body of src/StaticBTESolver.cpp:707-788) from
// a given state: the previous energy density e_prev_in[n_band][n_dir][n_cell]
// and the equilibrium temperature T_in[n_cell] of the source (ebar = C_b /
// Omega_tot (T_in - T_ref), as _recover_temperature :114-118 sets it).  Writes
// the new e (e_out, may be NULL), T (T_out) and returns the margin against
// e_prev_in.  Used to check that a field is a fixed point of the reference's
// iteration and to drive accelerated solves on the CPU.
double oracle_step(oracle_session* s, const double* e_prev_in, const double* T_in, int inner, double inner_tol,
                   int threads, double* e_out, double* T_out) {
    const int NC = s->N_cell, NF = s->N_face;
    const size_t ne = (size_t)s->N_band * s->N_dir * NC;
    s->e_prev.assign(e_prev_in, e_prev_in + ne);
    s->e_curr.assign(ne, 0.0);
    s->Tb.assign((size_t)NC * s->N_band, 0.0);
    s->ebar.assign((size_t)NC * s->N_band, 0.0);
    for (int c = 0; c < NC; ++c)
        for (int b = 0; b < s->N_band; ++b)
            s->ebar[(size_t)c * s->N_band + b] = s->bands[b].C / s->solid_angle * (T_in[c] - s->T_ref);
    s->T.assign(NC, 0.0);
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    const int nsys = s->N_band * s->N_dir;
    long long iters = 0, unconv = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : iters, unconv)
    for (int k = 0; k < nsys; ++k) {
        int b = k / s->N_dir, d = k % s->N_dir;
        std::vector<int> rowptr(NC + 1), col((size_t)NF * NC + 1);
        std::vector<double> val((size_t)NF * NC + 1), Re(NC);
        s->get_Ke(b, d, rowptr.data(), col.data(), val.data());
        s->get_Re(b, d, s->e_prev.data(), s->ebar.data(), Re.data());
        oracle::Csr A;
        A.n = NC;
        A.rowptr = rowptr;
        A.col.assign(col.begin(), col.begin() + rowptr[NC]);
        A.val.assign(val.begin(), val.begin() + rowptr[NC]);
        double* x = &s->e_curr[s->eidx(b, d, 0)];
        oracle::KrylovResult r = inner == ORACLE_INNER_BICGSTAB
                                     ? oracle::bicgstab_jacobi(A, Re.data(), x, inner_tol, 1000)
                                     : oracle::gmres_ilu0(A, Re.data(), x, inner_tol, 1e-50, 1e5, 1000);
        iters += r.iterations;
        if (!r.converged) ++unconv;
    }
    s->solves += nsys;
    s->inner_iters += iters;
    s->unconverged += unconv;
    s->reductions();
    const double m = s->margin();
    if (e_out) std::memcpy(e_out, s->e_curr.data(), sizeof(double) * ne);
    std::memcpy(T_out, s->T.data(), sizeof(double) * NC);
    s->heat_flux();
    return m;
}

void oracle_temperature(const oracle_session* s, double* T) {
    std::memcpy(T, s->T.data(), sizeof(double) * s->T.size());
}
void oracle_band_temperature(const oracle_session* s, double* Tb) {
    std::memcpy(Tb, s->Tb.data(), sizeof(double) * s->Tb.size());
}
void oracle_heat_flux(const oracle_session* s, double* q, double* q_band) {
    std::memcpy(q, s->q.data(), sizeof(double) * s->q.size());
    if (q_band) std::memcpy(q_band, s->q_band.data(), sizeof(double) * s->q_band.size());
}
int oracle_margins(const oracle_session* s, double* m, int cap) {
    int n = (int)s->margins.size();
    for (int i = 0; i < n && i < cap; ++i) m[i] = s->margins[i];
    return n;
}
void oracle_energy(const oracle_session* s, double* e) {
    std::memcpy(e, s->e_curr.data(), sizeof(double) * s->e_curr.size());
}
void oracle_inner_stats(const oracle_session* s, long long* st, double* seconds) {
    st[0] = s->solves; st[1] = s->inner_iters; st[2] = s->unconverged;
    *seconds = s->solve_seconds;
}

int oracle_assemble(const oracle_session* s, int band, int dir, const double* e_prev,
                    const double* ebar, int* rowptr, int* col, double* val, double* rhs) {
    s->get_Ke(band, dir, rowptr, col, val);
    s->get_Re(band, dir, e_prev, ebar, rhs);
    return rowptr[s->N_cell];
}

static oracle::Csr make_csr(int n, const int* rowptr, const int* col, const double* val) {
    oracle::Csr A;
    A.n = n;
    A.rowptr.assign(rowptr, rowptr + n + 1);
    A.col.assign(col, col + rowptr[n]);
    A.val.assign(val, val + rowptr[n]);
    return A;
}

int oracle_bicgstab_csr(int n, const int* rowptr, const int* col, const double* val,
                        const double* b, double* x, int maxit, double tol, int* converged) {
    oracle::Csr A = make_csr(n, rowptr, col, val);
    oracle::KrylovResult r = oracle::bicgstab_jacobi(A, b, x, tol, maxit);
    if (converged) *converged = r.converged;
    return r.iterations;
}

int oracle_gmres_csr(int n, const int* rowptr, const int* col, const double* val,
                     const double* b, double* x, int maxit, double rtol, int* converged) {
    oracle::Csr A = make_csr(n, rowptr, col, val);
    oracle::KrylovResult r = oracle::gmres_ilu0(A, b, x, rtol, 1e-50, 1e5, maxit);
    if (converged) *converged = r.converged;
    return r.iterations;
}

}  // extern "C"
