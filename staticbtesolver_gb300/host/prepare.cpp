// prepare.cpp -- angular quadrature, cell geometry and face connectivity.
//
// What is computed is fixed by the method (StaticBTESolver::setParam,
// src/StaticBTESolver.cpp:48-94, and _preprocess, :372-688); how it is
// computed here is this project's: flat arrays instead of per-face
// shared_ptr<Point>, and face matching through one hash map of sorted vertex
// keys (O(cells)) instead of a per-face scan of the vertex-to-cell lists and
// of all boundary elements.  Two behaviours of the reference are kept on
// purpose because they change results:
//  * the neighbour slot value 0 doubles as "no neighbour found" (:631, :667):
//    a face whose only match is cell 0, or that has no match, is looked up
//    among the boundary elements, and keeps 0 (an interior link to cell 0)
//    when none matches;
//  * the boundary element that wins is the first one in file order.
#include <fstream>
#include "prepare.h"

#include <chrono>
#include <cmath>
#include <unordered_map>

#include "../../include/bte_cuda.h"

namespace sbte {
namespace {

struct FaceKey {
    int v[3];
    bool operator==(const FaceKey& o) const { return v[0] == o.v[0] && v[1] == o.v[1] && v[2] == o.v[2]; }
};
struct FaceKeyHash {
    size_t operator()(const FaceKey& k) const {
        uint64_t h = (uint64_t)(uint32_t)k.v[0] * 0x9E3779B97F4A7C15ull;
        h ^= (uint64_t)(uint32_t)k.v[1] + 0x7F4A7C159E3779B9ull + (h << 6) + (h >> 2);
        h ^= (uint64_t)(uint32_t)k.v[2] + 0x94D049BB133111EBull + (h << 6) + (h >> 2);
        return (size_t)h;
    }
};
FaceKey make_key(int a, int b, int c = -1) {
    int v[3] = {a, b, c};
    if (v[0] > v[1]) std::swap(v[0], v[1]);
    if (c >= 0) {
        if (v[1] > v[2]) std::swap(v[1], v[2]);
        if (v[0] > v[1]) std::swap(v[0], v[1]);
    }
    return FaceKey{{v[0], v[1], v[2]}};
}

double now_ms() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Direction sets (src/StaticBTESolver.cpp:373-492).
int quadrature(Prepared& P, std::string& err) {
    const int dim = P.dim, nt = P.num_theta, np = P.num_phi;
    P.s.clear(); P.S.clear(); P.omega.clear();
    auto push = [&](double w, double sx, double sy, double sz, double Sx, double Sy, double Sz) {
        P.omega.push_back(w);
        P.s.insert(P.s.end(), {sx, sy, sz});
        P.S.insert(P.S.end(), {Sx, Sy, Sz});
    };
    if (P.DM == 2 && dim >= 2) {
        // 4 num_phi azimuthal bins of width pi/(2 num_phi), equal weights WFACTOR/(4 num_phi)
        const double dphi = 0.5 * M_PI / np;
        double phi = 0.5 * dphi;
        for (int k = 0; k < 4 * np; ++k, phi += dphi) {
            const double w = P.wfactor / (4 * np);
            push(w, std::sin(phi), std::cos(phi), 0, w * std::sin(phi), w * std::cos(phi), 0);
        }
    } else if (P.DM == 2) {
        // 1D, DM=2: Gauss-Legendre in theta over (0, pi), weight 2 W
        std::vector<double> g = staticbtesolver::GaussIntegrationPoints(0, M_PI, P.n_dir);
        P.wfactor = 0;
        for (int d = 0; d < P.n_dir; ++d) {
            const double ct = std::cos(g[2 * d]);
            push(g[2 * d + 1] * 2, ct, std::sqrt(1 - ct * ct), 0, 0, 0, 0);
            P.wfactor += g[2 * d + 1] * 2;
        }
    } else if (dim >= 2) {
        // DM=3: theta bins of width pi/(2 num_theta) (upper hemisphere in 2D,
        // whole sphere in 3D) times 4 num_phi azimuthal bins; control angle and
        // the angle-integrated direction S in closed form.
        const double dth = 0.5 * M_PI / nt, dphi = 0.5 * M_PI / np;
        const int ntheta = dim == 2 ? nt : 2 * nt;
        double th = 0.5 * dth;
        for (int t = 0; t < ntheta; ++t, th += dth) {
            double phi = 0.5 * dphi;
            for (int k = 0; k < 4 * np; ++k, phi += dphi) {
                const double W = P.wfactor;
                const double lat = std::sin(0.5 * dphi) * (dth - std::cos(2 * th) * std::sin(dth));
                push(W * 2 * std::sin(th) * std::sin(0.5 * dth) * dphi, std::sin(th) * std::sin(phi),
                     std::sin(th) * std::cos(phi), std::cos(th), W * std::sin(phi) * lat, W * std::cos(phi) * lat,
                     W * 0.5 * dphi * std::sin(2 * th) * std::sin(dth));
            }
        }
    } else {
        // 1D, DM=3: Gauss-Legendre in cos(theta) over (-1, 1) and in phi over
        // (-pi, pi); the reference uses node/pi of the phi rule as cos(phi).
        std::vector<double> g = staticbtesolver::GaussIntegrationPoints(-1, 1, nt);
        std::vector<double> gp = staticbtesolver::GaussIntegrationPoints(-M_PI, M_PI, np);
        P.wfactor = 0;
        for (int i = 0; i < nt; ++i) {
            const double ct = g[2 * i], st = std::sqrt(1 - ct * ct);
            for (int j = 0; j < np; ++j) {
                const double cp = gp[2 * j] / M_PI, sp = std::sqrt(1 - cp * cp);
                push(g[2 * i + 1] * gp[2 * j + 1], ct, st * cp, st * sp, 0, 0, 0);
                P.wfactor += g[2 * i + 1] * gp[2 * j + 1];
            }
        }
    }
    if ((int)P.omega.size() != P.n_dir) {
        err = "quadrature produced an unexpected number of directions";
        return BTE_ERR_INVALID_ARGUMENT;
    }
    return 0;
}

int geometry(const BTEMesh& mesh, Prepared& P, std::string& err) {
    const int n = P.n_cell, F = P.n_face, dim = P.dim;
    P.volume.assign(n, 0.0);
    P.centroid.assign((size_t)n * 3, 0.0);
    P.area.assign((size_t)n * F, 0.0);
    P.normal.assign((size_t)n * F * 3, 0.0);
    P.nbr.assign((size_t)n * F, 0);
    const auto& X = mesh.meshPts;
    if (dim == 1) {
        const double h = mesh.L_x / n;
        for (int c = 0; c < n; ++c) {
            P.centroid[3 * c] = h * (c + 0.5);
            P.volume[c] = h;
            P.area[2 * c] = P.area[2 * c + 1] = 1.0;
            P.normal[6 * c] = -1.0;
            P.normal[6 * c + 3] = 1.0;
            P.nbr[2 * c] = c - 1;
            P.nbr[2 * c + 1] = c + 1;
        }
        P.nbr[0] = -1;                      // left end is boundary entity 0
        P.nbr[2 * (n - 1) + 1] = -2;        // right end is boundary entity 1
        return 0;
    }
    const int nv = F;  // vertices per cell
    auto vert = [&](int c, int k) -> int {
        return dim == 2 ? mesh.elements2D[c]->index[k] : mesh.elements3D[c]->index[k];
    };
    for (int c = 0; c < n; ++c)
        for (int k = 0; k < nv; ++k)
            if (vert(c, k) < 0 || vert(c, k) >= (int)X.size()) {
                err = "mesh element refers to a point that does not exist";
                return BTE_ERR_INVALID_ARGUMENT;
            }
    std::unordered_map<FaceKey, int, FaceKeyHash> first_cell;  // face -> first (cell*F+face)
    first_cell.reserve((size_t)n * F);
    for (int c = 0; c < n; ++c) {
        staticbtesolver::Point p[4];
        for (int k = 0; k < nv; ++k) p[k] = *X[vert(c, k)];
        double cx = 0, cy = 0, cz = 0;
        for (int k = 0; k < nv; ++k) { cx += p[k].x; cy += p[k].y; cz += p[k].z; }
        P.centroid[3 * c] = cx / nv;
        P.centroid[3 * c + 1] = cy / nv;
        P.centroid[3 * c + 2] = dim == 3 ? cz / nv : 0.0;
        P.volume[c] = dim == 2 ? staticbtesolver::getArea(p[0], p[1], p[2])
                               : staticbtesolver::getVolume(p[0], p[1], p[2], p[3]);
        for (int f = 0; f < F; ++f) {
            // face f is opposite local vertex f; its normal points away from it
            const staticbtesolver::Point& q0 = p[f];
            const staticbtesolver::Point& q1 = p[(f + 1) % nv];
            const staticbtesolver::Point& q2 = p[(f + 2) % nv];
            staticbtesolver::Point nrm;
            double A;
            if (dim == 2) {
                A = (q1 - q2).length();
                nrm = staticbtesolver::Point(q2.y - q1.y, q1.x - q2.x, 0);
            } else {
                const staticbtesolver::Point& q3 = p[(f + 3) % nv];
                nrm = staticbtesolver::cross_prod(q3 - q1, q3 - q2);
                A = 0.5 * nrm.length();
            }
            if (staticbtesolver::dot_prod(nrm, q0 - q1) > 0) nrm = staticbtesolver::Point() - nrm;
            nrm = nrm / nrm.length();
            const size_t cf = (size_t)c * F + f;
            P.area[cf] = A;
            P.normal[3 * cf] = nrm.x;
            P.normal[3 * cf + 1] = nrm.y;
            P.normal[3 * cf + 2] = nrm.z;
            const FaceKey key = dim == 2 ? make_key(vert(c, (f + 1) % nv), vert(c, (f + 2) % nv))
                                         : make_key(vert(c, (f + 1) % nv), vert(c, (f + 2) % nv), vert(c, (f + 3) % nv));
            auto it = first_cell.find(key);
            if (it == first_cell.end()) {
                first_cell.emplace(key, (int)cf);
            } else {
                // the first cell that met this face and this one are neighbours
                const int other = it->second / F;
                if (P.nbr[cf] == 0) P.nbr[cf] = other;
                if (P.nbr[(size_t)it->second] == 0) P.nbr[(size_t)it->second] = c;
            }
        }
    }
    // boundary elements: first in file order wins
    std::unordered_map<FaceKey, int, FaceKeyHash> bnd;
    if (dim == 2) {
        for (const auto& sgm : mesh.elements1D)
            bnd.emplace(make_key(sgm->index[0], sgm->index[1]), sgm->entity_index);
    } else {
        for (const auto& tri : mesh.elements2D)
            bnd.emplace(make_key(tri->index[0], tri->index[1], tri->index[2]), tri->entity_index);
    }
    for (int c = 0; c < n; ++c)
        for (int f = 0; f < F; ++f) {
            const size_t cf = (size_t)c * F + f;
            if (P.nbr[cf] != 0) continue;
            const FaceKey key = dim == 2 ? make_key(vert(c, (f + 1) % nv), vert(c, (f + 2) % nv))
                                         : make_key(vert(c, (f + 1) % nv), vert(c, (f + 2) % nv), vert(c, (f + 3) % nv));
            auto it = bnd.find(key);
            if (it != bnd.end()) P.nbr[cf] = -it->second - 1;
        }
    return 0;
}

}  // namespace

int prepare(const BTEMesh& mesh, const BTEBand& bands, const BTEBoundaryCondition& bcs, int DM, int num_theta,
            int num_phi, double T_ref, Prepared& P, std::string& err) {
    P = Prepared();
    P.dim = mesh.dim;
    P.DM = DM;
    P.num_theta = num_theta;
    P.num_phi = num_phi;
    P.T_ref = T_ref;
    P.solid_angle = 4 * M_PI;
    if (DM != 2 && DM != 3) { err = "DM must be 2 or 3"; return BTE_ERR_INVALID_ARGUMENT; }
    if (num_theta <= 0 || num_phi <= 0) { err = "num_theta and num_phi must be positive"; return BTE_ERR_INVALID_ARGUMENT; }
    // setParam (src/StaticBTESolver.cpp:48-94)
    if (mesh.dim == 1) {
        P.T_ref = 0;  // the reference forces T_ref = 0 on 1D meshes
        P.n_cell = (int)mesh.elements1D.size();
        P.n_dir = DM == 3 ? num_theta * num_phi : num_theta;
        if (DM == 2) P.solid_angle = 2 * M_PI;
        P.n_face = 2;
    } else if (mesh.dim == 2) {
        P.n_cell = (int)mesh.elements2D.size();
        P.wfactor = DM == 3 ? 2.0 : 4 * M_PI;
        P.n_dir = DM == 3 ? 4 * num_theta * num_phi : 4 * num_phi;
        P.n_face = 3;
    } else if (mesh.dim == 3) {
        P.n_cell = (int)mesh.elements3D.size();
        P.wfactor = DM == 3 ? 1.0 : 2.0;
        P.n_dir = DM == 3 ? 8 * num_theta * num_phi : 4 * num_theta * num_phi;
        P.n_face = 4;
    } else {
        err = "mesh dimension must be 1, 2 or 3";
        return BTE_ERR_INVALID_ARGUMENT;
    }
    if (P.n_cell <= 0) { err = "mesh has no cells"; return BTE_ERR_INVALID_ARGUMENT; }
    if (mesh.dim == 3 && DM == 2) {
        // the reference has no DM=2 direction set for 3D meshes (:372-492 only builds DM=3 there)
        err = "DM=2 on a 3D mesh has no direction set";
        return BTE_ERR_INVALID_ARGUMENT;
    }
    double t0 = now_ms();
    int rc = quadrature(P, err);
    if (rc) return rc;
    double t1 = now_ms();
    rc = geometry(mesh, P, err);
    if (rc) return rc;
    P.ms_quadrature = t1 - t0;
    P.ms_geometry = now_ms() - t1;
    P.n_band = (int)bands.size();
    for (const auto& b : bands) {
        P.vg.push_back(b.group_velocity);
        P.tau.push_back(b.relaxation_time);
        P.C.push_back(b.Ctot);
        P.Lr.push_back(b.Lr);
    }
    if (P.n_band == 0) { err = "no bands"; return BTE_ERR_INVALID_ARGUMENT; }
    P.n_bc = (int)bcs.size();
    for (const auto& bc : bcs) {
        P.bc_index.push_back(bc.index);
        P.bc_type.push_back(bc.type);
        P.bc_T.push_back(bc.temperature);
    }
    return 0;
}

int upload(const Prepared& P, bte_ctx* ctx) {
    int rc = bte_set_geometry(ctx, P.dim, P.n_cell, P.n_face, P.nbr.data(), P.area.data(), P.normal.data(),
                              P.volume.data());
    if (rc) return rc;
    rc = bte_set_quadrature(ctx, P.n_dir, P.s.data(), P.S.data(), P.omega.data(), P.DM, P.num_theta, P.num_phi,
                            P.solid_angle, P.T_ref);
    if (rc) return rc;
    rc = bte_set_centroids(ctx, P.centroid.data());
    if (rc) return rc;
    rc = bte_set_bands(ctx, P.n_band, P.vg.data(), P.tau.data(), P.C.data(), P.Lr.data());
    if (rc) return rc;
    return bte_set_bcs(ctx, P.n_bc, P.bc_index.data(), P.bc_type.data(), P.bc_T.data());
}

bool write_tempcell(const std::string& path, int n, int dim, const double* centroid, const double* T, double L_x,
                    double L_y, double L_z) {
    std::ofstream out(path);
    if (!out) return false;
    for (int i = 0; i < n; ++i) {
        out << centroid[3 * i] / L_x << " ";
        if (dim >= 2) out << centroid[3 * i + 1] / L_y << " ";
        if (dim == 3) out << centroid[3 * i + 2] / L_z << " ";
        out << T[i] << "\n";
    }
    return static_cast<bool>(out);
}

}  // namespace sbte
