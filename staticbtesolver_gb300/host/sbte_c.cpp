// sbte_c.cpp -- C entry points of the host layer (include/sbte.h).
#include <cstring>
#include <fstream>
#include <string>

#include "../../include/sbte.h"
#include "prepare.h"

struct sbte_problem {
    sbte::Prepared P;
};

namespace {
thread_local std::string g_err;
}

extern "C" {

sbte_problem* sbte_open(const char* geo, const char* bc_file, const char* band_file, int DM, int num_theta,
                        int num_phi, double T_ref, double L_x, double L_y, double L_z) {
    g_err.clear();
    if (!geo || !bc_file || !band_file) { g_err = "null path"; return nullptr; }
    std::string g(geo);
    std::unique_ptr<BTEMesh> mesh;
    if (g.find('.') == std::string::npos) {
        int n = std::atoi(geo);
        if (n <= 0) { g_err = "1D cell count must be positive"; return nullptr; }
        mesh.reset(new BTEMesh(n, L_x));
    } else {
        std::ifstream f(g);
        if (!f.is_open()) { g_err = "cannot open mesh " + g; return nullptr; }
        mesh.reset(new BTEMesh(f, L_x, L_y, L_z));
    }
    std::ifstream bf(band_file), cf(bc_file);
    if (!bf.is_open()) { g_err = std::string("cannot open band file ") + band_file; return nullptr; }
    if (!cf.is_open()) { g_err = std::string("cannot open boundary file ") + bc_file; return nullptr; }
    BTEBand bands(bf);
    BTEBoundaryCondition bcs(cf);
    auto* p = new sbte_problem;
    if (sbte::prepare(*mesh, bands, bcs, DM, num_theta, num_phi, T_ref, p->P, g_err) != 0) {
        delete p;
        return nullptr;
    }
    return p;
}

const char* sbte_error(void) { return g_err.c_str(); }
void sbte_close(sbte_problem* p) { delete p; }

void sbte_counts(const sbte_problem* p, int* c) {
    c[0] = p->P.n_cell; c[1] = p->P.n_dir; c[2] = p->P.n_band; c[3] = p->P.n_face; c[4] = p->P.n_bc; c[5] = p->P.dim;
}

void sbte_quadrature(const sbte_problem* p, double* s, double* S, double* omega, double* sc) {
    const auto& P = p->P;
    std::memcpy(s, P.s.data(), sizeof(double) * P.s.size());
    std::memcpy(S, P.S.data(), sizeof(double) * P.S.size());
    std::memcpy(omega, P.omega.data(), sizeof(double) * P.omega.size());
    sc[0] = P.solid_angle; sc[1] = P.T_ref; sc[2] = P.wfactor; sc[3] = P.ms_quadrature; sc[4] = P.ms_geometry;
}

void sbte_geometry(const sbte_problem* p, double* volume, double* centroid, double* area, double* normal, int* nbr) {
    const auto& P = p->P;
    std::memcpy(volume, P.volume.data(), sizeof(double) * P.volume.size());
    std::memcpy(centroid, P.centroid.data(), sizeof(double) * P.centroid.size());
    std::memcpy(area, P.area.data(), sizeof(double) * P.area.size());
    std::memcpy(normal, P.normal.data(), sizeof(double) * P.normal.size());
    std::memcpy(nbr, P.nbr.data(), sizeof(int) * P.nbr.size());
}

void sbte_bands(const sbte_problem* p, double* vg, double* tau, double* C, double* Lr) {
    const auto& P = p->P;
    for (int b = 0; b < P.n_band; ++b) { vg[b] = P.vg[b]; tau[b] = P.tau[b]; C[b] = P.C[b]; Lr[b] = P.Lr[b]; }
}

void sbte_bcs(const sbte_problem* p, int* index, int* type, double* T) {
    const auto& P = p->P;
    for (int i = 0; i < P.n_bc; ++i) { index[i] = P.bc_index[i]; type[i] = P.bc_type[i]; T[i] = P.bc_T[i]; }
}

int sbte_upload(const sbte_problem* p, bte_ctx* ctx) { return sbte::upload(p->P, ctx); }

int sbte_write_tempcell(const char* path, int n, int dim, const double* centroid, const double* T, double L_x,
                        double L_y, double L_z) {
    if (!path || n < 0 || (n > 0 && (!centroid || !T))) {
        g_err = "sbte_write_tempcell: bad arguments";
        return BTE_ERR_INVALID_ARGUMENT;
    }
    if (!sbte::write_tempcell(path, n, dim, centroid, T, L_x, L_y, L_z)) {
        g_err = std::string("sbte_write_tempcell: cannot write ") + path;
        return BTE_ERR_INVALID_ARGUMENT;
    }
    return BTE_OK;
}

}  // extern "C"
