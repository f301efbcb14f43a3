// prepare.h -- host preprocessing of the StaticBTESolver API: angular quadrature
// and mesh geometry in the flat layout the C ABI (bte_cuda.h) takes.
#pragma once
#include <string>
#include <vector>

#include "../../include/StaticBTESolver/BTEBand.h"
#include "../../include/StaticBTESolver/BTEBoundaryCondition.h"
#include "../../include/StaticBTESolver/BTEMesh.h"

struct bte_ctx;

namespace sbte {

struct Prepared {
    int dim = 0, n_cell = 0, n_face = 0, n_dir = 0, n_band = 0, n_bc = 0;
    int DM = 0, num_theta = 0, num_phi = 0;
    double T_ref = 0, solid_angle = 0, wfactor = 0;
    std::vector<double> s, S, omega;                    // [n_dir*3], [n_dir*3], [n_dir]
    std::vector<double> volume, centroid, area, normal; // [n], [n*3], [n*F], [n*F*3]
    std::vector<int> nbr;                               // [n*F]
    std::vector<double> vg, tau, C, Lr;                 // [n_band]
    std::vector<int> bc_index, bc_type;                 // [n_bc]
    std::vector<double> bc_T;
    double ms_quadrature = 0, ms_geometry = 0;
};

// Returns 0 on success, otherwise a bte_status value with err filled in.
int prepare(const BTEMesh& mesh, const BTEBand& bands, const BTEBoundaryCondition& bcs, int DM,
            int num_theta, int num_phi, double T_ref, Prepared& out, std::string& err);

// bte_set_geometry / bte_set_quadrature / bte_set_bands / bte_set_bcs.
int upload(const Prepared& p, bte_ctx* ctx);

// Cell temperatures in the format of the reference's (commented-out) field
// dump, src/StaticBTESolver.cpp:818-831: one line per cell, "x/L_x y/L_y T"
// (3D: "x/L_x y/L_y z/L_z T"), default stream formatting.  1D meshes write
// "x/L_x T" (the reference would divide y = 0 by L_y = 0).  False if the file
// cannot be written.
bool write_tempcell(const std::string& path, int n, int dim, const double* centroid, const double* T, double L_x,
                    double L_y, double L_z);

}  // namespace sbte
