// oracle/ref_harness.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Runs the reference's own CPU solver (compiled from the reference sources by
// oracle/Makefile against the single-rank MPI and PETSc shims) and hands its
// results back through a C ABI.  The reference keeps its results private
// (includes/StaticBTESolver/StaticBTESolver.h:44-51) and only prints them, so
// this translation unit -- and only this one -- widens access to read
// cell_temperature, bc_heat_flux and bc_band_heat_flux after solve().  The
// class uses default (private) access, so the standard headers it needs are
// included first and the class key is switched to `struct` for its header only.  The
// per-iteration margins are parsed from the solver's stdout
// (src/StaticBTESolver.cpp:790).
#include <sstream>
#include <string>
#include <iostream>
#include <fstream>
#include <cstring>
#include <vector>
#include <memory>
#include <cassert>
#include <climits>
#include <cmath>
#include <iomanip>
#include <algorithm>
#define class struct
#include "StaticBTESolver.h"
#undef class

extern "C" void petsc_shim_stats(long long*, long long*, long long*);
extern "C" void petsc_shim_reset_stats();

extern "C" int ref_solve(const char* geo, const char* bc_file, const char* band_file, int DM,
                         int num_theta, int num_phi, double T_ref, int max_iter, double L_x,
                         double L_y, double L_z, double* T_out, int T_cap, double* q_out,
                         int q_cap, double* q_band_out, int q_band_cap, double* margins,
                         int margins_cap, int* counts /* n_cell, n_iter, n_bc, n_band, n_dir */,
                         long long* inner /* solves, iterations, unconverged */) {
    std::string g(geo);
    BTEMesh* mesh;
    if (g.find('.') == std::string::npos) {
        mesh = new BTEMesh(std::stoi(g), L_x);
    } else {
        std::ifstream f(g);
        if (!f.is_open()) return 1;
        mesh = new BTEMesh(f, L_x, L_y, L_z);
    }
    std::ifstream bf(band_file);
    if (!bf.is_open()) return 2;
    auto* bands = new BTEBand(bf);
    std::ifstream cf(bc_file);
    if (!cf.is_open()) return 3;
    auto* bcs = new BTEBoundaryCondition(cf);

    petsc_shim_reset_stats();
    std::ostringstream captured;
    std::streambuf* old = std::cout.rdbuf(captured.rdbuf());
    {
        StaticBTESolver solver(mesh, bcs, bands);
        solver.setParam(DM, num_theta, num_phi, T_ref);
        solver.solve(max_iter);
        std::cout.rdbuf(old);
        int n_cell = solver.N_cell;
        for (int i = 0; i < n_cell && i < T_cap; ++i) T_out[i] = solver.cell_temperature[i];
        int n_bc = (int)solver.bc_heat_flux.size();
        for (int i = 0; i < n_bc && i < q_cap; ++i) q_out[i] = solver.bc_heat_flux[i];
        int k = 0;
        for (int i = 0; i < n_bc; ++i)
            for (int b = 0; b < solver.N_band; ++b, ++k)
                if (k < q_band_cap) q_band_out[k] = solver.bc_band_heat_flux[i][b];
        counts[0] = n_cell;
        counts[2] = n_bc;
        counts[3] = solver.N_band;
        counts[4] = solver.N_dir;
    }
    std::istringstream in(captured.str());
    std::string line;
    int n_iter = 0;
    const std::string key = "Margin per band per cell: ";
    while (std::getline(in, line)) {
        auto p = line.find(key);
        if (p == std::string::npos) continue;
        if (n_iter < margins_cap) margins[n_iter] = std::stod(line.substr(p + key.size()));
        ++n_iter;
    }
    counts[1] = n_iter;
    petsc_shim_stats(&inner[0], &inner[1], &inner[2]);
    delete mesh;
    delete bands;
    delete bcs;
    return 0;
}
