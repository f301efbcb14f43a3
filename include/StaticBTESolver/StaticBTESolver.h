// StaticBTESolver.h -- the solver class of the StaticBTESolver API, running on
// one GB300 through the C ABI in bte_cuda.h.
//
// Constructor, setParam and solve keep the reference's signatures and meaning
// (includes/StaticBTESolver/StaticBTESolver.h:81,89,95): the caller owns mesh,
// bcs and bands; solve() preprocesses the mesh, runs the source iteration to
// margin <= 1e-5 or max_iter, and prints the same stdout lines as the
// reference (src/StaticBTESolver.cpp:691-696, :789-790, :873, :366).
// Everything below "Additions" is new API; the reference keeps its results
// private and only prints them.
#ifndef STATICBTESOLVER_GB300_STATICBTESOLVER_H
#define STATICBTESOLVER_GB300_STATICBTESOLVER_H

#include <memory>
#include <vector>

#include "BTEBand.h"
#include "BTEBoundaryCondition.h"
#include "BTEMesh.h"
#include <string>

#include "utility.h"

struct bte_ctx;
namespace sbte {
struct Prepared;
}

class StaticBTESolver {
public:
    StaticBTESolver(BTEMesh* mesh, BTEBoundaryCondition* bcs, BTEBand* bands);
    ~StaticBTESolver();
    StaticBTESolver(const StaticBTESolver&) = delete;
    StaticBTESolver& operator=(const StaticBTESolver&) = delete;

    void setParam(int DM, int num_theta, int num_phi, double T_ref);
    void solve(int max_iter);

    // ---- Additions
    void setForm(int form);                 // bte_form (0 plain FP64, 1 mixed, 2 sweep)
    // outer-iteration acceleration (bte_options.accel: 0 none, 1 learned, 2 Aitken,
    // 3 Anderson; every: interval or depth).  Learned needs setMlp first.
    void setAccel(int accel, int every);
    void setMlp(const std::vector<float>& params);  // bte_mlp_param_count() values
    // diffusion-synthetic correction after each outer iteration (bte_options.dsa;
    // tol/maxit of its low-order solve, 0 = defaults 1e-3 / 4000)
    void setDsa(bool on, double tol = 0, int maxit = 0);
    void setTolerance(double margin_tol);   // outer stop (reference: 1e-5)
    void setInnerTolerance(double tol);     // inner relative residual (reference: 1e-9)
    void setVerbose(bool verbose);          // print the reference's stdout lines (default true)
    int status() const { return status_; }  // bte_status of the last solve
    int iterations() const { return n_iter_; }
    const std::vector<double>& temperature() const { return cell_temperature_; }       // [N_cell]
    const std::vector<double>& bandTemperature() const { return cell_band_temperature_; }  // [N_cell][N_band]
    const std::vector<double>& heatFlux() const { return bc_heat_flux_; }              // [N_bc]
    const std::vector<double>& bandHeatFlux() const { return bc_band_heat_flux_; }     // [N_bc][N_band]
    const std::vector<double>& margins() const { return margins_; }
    double iterationMilliseconds() const { return ms_iteration_; }
    // The field dump the reference has commented out (src/StaticBTESolver.cpp:818-831):
    // "x/L_x y/L_y [z/L_z] T" per cell; false if nothing was solved or the file fails.
    bool writeTempcell(const std::string& path = "Tempcell.dat") const;

private:
    BTEMesh* mesh_;
    BTEBoundaryCondition* bcs_;
    BTEBand* bands_;
    int DM_ = 3, num_theta_ = 4, num_phi_ = 4;
    double T_ref_ = 300;
    int form_ = 0;
    int accel_ = 0, accel_every_ = 8;
    bool dsa_ = false;
    double dsa_tol_ = 0;
    int dsa_maxit_ = 0;
    std::vector<float> mlp_;
    double tol_ = 1e-5, inner_tol_ = 1e-9;
    bool verbose_ = true;
    int status_ = 0, n_iter_ = 0;
    double ms_iteration_ = 0;
    bte_ctx* ctx_ = nullptr;
    std::vector<double> cell_temperature_, cell_band_temperature_, bc_heat_flux_, bc_band_heat_flux_, margins_;
    std::vector<double> cell_centroid_;
    int dim_ = 0;
};

#endif
