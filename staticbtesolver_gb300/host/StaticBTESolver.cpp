// StaticBTESolver.cpp -- the reference's solver class over the GB300 C ABI.
#include "../../include/StaticBTESolver/StaticBTESolver.h"

#include <chrono>
#include <cstdio>
#include <iostream>

#include "../../include/bte_cuda.h"
#include "prepare.h"

namespace {
struct Printer {
    bool on;
};
void print_iteration(void* user, int iteration, double margin, double ms) {
    if (!static_cast<Printer*>(user)->on) return;
    // src/StaticBTESolver.cpp:789-792
    std::cout << "----------------------------------------------------------------------------------" << std::endl;
    std::cout << "Iteration #" << iteration << "\t Margin per band per cell: " << margin << std::endl;
    std::cout << "Time taken by inner loop: " << ms << " milliseconds" << std::endl;
}
}  // namespace

StaticBTESolver::StaticBTESolver(BTEMesh* mesh, BTEBoundaryCondition* bcs, BTEBand* bands)
    : mesh_(mesh), bcs_(bcs), bands_(bands) {}

StaticBTESolver::~StaticBTESolver() {
    if (ctx_) bte_destroy(ctx_);
}

void StaticBTESolver::setParam(int DM, int num_theta, int num_phi, double T_ref) {
    DM_ = DM;
    num_theta_ = num_theta;
    num_phi_ = num_phi;
    T_ref_ = T_ref;
}

void StaticBTESolver::setForm(int form) { form_ = form; }
void StaticBTESolver::setAccel(int accel, int every) {
    accel_ = accel;
    accel_every_ = every;
}
void StaticBTESolver::setMlp(const std::vector<float>& params) { mlp_ = params; }
void StaticBTESolver::setDsa(bool on, double tol, int maxit) {
    dsa_ = on;
    dsa_tol_ = tol;
    dsa_maxit_ = maxit;
}
void StaticBTESolver::setTolerance(double tol) { tol_ = tol; }
void StaticBTESolver::setInnerTolerance(double tol) { inner_tol_ = tol; }
void StaticBTESolver::setVerbose(bool v) { verbose_ = v; }

void StaticBTESolver::solve(int max_iter) {
    sbte::Prepared P;
    std::string err;
    status_ = sbte::prepare(*mesh_, *bands_, *bcs_, DM_, num_theta_, num_phi_, T_ref_, P, err);
    if (status_ != 0) {
        std::cerr << "StaticBTESolver: " << err << std::endl;
        return;
    }
    if (verbose_) {  // src/StaticBTESolver.cpp:691-696
        std::cout << "N_cell: " << P.n_cell << std::endl
                  << "N_dir: " << P.n_dir << std::endl
                  << "N_band: " << P.n_band << std::endl
                  << "num_theta: " << num_theta_ << std::endl
                  << "num_phi: " << num_phi_ << std::endl
                  << std::endl;
    }
    if (!ctx_) {
        status_ = bte_create(&ctx_, 0);
        if (status_ != BTE_OK) {
            std::cerr << "StaticBTESolver: " << bte_last_error(nullptr) << std::endl;
            ctx_ = nullptr;
            return;
        }
    }
    status_ = sbte::upload(P, ctx_);
    if (status_ != BTE_OK) {
        std::cerr << "StaticBTESolver: " << bte_last_error(ctx_) << std::endl;
        return;
    }
    bte_options o;
    bte_default_options(&o);
    o.max_iter = max_iter;
    o.tol = tol_;
    o.form = form_;
    o.accel = accel_;
    o.accel_every = accel_every_;
    o.dsa = dsa_ ? 1 : 0;
    o.dsa_tol = dsa_tol_;
    o.dsa_maxit = dsa_maxit_;
    if (accel_ == 1 || accel_ == 2) {  // the per-cell extrapolations use the centroids
        status_ = bte_set_centroids(ctx_, P.centroid.data());
        if (status_ == BTE_OK && accel_ == 1) {
            if ((int)mlp_.size() != bte_mlp_param_count()) {
                std::cerr << "StaticBTESolver: the learned accelerator needs setMlp with " << bte_mlp_param_count()
                          << " values" << std::endl;
                status_ = BTE_ERR_STATE;
                return;
            }
            status_ = bte_set_mlp(ctx_, mlp_.data());
        }
        if (status_ != BTE_OK) {
            std::cerr << "StaticBTESolver: " << bte_last_error(ctx_) << std::endl;
            return;
        }
    }
    o.inner_tol = inner_tol_;
    Printer pr{verbose_};
    o.on_iteration = print_iteration;
    o.user = &pr;
    bte_report rep;
    auto t0 = std::chrono::steady_clock::now();
    status_ = bte_solve(ctx_, &o, &rep);
    ms_iteration_ = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (status_ != BTE_OK && status_ != BTE_ERR_NOT_CONVERGED) {
        std::cerr << "StaticBTESolver: " << bte_status_string((bte_status)status_) << ": " << bte_last_error(ctx_)
                  << std::endl;
        return;
    }
    n_iter_ = rep.n_iter;
    if (verbose_) {
        if (rep.converged) std::cout << std::endl;  // :800
        std::cout << "Time taken by iteration: " << ms_iteration_ << " milliseconds" << std::endl;  // :873
    }
    cell_temperature_.assign(P.n_cell, 0.0);
    cell_band_temperature_.assign((size_t)P.n_cell * P.n_band, 0.0);
    bc_heat_flux_.assign(P.n_bc, 0.0);
    bc_band_heat_flux_.assign((size_t)P.n_bc * P.n_band, 0.0);
    bte_get_temperature(ctx_, cell_temperature_.data());
    bte_get_band_temperature(ctx_, cell_band_temperature_.data());
    if (P.n_bc > 0) bte_get_heat_flux(ctx_, bc_heat_flux_.data(), bc_band_heat_flux_.data());
    cell_centroid_ = P.centroid;
    dim_ = mesh_->dim;
    margins_.assign(rep.n_iter, 0.0);
    int nm = 0;
    bte_get_margins(ctx_, margins_.data(), (int)margins_.size(), &nm);
    if (verbose_)
        for (int i = 0; i < P.n_bc; ++i)  // :365-368
            std::cout << "heat flux of Boundary Condition #" << -1 - P.bc_index[i] << ": " << bc_heat_flux_[i]
                      << std::endl;
}

bool StaticBTESolver::writeTempcell(const std::string& path) const {
    const int n = (int)cell_temperature_.size();
    if (n == 0 || (int)cell_centroid_.size() != 3 * n) return false;
    return sbte::write_tempcell(path, n, dim_, cell_centroid_.data(), cell_temperature_.data(), mesh_->L_x, mesh_->L_y,
                                mesh_->L_z);
}
