// oracle/bte_oracle.h -- TEST INFRASTRUCTURE ONLY (the oracle).
//
// A CPU restatement, in plain C++, of the reference's steady-state DOM-FVM
// phonon BTE solve (src/StaticBTESolver.cpp), used by tests/ as the checker for
// the CUDA path, by __graft_entry__.smoke(), and by bench.py's CPU-baseline
// leg.  The product never links or calls it.  Each function cites the
// reference file:line it follows.
//
// Pinning: the restatement is checked against the five golden logs shipped with
// the reference (tests/{2DM1DG,3DM1DG,2DM2DG,3DM2DG,3DM3DG}/*.sol, heat fluxes and
// margin trajectories) and against the reference's own CPU code compiled here
// from its sources (oracle/Makefile `ref`, oracle/ref_harness.cpp).
#pragma once
#ifdef __cplusplus
extern "C" {
#endif

// Inner solver used for each (band, direction) system.
enum oracle_inner {
    ORACLE_INNER_GMRES_ILU0 = 0,  // the reference CPU path (PETSc defaults), rtol 1e-9
    ORACLE_INNER_BICGSTAB = 1,    // the reference GPU path (src/bicgstab.hpp), tol 1e-9
};

typedef struct oracle_session oracle_session;

// geo: an .mphtxt path, or a decimal cell count for the uniform 1D mesh
// (src/BTEMain.cpp:118-141).  Returns NULL on a read error.
oracle_session* oracle_open(const char* geo, const char* bc_file, const char* band_file, int DM,
                            int num_theta, int num_phi, double T_ref, double L_x, double L_y,
                            double L_z);
void oracle_close(oracle_session* s);

// counts: n_cell, n_dir, n_band, n_face, n_bc, dim
void oracle_counts(const oracle_session* s, int* counts);

// Quadrature (src/StaticBTESolver.cpp:373-492): s[n_dir*3], S[n_dir*3], omega[n_dir];
// scalars: solid_angle, WFACTOR, T_ref (after setParam's 1D override).
void oracle_quadrature(const oracle_session* s, double* dirs, double* S, double* omega,
                       double* scalars);
// Geometry (src/StaticBTESolver.cpp:494-688): volume[n_cell], centroid[n_cell*3],
// area[n_cell*n_face], normal[n_cell*n_face*3], nbr[n_cell*n_face].
void oracle_geometry(const oracle_session* s, double* volume, double* centroid, double* area,
                     double* normal, int* nbr);

// Run the source iteration.  inner: enum oracle_inner; inner_tol: 1e-9 for the
// reference; outer_tol: the margin threshold (1e-5 in the current reference
// source, src/StaticBTESolver.cpp:798; the shipped .sol logs stop below 1e-4).
// threads: OpenMP threads over the independent (band, direction) systems of one
// outer iteration (the results do not depend on it).  max_systems > 0 stops
// after that many inner solves (timing samples; results then meaningless).
// Returns the number of outer iterations run.
int oracle_run(oracle_session* s, int max_iter, double outer_tol, int inner, double inner_tol,
               int threads, long long max_systems);

// One outer iteration from a given state (e_prev_in [n_band][n_dir][n_cell], the
// source temperature T_in [n_cell]): writes e_out (may be NULL) and T_out,
// returns the margin against e_prev_in.  The results getters below then
// describe this iteration.
double oracle_step(oracle_session* s, const double* e_prev_in, const double* T_in, int inner, double inner_tol,
                   int threads, double* e_out, double* T_out);

// Results after oracle_run.
void oracle_temperature(const oracle_session* s, double* T);          // [n_cell]
void oracle_band_temperature(const oracle_session* s, double* Tb);    // [n_cell*n_band]
void oracle_heat_flux(const oracle_session* s, double* q, double* q_band);  // [n_bc], [n_bc*n_band]
int oracle_margins(const oracle_session* s, double* m, int cap);
void oracle_energy(const oracle_session* s, double* e);  // e_curr [n_band][n_dir][n_cell]
// inner-solver statistics: solves, total iterations, unconverged, seconds in solves
void oracle_inner_stats(const oracle_session* s, long long* st, double* seconds);

// One (band, direction) system as the reference assembles it
// (_get_Ke :122-160, _get_Re :162-269), given the previous energy density
// e_prev[n_band][n_dir][n_cell] and the equilibrium density ebar[n_cell][n_band].
// rowptr[n_cell+1], col/val[n_face*n_cell+1], rhs[n_cell]. Returns nnz.
int oracle_assemble(const oracle_session* s, int band, int dir, const double* e_prev,
                    const double* ebar, int* rowptr, int* col, double* val, double* rhs);

// Stand-alone inner solvers on a CSR system (the reference's operator boundary:
// src/bicgstab.hpp:65,96,138 and src/StaticBTESolver.cpp:271).  Returns iterations.
int oracle_bicgstab_csr(int n, const int* rowptr, const int* col, const double* val,
                        const double* b, double* x, int maxit, double tol, int* converged);
int oracle_gmres_csr(int n, const int* rowptr, const int* col, const double* val,
                     const double* b, double* x, int maxit, double rtol, int* converged);

#ifdef __cplusplus
}
#endif
