/*
 * bte_cuda.h -- C ABI of the GB300 (sm_103a) phonon BTE solve.
 *
 * This is the drop-in boundary for the hot path of yuchengs/StaticBTESolver:
 * the steady-state discrete-ordinates finite-volume source iteration
 * (StaticBTESolver::_iteration, src/StaticBTESolver.cpp:690-808) with its upwind
 * assembly (_get_Ke :122-160, _get_Re :162-269), its per-(band, direction)
 * inner solve (CPU: _solve_matrix :271-308; GPU: BICGSTAB in
 * src/bicgstab.hpp:33-321), the reductions that close each outer iteration
 * (_get_cell_temperature :96-104, _recover_temperature :106-120,
 * _get_margin :311-321) and the heat flux (_get_heat_flux :323-370).
 *
 * Plain pointers and sizes only.  Every call returns a bte_status; nothing
 * exits the process.  A context owns one CUDA stream and all device memory it
 * allocates; it is not thread-safe (one host thread per context at a time).
 * Host input arrays are copied during the call and may be freed afterwards.
 */
#ifndef BTE_CUDA_H
#define BTE_CUDA_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum bte_status {
    BTE_OK = 0,
    BTE_ERR_INVALID_ARGUMENT = 1, /* bad size, index or pointer */
    BTE_ERR_STATE = 2,            /* call out of order (e.g. solve before set_geometry) */
    BTE_ERR_CUDA = 3,             /* a CUDA runtime call failed; see bte_last_error */
    BTE_ERR_OUT_OF_MEMORY = 4,
    BTE_ERR_UNSUPPORTED_BC = 5,   /* boundary type the reference aborts on (:218, :244, :254) */
    BTE_ERR_NOT_CONVERGED = 6,    /* outer iteration hit max_iter (results are still valid) */
    BTE_ERR_NUMERICAL = 7,        /* NaN/Inf in the outer iterate or in band data */
    BTE_ERR_NO_DEVICE = 8
} bte_status;

/* How each (band, direction) system is solved inside one outer iteration. */
typedef enum bte_form {
    /* FP64 right-Jacobi BiCGSTAB, x0 = 0, ||r||/||r0|| < inner_tol, at most
     * inner_maxit iterations (then the last iterate), breakdown restart with
     * r_hat = 6.8 b + 0.6: the reference GPU inner solve
     * (src/bicgstab.hpp:138-300), all systems of an outer iteration batched
     * into one launch per BiCGSTAB phase (see bte_options.plain_cycles). */
    BTE_FORM_PLAIN = 0,
    /* FP32 BiCGSTAB inside FP64 iterative refinement: x starts from the
     * previous outer iterate; each cycle computes the FP64 residual b - A x,
     * retires the systems with ||b - A x|| <= inner_tol * ||b|| (the
     * reference's criterion for x0 = 0), solves A dx = r for the others with
     * right-Jacobi BiCGSTAB in FP32 (relative tolerance 1e-4, on geometry
     * scaled per direction by 1 / mean(V Omega_d)) and adds dx in FP64; at
     * most 30 cycles. */
    BTE_FORM_MIXED = 1,
    /* FP64 upwind sweep: each system is lower triangular in the topological
     * order of its direction's upwind graph, so one level-scheduled forward
     * substitution solves it exactly (to rounding).  Edges closing a cycle of
     * the upwind graph are lagged and Gauss-Seidel sweeps repeat until
     * ||b - A x|| <= inner_tol ||b|| (at most inner_maxit sweeps).  The level
     * order is built once per geometry and quadrature. */
    BTE_FORM_SWEEP = 2
} bte_form;

typedef struct bte_ctx bte_ctx;

/* Per-outer-iteration callback: iteration index, margin, milliseconds spent. */
typedef void (*bte_iteration_cb)(void* user, int iteration, double margin, double ms);

typedef struct bte_options {
    int max_iter;         /* outer iterations (StaticBTESolver::solve(max_iter)) */
    double tol;           /* stop when margin <= tol (reference: 1e-5, :798) */
    int form;             /* bte_form */
    double inner_tol;     /* 1e-9 in the reference (:699) */
    int inner_maxit;      /* 1000 in the reference (:699) */
    int batch_systems;    /* systems per batch; 0 = as many as fit in device memory */
    bte_iteration_cb on_iteration; /* may be NULL */
    void* user;
    int profile;          /* nonzero: time every inner-solve kernel with CUDA events
                             (bte_get_kernel_stats); adds event records between launches */
    int accel;            /* outer-iteration acceleration: 0 none (the reference), 1 learned
                             (the MLP set by bte_set_mlp), 2 Aitken per cell (non-learned),
                             3 Anderson mixing of T and the boundary-cell intensities
                             (non-learned) */
    int accel_every;      /* 1, 2: outer iterations between extrapolations (>= 4);
                             3: Anderson depth (1..8) */
    int keep_history;     /* nonzero: keep T after every outer iteration (bte_get_history) */
    int dsa;              /* nonzero: diffusion-synthetic acceleration of the outer iteration (below);
                             with BTE_FORM_MIXED the inner solves then run to min(inner_tol, 1e-11) */
    double dsa_tol;       /* relative residual of its low-order solve (0: 1e-3) */
    int dsa_maxit;        /* iteration limit of its low-order solve (0: 4000) */
    int plain_cycles;     /* BTE_FORM_PLAIN: 0 or 1 = the reference's semantics (a system stops at
                             inner_maxit and keeps its last iterate); k > 1 = an unconverged system
                             goes on to k x inner_maxit iterations and keeps the iterate with the
                             smallest residual seen after inner_maxit / 2 */
} bte_options;

/* Per-kernel totals of the last profiled bte_solve. */
typedef struct bte_kernel_stat {
    char name[32];
    long long launches;
    double ms;          /* summed CUDA-event durations on the solve stream */
    double bytes;       /* algorithmic HBM bytes of the work done by those launches */
} bte_kernel_stat;

typedef struct bte_report {
    int n_iter;                /* outer iterations run */
    int converged;             /* margin <= tol reached */
    double final_margin;
    long long inner_solves;    /* (band, direction) systems solved */
    long long inner_iterations;/* BiCGSTAB iterations summed over systems */
    long long inner_unconverged;
    long long refinements;     /* FP64 refinement cycles (mixed form) */
    double ms_total;           /* device time of the outer loop (accelerator included) */
    double ms_rhs;             /* right-hand-side assembly */
    double ms_inner;           /* inner solves (sweep form from its second iteration on: the
                                  whole iteration, replayed as a CUDA graph) */
    double ms_reduce;          /* temperature / margin reductions and the accelerator */
    long long kernel_launches; /* kernels this library launched during the solve */
    int sweep_group;           /* sweep form: bands per block and threads per block */
    int sweep_threads;         /* chosen by timing candidate shapes on a plan's first sweep */
    int accel_steps;           /* outer-iteration extrapolations (accel 1, 2) or mixes (3) applied */
    int accel_reverts;         /* extrapolations undone (state restored) */
    int sweep_ring;            /* sweep form: solved positions kept in shared memory per band */
    int sweep_margin;          /* sweep form, acyclic plan: 1 the sweep sums the margin, 0 the reduction
                                  does (timed against each other with the launch shape) */
    int dsa_solves;            /* low-order corrections applied (dsa) */
    long long dsa_iterations;  /* conjugate-gradient iterations summed over them */
    double ms_dsa;             /* device time of the corrections (included in ms_reduce and ms_total) */
    int sweep_kernel;          /* sweep form: the kernel the autotuner chose -- 0 level-synchronous (k_sweep),
                                  1 staged (levels copied to shared memory ahead by bulk copies, right-hand
                                  side from a level-ordered pre-pass), 2 level-synchronous over levels
                                  split into slices of one position per thread */
    double ms_host_setup;      /* host wall time of this call's set-up after new inputs (uploads, geometry) */
    double ms_host_plan;       /* ... of building the sweep plan (level order, layout) after new geometry */
    double ms_host_order;      /*     of which the level order (host threads over directions) */
    double ms_host_dsa;        /* ... of building the low-order operator of dsa after new inputs (its host
                                  part runs on a host thread next to the sweep plan's, so the two overlap) */
    double ms_wall;            /* host wall time of the whole call (set-up, solve, read-backs) */
    int sweep_host_dirs;       /* sweep form: directions of the current plan whose level order was built on the
                                  host (a cycle in the upwind graph, or a wave wider than the device's frontier
                                  buffers); the others on the device */
} bte_report;

/* Fill opts with the reference's defaults (max_iter 10000 as BTEcmd's -I default,
 * tol 1e-5, FP64 plain form, inner_tol 1e-9, inner_maxit 1000). */
void bte_default_options(bte_options* opts);
const char* bte_status_string(bte_status s);
/* Last error message recorded on ctx (or the thread's last create error if ctx is NULL). */
const char* bte_last_error(const bte_ctx* ctx);

/* Replaces the device binding in StaticBTESolver::StaticBTESolver
 * (src/StaticBTESolver.cpp:35-38): device = rank % device_count there. */
bte_status bte_create(bte_ctx** ctx, int device);
bte_status bte_destroy(bte_ctx* ctx);

/* Mesh geometry after StaticBTESolver::_preprocess (src/StaticBTESolver.cpp:494-688).
 * dim 1/2/3; n_face 2/3/4.  nbr[c*n_face+f] >= 0 is the neighbouring cell,
 * < 0 encodes boundary entity e as -e-1 (the reference's convention).
 * area[c*n_face+f]; normal[(c*n_face+f)*3 + xyz] (outward unit normal);
 * volume[c]. */
bte_status bte_set_geometry(bte_ctx* ctx, int dim, int n_cell, int n_face, const int* nbr,
                            const double* area, const double* normal, const double* volume);

/* Angular quadrature (src/StaticBTESolver.cpp:48-94 and :373-492).
 * s[d*3+xyz] unit directions, S[d*3+xyz] angle-integrated directions (unused in
 * 1D), omega[d] control angles.  DM, num_theta, num_phi as given to setParam;
 * solid_angle is 4 pi (2 pi for DM=2 on a 1D mesh); T_ref after setParam's
 * 1D override (0 for 1D meshes). */
bte_status bte_set_quadrature(bte_ctx* ctx, int n_dir, const double* s, const double* S,
                              const double* omega, int DM, int num_theta, int num_phi,
                              double solid_angle, double T_ref);

/* Bands (src/BTEBand.cpp:8-26): group velocity, relaxation time, Ctot, Lr.
 * A NaN or infinite value returns BTE_ERR_NUMERICAL (the reference would carry
 * it into every outer iterate). */
bte_status bte_set_bands(bte_ctx* ctx, int n_band, const double* vg, const double* tau,
                         const double* C, const double* Lr);

/* Boundary conditions (src/BTEBoundaryCondition.cpp:7-23): index = -entity-1,
 * type 1 isothermal, 2 diffuse, 31/32/33 specular; T in kelvin. */
bte_status bte_set_bcs(bte_ctx* ctx, int n_bc, const int* index, const int* type, const double* T);

/* Run the source iteration (src/StaticBTESolver.cpp:690-808) from e = 0.
 * report may be NULL.  Returns BTE_ERR_NOT_CONVERGED when max_iter ran out
 * (the fields are still those of the last iteration, as in the reference). */
bte_status bte_solve(bte_ctx* ctx, const bte_options* opts, bte_report* report);

/* Results of the last bte_solve, copied to host arrays. */
bte_status bte_get_temperature(bte_ctx* ctx, double* T /* [n_cell] */);
bte_status bte_get_band_temperature(bte_ctx* ctx, double* Tb /* [n_cell*n_band] */);
/* q_bc[n_bc] (the printed "heat flux of Boundary Condition #k"); q_bc_band
 * [n_bc*n_band] may be NULL. */
bte_status bte_get_heat_flux(bte_ctx* ctx, double* q_bc, double* q_bc_band);
/* Energy density e[b][d][c] (the reference's ee_curr), n_band*n_dir*n_cell values. */
bte_status bte_get_energy(bte_ctx* ctx, double* e);
/* Margins of the outer iterations run, up to cap values; returns how many via *n. */
bte_status bte_get_margins(bte_ctx* ctx, double* margins, int cap, int* n);

/* Learned outer-iteration acceleration (no counterpart in the reference; the
 * plain source iteration still runs to the same margin, so the accelerator
 * changes how fast the fixed point is reached, not which one).  Every
 * accel_every outer iterations each cell's temperature is reset to an
 * extrapolation from its last four values and the equilibrium energy density
 * follows.  With d_i = T_{k-i+1} - T_{k-i}, s = |d1| + |d2| + |d3| and the
 * Aitken estimate A = d1 r / (1 - r) / s (r = d1 / d2, used when 0 < r < 1,
 * else 0, clipped to +-64): accel = 2 jumps by s A; accel = 1 jumps by
 * s clip(A + clip(y, +-8), +-64), where y is a per-cell MLP's learned correction
 * (8 -> 128 -> 128 -> 128 -> 1, BF16 weights, FP32 accumulation on the tensor
 * cores).  MLP inputs: d1/s, d2/s, d3/s, A/64, x and y of the centroid scaled
 * to [0, 1] over the mesh, log(V / mean V), log10(Kn) with Kn =
 * (sum_b Lr_b v_b tau_b / sum_b Lr_b) / V^(1/dim).  The state before each
 * jump is kept; if the margin accel_every-1 iterations after a jump is not
 * below the margin at the jump, the state is restored and extrapolation stops
 * for the rest of the solve, so a bad jump costs accel_every-1 iterations and
 * no more.  Parameters: FP32,
 * bte_mlp_param_count() values, W1[8][128] b1 W2[128][128] b2 W3[128][128] b3
 * W4[128][1] b4. */
/* accel = 3 (Anderson mixing, no counterpart in the reference): the outer
 * iteration is a fixed-point map x -> G(x) on its state x = (T, the
 * intensities at the cells with boundary faces, scaled by Omega_tot / C_b),
 * which is all the next sweep reads besides constants.  With the last
 * accel_every + 1 pairs (g_i = G(x_i), f_i = g_i - x_i) the next iteration
 * starts from sum_i alpha_i g_i, alpha minimising ||sum_i alpha_i f_i||_2
 * subject to sum_i alpha_i = 1 (Gram matrix on the GPU in a fixed order, the
 * small system on the host); the history restarts when the margin grows
 * tenfold or a weight exceeds 1e3.  The plain iteration's margin still
 * decides convergence. */
/* dsa != 0 (diffusion-synthetic acceleration, no counterpart in the reference;
 * any form, combinable with accel): after each outer iteration that has not
 * met the tolerance, the change r = T_new - T_old of the equilibrium
 * temperature drives one low-order diffusion solve on the same cells,
 *   sum_f W_f (x_c - x_nb) + sum_{isothermal wall faces} W_f x_c = V_c r_c,
 *   W_f = (A_f / Omega_tot) sum_b Lr_b L_b (G_f + L_b q_f / (4 delta_f)) / sum_b Lr_b,
 * L_b = v_b tau_b, G_f = 1/2 sum_d |g_df| (the upwind scheme's own numerical
 * diffusion, g = S.n), q_f = sum_d g_df (s_d.n_f), delta_f the centroid
 * distance across the face; diffuse and specular walls are adiabatic.  The
 * next iteration's source is T_new + x (the boundary cells' intensities,
 * which the walls reflect, shift by C_b / Omega_tot x).  In the diffusive
 * regime, where the source iteration's error shrinks by ~1e-6 per outer
 * iteration, this shrinks it by ~5-10x per iteration.  The low-order solve is
 * conjugate gradients (FP32 vectors, FP64 dot products) in one cooperative
 * kernel; it needs at least one isothermal wall (otherwise dsa is ignored).
 * Convergence is still the reference's margin between consecutive transport
 * iterates, and the returned fields are the last transport iterate's. */
int bte_mlp_param_count(void);
bte_status bte_set_mlp(bte_ctx* ctx, const float* params);
/* Cell centroids [n_cell][3] (used only for the accelerator's features). */
bte_status bte_set_centroids(bte_ctx* ctx, const double* centroid);
/* T after every outer iteration of the last solve run with keep_history, row-major
 * [iteration][n_cell], up to cap_iters rows; *n_iters = rows available. */
bte_status bte_get_history(bte_ctx* ctx, double* T, int cap_iters, int* n_iters);
/* MLP on the current device, host buffers: X [M][8] FP32 features. */
bte_status bte_mlp_predict(const float* X, int M, const float* params, float* y);
/* Full-batch loss 0.5 mean (y - Y)^2 and its gradient w.r.t. the parameters. */
bte_status bte_mlp_gradient(const float* X, const float* Y, int M, const float* params, float* grad,
                            double* loss);
/* Adam training on the GPU: steps minibatches of batch rows drawn with seed;
 * params in/out (FP32); loss_hist[steps] (may be NULL). */
bte_status bte_mlp_train(const float* X, const float* Y, int M, int steps, int batch, float lr,
                         unsigned seed, float* params, float* loss_hist);

/* Kernel statistics of the last solve run with opts->profile set; *n = entries. */
bte_status bte_get_kernel_stats(bte_ctx* ctx, bte_kernel_stat* stats, int cap, int* n);

/* The sweep autotuner's table from the first sweep of the current plan (empty
 * when the choice came from the per-process cache): candidate k ran with
 * group[k] bands and threads[k] threads per block and ring[k] positions per
 * band, with kernel[k] (0 level-synchronous, 1 staged, 2 split levels, as
 * bte_report.sweep_kernel), in ms[k] milliseconds.  Entries are written up
 * to cap (arrays may be NULL when cap is 0); *n = candidates timed.  The
 * environment variable BTE_SWEEP_KERNEL=level|staged|split restricts the
 * candidates to one kernel (the temperatures are the same to the bit either
 * way). */
bte_status bte_get_sweep_tuning(bte_ctx* ctx, int* group, int* threads, int* ring, int* kernel, float* ms, int cap,
                                int* n);

/* Diagnostics: the current sweep plan's level order of direction d (no
 * counterpart in the reference): perm[k] = the cell at position k (n_cell
 * entries); lvl = the level starts, then n_cell (*nlev + 1 entries, written up
 * to cap_lvl).  Built on the device (one block per direction, Kahn's waves,
 * each wave in cell-index order); BTE_LEVEL_ORDER=host builds it on the host
 * instead (the same order).  BTE_ERR_STATE before a sweep-form solve. */
bte_status bte_get_level_order(bte_ctx* ctx, int d, int* perm, int* lvl, int cap_lvl, int* nlev);

/* The reference's inner-solve operator boundary (src/bicgstab.hpp:65,96,138):
 * BICGSTAB(n, maxit, tol); init(rowptr, colind, val, nnz, b); solve(x) --
 * right-Jacobi BiCGSTAB on one CSR system held in host memory.
 * iterations and converged may be NULL. */
bte_status bte_bicgstab_csr(int n, const int* rowptr, const int* colind, const double* val,
                            int nnz, const double* b, double* x, int maxit, double tol,
                            int* iterations, int* converged);

/* The low-order solve of dsa on host buffers: n cells with n_face face slots,
 * nb[f*n+c] the cell coupled to c through slot f (-1: none, or a wall held at
 * x = 0 when W[f*n+c] > 0), W[f*n+c] >= 0 the coupling (the operator must be
 * symmetric: W of (c, f) equals W of the slot of nb that names c).  Solves
 * sum_f W[f][c] (x_c - x_nb) = b_c (x_nb = 0 for walls) to a relative
 * residual tol of the Jacobi-scaled system within maxit iterations, on the
 * current device.  iterations and relres may be NULL. */
bte_status bte_dsa_solve(int n, int n_face, const int* nb, const double* W, const double* b, double* x,
                         double tol, int maxit, int* iterations, double* relres);

/* Allocation-free variant of bte_bicgstab_csr.  No counterpart in the
 * reference: it exists for callers that cannot allocate device memory -- code
 * whose device memory belongs to another allocator with a fixed budget, or
 * that must not trigger the device-wide synchronisation of cudaMalloc/cudaFree
 * in the middle of its stream work.  rowptr, colind, val, b and x are DEVICE
 * pointers owned by the caller; stream is a cudaStream_t (NULL: the legacy
 * default stream).  All scratch (work vectors, scalars, partial sums) lives in
 * one static device array of about 21 MB that every GPU loading this library
 * keeps until exit; it calls no cudaMalloc, cudaFree or allocating library
 * routine.  Limits: n <= 262144 unknowns, maxit <= 10000; larger values and a
 * malformed CSR return BTE_ERR_INVALID_ARGUMENT (message in bte_last_error(NULL)).
 * Every call looks up the array's device address in the current device's
 * context (so a context recreated after cudaDeviceReset is followed); the
 * first call on a device also loads the library's device code there and should
 * come before any stream capture.  Calls share the array: calls that overlap
 * on the GPU race.  The call returns after the solve has finished, and after
 * any of its kernels still queued when it fails. */
bte_status bte_bicgstab_csr_noalloc(int n, const int* rowptr, const int* colind, const double* val,
                                    int nnz, const double* b, double* x, int maxit, double tol,
                                    void* stream, int* iterations, int* converged);

#ifdef __cplusplus
}
#endif
#endif /* BTE_CUDA_H */
