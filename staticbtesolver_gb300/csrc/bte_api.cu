// bte_api.cu -- C ABI (include/bte_cuda.h) of the GB300 phonon BTE solve.
//
// One context = one device, one stream, resident inputs and state.  bte_solve
// runs the reference's source iteration (src/StaticBTESolver.cpp:690-808) with
// every (band, direction) system of a batch solved together by the batched
// BiCGSTAB kernels in bte_kernels.cuh, then the fused reductions and the heat
// flux of bte_transport.cuh.  Nothing here synchronises with the host inside a
// BiCGSTAB group; the host reads one counter per group and one margin per
// outer iteration.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <tuple>
#include <string>
#include <thread>
#include <vector>

#include "../../include/bte_cuda.h"
#include "bte_kernels.cuh"
#include "bte_transport.cuh"
#include "bte_mlp.cuh"
#include "bte_dsa.cuh"
#include "dsa_setup.h"
#include "sweep_order.h"
#include <random>

namespace {

thread_local std::string g_create_error;

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    cudaError_t alloc(size_t n) {
        if (n <= bytes && p) return cudaSuccess;
        release();
        if (n == 0) n = 16;
        cudaError_t e = cudaMalloc(&p, n);
        if (e == cudaSuccess) bytes = n;
        else p = nullptr;
        return e;
    }
    template <typename T>
    T* as() const { return static_cast<T*>(p); }
};

constexpr int kGroup = 8;  // BiCGSTAB iterations launched between host checks

enum KernelKind { KK_P, KK_SPMV1, KK_S, KK_SPMV2, KK_X, KK_INIT, KK_RHS, KK_REDUCE, KK_DIFFUSE, KK_HEAT, KK_SWEEP,
                  KK_SWEEP_RES, KK_DSA, KK_BICG, kNumKinds };
const char* kKindNames[kNumKinds] = {"bicg_p_update", "bicg_spmv1",   "bicg_s_update", "bicg_spmv2",
                                     "bicg_x_update", "bicg_init",    "rhs_assembly",  "reduce_margin",
                                     "diffuse_wall",  "heat_flux",    "upwind_sweep",  "sweep_residual",
                                     "dsa_correction", "bicg_persistent"};

}  // namespace

// Launch shape of the upwind sweep: bands per block, threads per block, ring
// positions per band, dynamic shared memory.
struct SweepShape {
    int G = 2, threads = 128, W = 2048;
    size_t smem = 0;
    bool margin = false;  // acyclic plans: the sweep sums the margin partials (else k_reduce does)
    bool staged = false;  // k_sweep_staged (levels staged by bulk copies, right-hand side formed a stage ahead)
    bool split = false;   // k_sweep over the levels split into slices of cap positions (one per thread)
    int cap = 0;          // staged, split: positions per stage
    int kind() const { return staged ? 1 : split ? 2 : 0; }
};

// Stage bounds of the staged sweep for one stage width: per direction, its
// levels split into slices of at most cap positions.
struct StageList {
    DevBuf stages, off;
};

struct bte_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t setup_stream = nullptr;  // the low-order operator's set-up, next to the sweep plan's
    std::mutex err_mutex;                 // err is written from the set-up thread too
    std::string err;
    // inputs (host copies)
    int dim = 0, n = 0, F = 0;
    std::vector<int> nbr;
    std::vector<double> area, normal, volume;
    int n_dir = 0, DM = 0, num_theta = 0, num_phi = 0;
    std::vector<double> s, S, omega;
    double solid_angle = 0, T_ref = 0;
    int n_band = 0;
    std::vector<double> vg, tau, Cb, Lr;
    int n_bc = 0;
    std::vector<int> bc_index, bc_type;
    std::vector<double> bc_T;
    bool has_geom = false, has_quad = false, has_bands = false, has_bcs = false;
    bool dirty = true;
    // derived sizes
    size_t Np = 0;
    int nchunk = 0;
    int nbf = 0, ndiff = 0;
    std::vector<int> h_bf_bc;
    // device state
    DevBuf d_normal, d_area, d_nbr, d_volume, d_s, d_S, d_omega;
    DevBuf d_dg, d_vo, d_fc, d_nb, d_kb, d_Cb, d_Lr, d_vg;
    DevBuf d_bptr, d_bf_cell, d_bf_kind, d_bf_bc, d_bf_diff, d_cin, d_eiso, d_mirror, d_ediff;
    DevBuf d_dlist, d_wdiff, d_wden, d_hw, d_bf_area;
    DevBuf d_e0, d_e1, d_ebar, d_Tb, d_T, d_mpart, d_margin, d_hpart, d_qband, d_q;
    // batch work
    int nbb = 0;
    DevBuf w_r, w_rw, w_p, w_ph, w_q, w_z, w_t, w_b, w_invD, w_xb;
    DevBuf s_done, s_iters, s_flagA, s_flagB, s_rho, s_alpha, s_omega, s_nrmr, s_nrm0, s_part, s_active, s_best;
    int active_cap = 0;
    double* h_pinned = nullptr;  // [4]
    int* h_pinned_i = nullptr;   // [4]
    std::vector<int> h_done, h_iters;
    // learned accelerator
    std::vector<double> centroid;
    bool has_mlp = false;
    DevBuf d_params, d_wpack, d_centroid, d_ring, d_feat, d_scale, d_y;
    std::vector<double> history;
    int history_rows = 0;
    // mixed form: scaled FP32 geometry and FP32 work vectors
    bool mixed_ready = false;
    DevBuf d_dg32, d_vo32, d_fc32, d_kb32, d_kappa;
    DevBuf x_xb, x_r, x_rw, x_p, x_ph, x_q, x_z, x_t, x_b, x_invD, x_dx, m_part, m_skip, m_active;
    // upwind sweep plan (form BTE_FORM_SWEEP)
    bool plan_ready = false;
    int plan_lagged_dirs = 0;
    bool sweep_margin = false;  // the sweep sums the margin partials (d_spart), chosen with the launch shape
    long long plan_levels = 0;
    DevBuf p_cell, p_dg, p_vo, p_nb, p_fc, p_lvl, p_lvl_off, p_part, p_bad, p_voi, p_kinv, d_spart, p_bidx, p_binvd;
    DevBuf d_bcell, d_bidx, d_bsum;
    // staged sweep: plan records, level-ordered right-hand side of a batch,
    // error flag of its bounded waits, stage lists by width; row length n2
    DevBuf p_rec, d_sweep_err;
    // level-order work: inflow masks, order, positions, level starts, in-degrees, counts
    DevBuf lo_mask, lo_perm, lo_pos, lo_lvl, lo_indeg, lo_small, lo_down;
    int plan_host_dirs = 0;  // directions the last plan ordered on the host
    std::vector<int> plan_lvl, plan_lvl_off;  // host copies of the level starts
    std::map<int, std::unique_ptr<StageList>> stage_lists;
    int n2 = 0;
    double ms_last_order = 0.0;  // host wall time of the last plan's level order
    DevBuf d_snap_e, d_snap_T, d_snap_ebar;  // accelerator: state before the last jump
    DevBuf d_aa_x, d_aa_g, d_aa_f, d_aa_part, d_aa_gram, d_aa_alpha, d_aa_flag;  // Anderson mixing
    double aa_prev_margin = 0.0;  // cells with boundary faces, cell -> row, boundary rhs per (system, row)
    int nbcell = 0;
    // inflow faces per cell at most (the sweep's face slots)
    int plan_fm = 2;
    // sweep kernel and launch shape picked by timing the candidates on the
    // first sweep of a plan
    SweepShape sweep_shape{};
    bool sweep_tuned = false;
    std::vector<SweepShape> sweep_tune_cand;
    std::vector<float> sweep_tune_ms;
    // profiling (opts->profile): events around each launch, resolved after a sync
    bool profile = false;
    std::vector<cudaEvent_t> ev_pool;
    struct Pending { int kind, iter; size_t ev; double bytes_fixed, bytes_per_active; };
    std::vector<Pending> pending;
    size_t ev_next = 0;
    bte_kernel_stat stats[kNumKinds];
    std::vector<int> h_active;
    // diffusion-synthetic acceleration: the scaled low-order operator and its
    // conjugate-gradient work (bte_dsa.cuh), the source temperature of the
    // running outer iteration, the right-hand side and the correction
    bool dsa_ready = false;
    int dsa_walls = 0;   // wall faces held at a fixed temperature
    int dsa_blocks = 0;  // cooperative grid of k_dsa_cg
    DevBuf d_lo_agg, d_lo_nagg;  // aggregate of each cell / of each face's neighbour (solve numbering)
    DevBuf d_lo_nb, d_lo_w, d_lo_dsc, d_Tsrc, d_dsa_b, d_dsa_x, d_dsa_xc, d_dsa_order, d_dsa_pos;
    DevBuf d_co_ainv, d_co_need_ptr, d_co_need, d_co_sums, d_co_sums0;
    DevBuf cg_r, cg_aw, cg_s, cg_x, cg_p, cg_u, cg_part, cg_bar, cg_stat, cg_relres;
    std::vector<int> dsa_order;  // position -> cell of the low-order solve's numbering
    int dsa_chunk = 0, dsa_seg = 0, dsa_n_agg = 0;
    bool dsa_stage = false;  // rows of the coarse inverse staged in shared memory
    bool dsa_topo = false;   // each block's couplings staged in shared memory
    int dsa_rows = 0;        // the longest need list (staged rows of the coarse inverse)
    size_t dsa_smem = 0;     // dynamic shared memory of k_dsa_pcg
    // results
    double* e_curr = nullptr;
    double* e_prev = nullptr;
    bool solved = false;
    std::vector<double> margins;
    long long launches = 0;
};

#define BTE_CUDA(call)                                                                    \
    do {                                                                                  \
        cudaError_t _e = (call);                                                          \
        if (_e != cudaSuccess) {                                                          \
            ctx->err = std::string(#call) + ": " + cudaGetErrorString(_e);                \
            return _e == cudaErrorMemoryAllocation ? BTE_ERR_OUT_OF_MEMORY : BTE_ERR_CUDA; \
        }                                                                                 \
    } while (0)

#define BTE_LAUNCHED()                                                                    \
    do {                                                                                  \
        ++ctx->launches;                                                                  \
        cudaError_t _e = cudaGetLastError();                                              \
        if (_e != cudaSuccess) {                                                          \
            ctx->err = std::string("kernel launch: ") + cudaGetErrorString(_e);           \
            return BTE_ERR_CUDA;                                                          \
        }                                                                                 \
    } while (0)

static bte_status fail(bte_ctx* ctx, bte_status st, const std::string& msg) {
    if (ctx) {
        std::lock_guard<std::mutex> lock(ctx->err_mutex);
        ctx->err = msg;
    }
    return st;
}

// Profiling: record an event pair around a launch; bytes = fixed + per_active * active[iter].
static cudaError_t prof_begin(bte_ctx* ctx, size_t* slot) {
    if (!ctx->profile) return cudaSuccess;
    if (ctx->ev_next + 2 > ctx->ev_pool.size()) {
        size_t add = std::max<size_t>(1024, ctx->ev_pool.size());
        for (size_t k = 0; k < add; ++k) {
            cudaEvent_t e;
            cudaError_t err = cudaEventCreate(&e);
            if (err != cudaSuccess) return err;
            ctx->ev_pool.push_back(e);
        }
    }
    *slot = ctx->ev_next;
    ctx->ev_next += 2;
    return cudaEventRecord(ctx->ev_pool[*slot], ctx->stream);
}
static cudaError_t prof_end(bte_ctx* ctx, size_t slot, int kind, int iter, double bytes_fixed,
                            double bytes_per_active) {
    if (!ctx->profile) return cudaSuccess;
    ctx->pending.push_back({kind, iter, slot, bytes_fixed, bytes_per_active});
    return cudaEventRecord(ctx->ev_pool[slot + 1], ctx->stream);
}
// After a stream sync: fold pending launches into the per-kind totals.
static void prof_resolve(bte_ctx* ctx, const int* active, int n_active) {
    for (const auto& p : ctx->pending) {
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->ev_pool[p.ev], ctx->ev_pool[p.ev + 1]);
        bte_kernel_stat& st = ctx->stats[p.kind];
        st.launches += 1;
        st.ms += ms;
        double act = (active && p.iter >= 0 && p.iter < n_active) ? active[p.iter] : 0.0;
        if (active && p.iter == -2)  // one launch over every iteration: all active system-iterations
            for (int k = 0; k < n_active; ++k) act += active[k];
        st.bytes += p.bytes_fixed + p.bytes_per_active * act;
    }
    ctx->pending.clear();
    ctx->ev_next = 0;
}

template <typename T>
static cudaError_t upload(DevBuf& buf, const std::vector<T>& h, cudaStream_t st) {
    cudaError_t e = buf.alloc(h.size() * sizeof(T));
    if (e != cudaSuccess) return e;
    if (h.empty()) return cudaSuccess;
    return cudaMemcpyAsync(buf.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, st);
}

extern "C" {

void bte_default_options(bte_options* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->max_iter = 10000;
    o->tol = 1e-5;
    o->form = BTE_FORM_PLAIN;
    o->inner_tol = 1e-9;
    o->inner_maxit = 1000;
    o->batch_systems = 0;
}

const char* bte_status_string(bte_status s) {
    switch (s) {
        case BTE_OK: return "ok";
        case BTE_ERR_INVALID_ARGUMENT: return "invalid argument";
        case BTE_ERR_STATE: return "call out of order";
        case BTE_ERR_CUDA: return "CUDA error";
        case BTE_ERR_OUT_OF_MEMORY: return "out of device memory";
        case BTE_ERR_UNSUPPORTED_BC: return "unsupported boundary condition";
        case BTE_ERR_NOT_CONVERGED: return "outer iteration did not converge within max_iter";
        case BTE_ERR_NUMERICAL: return "non-finite value in the outer iterate";
        case BTE_ERR_NO_DEVICE: return "no CUDA device";
    }
    return "unknown status";
}

const char* bte_last_error(const bte_ctx* ctx) { return ctx ? ctx->err.c_str() : g_create_error.c_str(); }

bte_status bte_create(bte_ctx** out, int device) {
    if (!out) return BTE_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        g_create_error = std::string("no CUDA device: ") + cudaGetErrorString(e);
        return BTE_ERR_NO_DEVICE;
    }
    if (device < 0) device = 0;
    device %= count;
    e = cudaSetDevice(device);
    if (e != cudaSuccess) {
        g_create_error = cudaGetErrorString(e);
        return BTE_ERR_CUDA;
    }
    auto* ctx = new bte_ctx;
    ctx->device = device;
    e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&ctx->h_pinned, 4 * sizeof(double));
    if (e == cudaSuccess) e = cudaMallocHost((void**)&ctx->h_pinned_i, 4 * sizeof(int));
    if (e != cudaSuccess) {
        g_create_error = cudaGetErrorString(e);
        delete ctx;
        return BTE_ERR_CUDA;
    }
    *out = ctx;
    return BTE_OK;
}

bte_status bte_destroy(bte_ctx* ctx) {
    if (!ctx) return BTE_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (cudaEvent_t e : ctx->ev_pool) cudaEventDestroy(e);
    if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
    if (ctx->h_pinned_i) cudaFreeHost(ctx->h_pinned_i);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    if (ctx->setup_stream) cudaStreamDestroy(ctx->setup_stream);
    delete ctx;
    return BTE_OK;
}

bte_status bte_set_geometry(bte_ctx* ctx, int dim, int n_cell, int n_face, const int* nbr,
                            const double* area, const double* normal, const double* volume) {
    if (!ctx) return BTE_ERR_INVALID_ARGUMENT;
    if (dim < 1 || dim > 3 || n_face != dim + 1 || n_cell <= 0 || !nbr || !area || !normal || !volume)
        return fail(ctx, BTE_ERR_INVALID_ARGUMENT, "bte_set_geometry: bad dim/n_cell/n_face or null array");
    const size_t nf = (size_t)n_cell * n_face;
    for (size_t i = 0; i < nf; ++i) {
        if (nbr[i] >= n_cell)
            return fail(ctx, BTE_ERR_INVALID_ARGUMENT, "bte_set_geometry: neighbour index out of range");
        if (!std::isfinite(area[i]) || !std::isfinite(normal[3 * i]) || !std::isfinite(normal[3 * i + 1]) ||
            !std::isfinite(normal[3 * i + 2]))
            return fail(ctx, BTE_ERR_INVALID_ARGUMENT, "bte_set_geometry: non-finite area or normal");
    }
    for (int c = 0; c < n_cell; ++c)
        if (!std::isfinite(volume[c]))
            return fail(ctx, BTE_ERR_INVALID_ARGUMENT, "bte_set_geometry: non-finite volume");
    ctx->dim = dim; ctx->n = n_cell; ctx->F = n_face;
    ctx->nbr.assign(nbr, nbr + nf);
    ctx->area.assign(area, area + nf);
    ctx->normal.assign(normal, normal + 3 * nf);
    ctx->volume.assign(volume, volume + n_cell);
    ctx->centroid.clear();
    ctx->has_geom = true;
    ctx->dirty = true;
    ctx->solved = false;
    return BTE_OK;
}

bte_status bte_set_quadrature(bte_ctx* ctx, int n_dir, const double* s, const double* S,
                              const double* omega, int DM, int num_theta, int num_phi,
                              double solid_angle, double T_ref) {
    if (!ctx) return BTE_ERR_INVALID_ARGUMENT;
    if (n_dir <= 0 || !s || !S || !omega || (DM != 2 && DM != 3) || num_phi <= 0 || num_theta <= 0)
        return fail(ctx, BTE_ERR_INVALID_ARGUMENT, "bte_set_quadrature: bad n_dir/DM/angles or null array");
    ctx->n_dir = n_dir; ctx->DM = DM; ctx->num_theta = num_theta; ctx->num_phi = num_phi;
    ctx->s.assign(s, s + 3 * n_dir);
    ctx->S.assign(S, S + 3 * n_dir);
    ctx->omega.assign(omega, omega + n_dir);
    ctx->solid_angle = solid_angle;
    ctx->T_ref = T_ref;
    ctx->has_quad = true;
    ctx->dirty = true;
    ctx->solved = false;
    return BTE_OK;
}

bte_status bte_set_bands(bte_ctx* ctx, int n_band, const double* vg, const double* tau,
                         const double* C, const double* Lr) {
    if (!ctx) return BTE_ERR_INVALID_ARGUMENT;
    if (n_band <= 0 || !vg || !tau || !C || !Lr)
        return fail(ctx, BTE_ERR_INVALID_ARGUMENT, "bte_set_bands: n_band <= 0 or null array");
    for (int b = 0; b < n_band; ++b)
        if (!std::isfinite(vg[b]) || !std::isfinite(tau[b]) || !std::isfinite(C[b]) || !std::isfinite(Lr[b]))
            return fail(ctx, BTE_ERR_NUMERICAL, "bte_set_bands: non-finite group velocity, relaxation time, "
                                                "heat capacity or Lr in band " + std::to_string(b));
    ctx->n_band = n_band;
    ctx->vg.assign(vg, vg + n_band);
    ctx->tau.assign(tau, tau + n_band);
    ctx->Cb.assign(C, C + n_band);
    ctx->Lr.assign(Lr, Lr + n_band);
    ctx->has_bands = true;
    ctx->dirty = true;
    ctx->solved = false;
    return BTE_OK;
}

bte_status bte_set_bcs(bte_ctx* ctx, int n_bc, const int* index, const int* type, const double* T) {
    if (!ctx) return BTE_ERR_INVALID_ARGUMENT;
    if (n_bc < 0 || (n_bc > 0 && (!index || !type || !T)))
        return fail(ctx, BTE_ERR_INVALID_ARGUMENT, "bte_set_bcs: bad n_bc or null array");
    for (int i = 0; i < n_bc; ++i)
        for (int j = 0; j < i; ++j)
            if (index[i] == index[j])
                return fail(ctx, BTE_ERR_INVALID_ARGUMENT,
                            "bte_set_bcs: two boundary-condition rows name the same boundary entity");
    ctx->n_bc = n_bc;
    ctx->bc_index.assign(index, index + n_bc);
    ctx->bc_type.assign(type, type + n_bc);
    ctx->bc_T.assign(T, T + n_bc);
    ctx->has_bcs = true;
    ctx->dirty = true;
    ctx->solved = false;
    return BTE_OK;
}

}  // extern "C"

// Specular partner of direction d (src/StaticBTESolver.cpp:205-252).
static int mirror_of(int type, int dim, int d, int num_phi) {
    const int it = d / (4 * num_phi);
    int ip = d % (4 * num_phi);
    if (type == 31) {
        if (dim == 2) ip = ip >= 2 * num_phi ? 6 * num_phi - ip - 1 : 2 * num_phi - ip - 1;
        else ip = 4 * num_phi - ip - 1;
        return it * 4 * num_phi + ip;
    }
    if (type == 32) {
        if (dim == 2) return it * 4 * num_phi + (4 * num_phi - ip - 1);
        const int ix = ip / (2 * num_phi), isx = 2 * num_phi - ip % (2 * num_phi) - 1;
        return it * 4 * num_phi + isx + ix * 2 * num_phi;
    }
    // 33: the polar index is mirrored with num_phi, as the reference does (:250)
    const int iz = 2 * num_phi - it - 1;
    return ip + iz * 4 * num_phi;
}

// Upload inputs, build boundary tables, per-direction geometry and state buffers.
// BTE_HOST_TIMING=1: each host set-up step's wall time goes to stderr
// (a diagnostic of the end-to-end cost of new inputs).
struct HostTimer {
    const char* what;
    std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
    static bool on() {
        static const bool v = [] { const char* e = std::getenv("BTE_HOST_TIMING"); return e && *e && *e != '0'; }();
        return v;
    }
    explicit HostTimer(const char* w) : what(w) {}
    void lap(const char* step) {
        if (!on()) return;
        const auto now = std::chrono::steady_clock::now();
        std::fprintf(stderr, "[bte host] %s: %s %.3f ms\n", what, step,
                     std::chrono::duration<double, std::milli>(now - t).count());
        t = now;
    }
};

static bte_status setup(bte_ctx* ctx, int batch_systems) {
    const int n = ctx->n, F = ctx->F, ND = ctx->n_dir, NB = ctx->n_band, dim = ctx->dim;
    ctx->Np = (size_t)((n + bte::CH - 1) / bte::CH) * bte::CH;
    ctx->nchunk = (int)(ctx->Np / bte::CH);
    const size_t Np = ctx->Np;
    cudaStream_t st = ctx->stream;

    // ---- boundary faces matched to boundary-condition rows, sorted by (cell, face)
    std::vector<int> bptr(Np + 1, 0), bf_cell, bf_face, bf_kind, bf_bc, bf_diff;
    for (int c = 0; c < n; ++c) {
        bptr[c] = (int)bf_cell.size();
        for (int f = 0; f < F; ++f) {
            const int code = ctx->nbr[(size_t)c * F + f];
            if (code >= 0) continue;
            for (int i = 0; i < ctx->n_bc; ++i) {
                if (ctx->bc_index[i] != code) continue;
                const int t = ctx->bc_type[i];
                const bool ok = t == 1 || t == 2 || ((t == 31 || t == 32) && dim >= 2) || (t == 33 && dim == 3);
                if (!ok) {
                    char buf[160];
                    std::snprintf(buf, sizeof(buf),
                                  "boundary condition type %d on entity %d is not supported for a %dD mesh", t,
                                  -code - 1, dim);
                    return fail(ctx, BTE_ERR_UNSUPPORTED_BC, buf);
                }
                bf_cell.push_back(c); bf_face.push_back(f); bf_kind.push_back(t); bf_bc.push_back(i);
                bf_diff.push_back(-1);
                break;
            }
        }
    }
    for (size_t c = n; c <= Np; ++c) bptr[c] = (int)bf_cell.size();
    const int nbf = (int)bf_cell.size();
    ctx->nbf = nbf;
    ctx->h_bf_bc = bf_bc;
    std::vector<double> cin((size_t)ND * std::max(nbf, 1), 0.0), hw((size_t)std::max(nbf, 1) * ND, 0.0),
        bf_area(std::max(nbf, 1), 0.0);
    std::vector<int> dlist;
    std::vector<double> wdiff, wden;
    for (int k = 0; k < nbf; ++k) {
        const size_t cf = (size_t)bf_cell[k] * F + bf_face[k];
        const double* nn = &ctx->normal[3 * cf];
        const double A = ctx->area[cf];
        bf_area[k] = A;
        double wsum = 0.0;
        std::vector<double> w(ND, 0.0);
        for (int d = 0; d < ND; ++d) {
            const double sn = ctx->s[3 * d] * nn[0] + ctx->s[3 * d + 1] * nn[1] + ctx->s[3 * d + 2] * nn[2];
            const double Sn = ctx->S[3 * d] * nn[0] + ctx->S[3 * d + 1] * nn[1] + ctx->S[3 * d + 2] * nn[2];
            const double g = dim > 1 ? Sn : sn;
            if (sn < 0) cin[(size_t)d * nbf + k] = A * g;
            // heat-flux weights (:336-351)
            if (ctx->DM == 3 && dim == 3) hw[(size_t)k * ND + d] = sn * A * ctx->omega[d];
            else if (dim == 1) hw[(size_t)k * ND + d] = sn * ctx->omega[d];
            else hw[(size_t)k * ND + d] = Sn * A;
            // diffuse-wall weights over outgoing directions (:183-203)
            if (sn > 0) {
                if (dim == 3) { w[d] = Sn * ctx->omega[d]; wsum += Sn * ctx->omega[d]; }
                else if (dim == 2) { w[d] = Sn; wsum += Sn; }
                else w[d] = sn * ctx->omega[d];
            }
        }
        if (bf_kind[k] == 2) {
            bf_diff[k] = (int)dlist.size();
            dlist.push_back(k);
            wdiff.insert(wdiff.end(), w.begin(), w.end());
            wden.push_back(dim != 1 ? wsum : M_PI);
        }
    }
    ctx->ndiff = (int)dlist.size();
    std::vector<double> eiso((size_t)NB * std::max(ctx->n_bc, 1), 0.0);
    for (int b = 0; b < NB; ++b)
        for (int i = 0; i < ctx->n_bc; ++i)
            eiso[(size_t)b * ctx->n_bc + i] = ctx->Cb[b] / ctx->solid_angle * (ctx->bc_T[i] - ctx->T_ref);
    std::vector<int> mir(3 * ND, 0);
    for (int d = 0; d < ND; ++d) {
        mir[d] = dim >= 2 ? mirror_of(31, dim, d, ctx->num_phi) : d;
        mir[ND + d] = dim >= 2 ? mirror_of(32, dim, d, ctx->num_phi) : d;
        mir[2 * ND + d] = dim == 3 ? mirror_of(33, dim, d, ctx->num_phi) : d;
    }
    for (int t = 0; t < 3; ++t)
        for (int d = 0; d < ND; ++d)
            if (mir[t * ND + d] < 0 || mir[t * ND + d] >= ND) {
                bool used = false;
                for (int k = 0; k < nbf; ++k) used |= bf_kind[k] == 31 + t;
                if (used)
                    return fail(ctx, BTE_ERR_UNSUPPORTED_BC,
                                "specular boundary needs num_theta == num_phi for this direction set");
                mir[t * ND + d] = d;
            }
    std::vector<double> kb(NB);
    for (int b = 0; b < NB; ++b) kb[b] = ctx->vg[b] * ctx->tau[b];
    if (dlist.empty()) { dlist.push_back(0); wdiff.assign(ND, 0.0); wden.push_back(1.0); }
    if (bf_cell.empty()) { bf_cell.push_back(0); bf_kind.push_back(1); bf_bc.push_back(0); bf_diff.push_back(-1); }

    // ---- uploads
    std::vector<int> nbpad((size_t)F * Np);
    for (int f = 0; f < F; ++f)
        for (size_t c = 0; c < Np; ++c) {
            int v = c < (size_t)n ? ctx->nbr[c * F + f] : -1;
            nbpad[(size_t)f * Np + c] = v >= 0 ? v : (int)c;
        }
    BTE_CUDA(upload(ctx->d_normal, ctx->normal, st));
    BTE_CUDA(upload(ctx->d_area, ctx->area, st));
    BTE_CUDA(upload(ctx->d_nbr, ctx->nbr, st));
    BTE_CUDA(upload(ctx->d_volume, ctx->volume, st));
    BTE_CUDA(upload(ctx->d_s, ctx->s, st));
    BTE_CUDA(upload(ctx->d_S, ctx->S, st));
    BTE_CUDA(upload(ctx->d_omega, ctx->omega, st));
    BTE_CUDA(upload(ctx->d_nb, nbpad, st));
    BTE_CUDA(upload(ctx->d_kb, kb, st));
    BTE_CUDA(upload(ctx->d_Cb, ctx->Cb, st));
    BTE_CUDA(upload(ctx->d_Lr, ctx->Lr, st));
    BTE_CUDA(upload(ctx->d_vg, ctx->vg, st));
    BTE_CUDA(upload(ctx->d_bptr, bptr, st));
    {
        std::vector<int> bcell, bidx(n, -1);
        for (int c = 0; c < n; ++c)
            if (bptr[c + 1] > bptr[c]) { bidx[c] = (int)bcell.size(); bcell.push_back(c); }
        ctx->nbcell = (int)bcell.size();
        if (bcell.empty()) bcell.push_back(0);
        BTE_CUDA(upload(ctx->d_bcell, bcell, st));
        BTE_CUDA(upload(ctx->d_bidx, bidx, st));
    }
    BTE_CUDA(upload(ctx->d_bf_cell, bf_cell, st));
    BTE_CUDA(upload(ctx->d_bf_kind, bf_kind, st));
    BTE_CUDA(upload(ctx->d_bf_bc, bf_bc, st));
    BTE_CUDA(upload(ctx->d_bf_diff, bf_diff, st));
    BTE_CUDA(upload(ctx->d_cin, cin, st));
    BTE_CUDA(upload(ctx->d_eiso, eiso, st));
    BTE_CUDA(upload(ctx->d_mirror, mir, st));
    BTE_CUDA(upload(ctx->d_dlist, dlist, st));
    BTE_CUDA(upload(ctx->d_wdiff, wdiff, st));
    BTE_CUDA(upload(ctx->d_wden, wden, st));
    BTE_CUDA(upload(ctx->d_hw, hw, st));
    BTE_CUDA(upload(ctx->d_bf_area, bf_area, st));
    BTE_CUDA(ctx->d_ediff.alloc(sizeof(double) * NB * std::max(nbf, 1)));
    BTE_CUDA(cudaMemsetAsync(ctx->d_ediff.p, 0, ctx->d_ediff.bytes, st));

    // ---- per-direction geometry (one launch)
    BTE_CUDA(ctx->d_dg.alloc(sizeof(double) * ND * Np));
    BTE_CUDA(ctx->d_vo.alloc(sizeof(double) * ND * Np));
    BTE_CUDA(ctx->d_fc.alloc(sizeof(double) * ND * F * Np));
    {
        dim3 grid((unsigned)((Np + 255) / 256), ND);
        bte::k_direction_geometry<<<grid, 256, 0, st>>>(
            ctx->d_normal.as<double>(), ctx->d_area.as<double>(), ctx->d_nbr.as<int>(), ctx->d_volume.as<double>(),
            ctx->d_s.as<double>(), ctx->d_S.as<double>(), ctx->d_omega.as<double>(), n, F, dim, Np,
            ctx->d_dg.as<double>(), ctx->d_vo.as<double>(), ctx->d_fc.as<double>());
        BTE_LAUNCHED();
    }

    // ---- state
    const size_t ne = (size_t)NB * ND * Np;
    BTE_CUDA(ctx->d_e0.alloc(sizeof(double) * ne));
    BTE_CUDA(ctx->d_e1.alloc(sizeof(double) * ne));
    BTE_CUDA(ctx->d_ebar.alloc(sizeof(double) * NB * Np));
    BTE_CUDA(ctx->d_Tb.alloc(sizeof(double) * NB * Np));
    BTE_CUDA(ctx->d_T.alloc(sizeof(double) * Np));
    BTE_CUDA(ctx->d_mpart.alloc(sizeof(double) * NB * (Np / bte::THREADS + 1)));
    BTE_CUDA(ctx->d_margin.alloc(sizeof(double) * 2));
    BTE_CUDA(ctx->d_hpart.alloc(sizeof(double) * NB * std::max(nbf, 1)));
    BTE_CUDA(ctx->d_qband.alloc(sizeof(double) * std::max(ctx->n_bc, 1) * NB));
    BTE_CUDA(ctx->d_q.alloc(sizeof(double) * std::max(ctx->n_bc, 1)));

    // ---- batch work buffers: nbb bands x all directions per batch
    size_t free_b = 0, total_b = 0;
    BTE_CUDA(cudaMemGetInfo(&free_b, &total_b));
    // (the PLAIN form's 10 work vectors per system set the batch; they are
    // allocated on its first use, the MIXED form allocates its own)
    const size_t per_sys = sizeof(double) * Np * 10 + sizeof(double) * 7 * ctx->nchunk + 64;
    int nbb = NB;
    if (batch_systems > 0) nbb = std::max(1, std::min(NB, batch_systems / ND));
    const size_t reserve = (size_t)2 << 30;
    while (nbb > 1 && (size_t)nbb * ND * per_sys + reserve > free_b) nbb = (nbb + 1) / 2;
    ctx->nbb = nbb;
    const size_t S = (size_t)nbb * ND;
    BTE_CUDA(ctx->s_done.alloc(sizeof(int) * S));
    BTE_CUDA(ctx->s_iters.alloc(sizeof(int) * S));
    BTE_CUDA(ctx->s_flagA.alloc(sizeof(int) * 2 * S));
    BTE_CUDA(ctx->s_flagB.alloc(sizeof(int) * 2 * S));
    BTE_CUDA(ctx->s_rho.alloc(sizeof(double) * 2 * S));
    BTE_CUDA(ctx->s_alpha.alloc(sizeof(double) * S));
    BTE_CUDA(ctx->s_omega.alloc(sizeof(double) * S));
    BTE_CUDA(ctx->s_nrmr.alloc(sizeof(double) * S));
    BTE_CUDA(ctx->s_nrm0.alloc(sizeof(double) * S));
    BTE_CUDA(ctx->s_best.alloc(sizeof(double) * 2 * S));
    BTE_CUDA(ctx->s_part.alloc(sizeof(double) * 7 * S * ctx->nchunk));
    ctx->h_done.resize(S);
    ctx->h_iters.resize(S);
    ctx->plan_ready = false;
    ctx->mixed_ready = false;
    ctx->dsa_ready = false;
    ctx->dirty = false;
    return BTE_OK;
}

// FP32 geometry for the mixed form, scaled per direction by 1 / mean(V Omega_d).
static bte_status setup_mixed(bte_ctx* ctx) {
    const int n = ctx->n, F = ctx->F, ND = ctx->n_dir, NB = ctx->n_band;
    const size_t Np = ctx->Np;
    cudaStream_t st = ctx->stream;
    double vmean = 0;
    for (double v : ctx->volume) vmean += v;
    vmean /= n;
    std::vector<double> kappa(ND);
    for (int d = 0; d < ND; ++d) kappa[d] = 1.0 / (ctx->dim > 1 ? vmean * ctx->omega[d] : vmean);
    std::vector<float> kb32(NB);
    for (int b = 0; b < NB; ++b) kb32[b] = (float)(ctx->vg[b] * ctx->tau[b]);
    BTE_CUDA(upload(ctx->d_kappa, kappa, st));
    BTE_CUDA(upload(ctx->d_kb32, kb32, st));
    BTE_CUDA(ctx->d_dg32.alloc(sizeof(float) * ND * Np));
    BTE_CUDA(ctx->d_vo32.alloc(sizeof(float) * ND * Np));
    BTE_CUDA(ctx->d_fc32.alloc(sizeof(float) * ND * F * Np));
    bte::k_geometry32<<<dim3((unsigned)((Np + 255) / 256), ND), 256, 0, st>>>(
        ctx->d_dg.as<double>(), ctx->d_vo.as<double>(), ctx->d_fc.as<double>(), ctx->d_kappa.as<double>(), n, F, Np,
        ctx->d_dg32.as<float>(), ctx->d_vo32.as<float>(), ctx->d_fc32.as<float>());
    BTE_LAUNCHED();
    const size_t S = (size_t)ctx->nbb * ND;
    for (DevBuf* b : {&ctx->x_r, &ctx->x_rw, &ctx->x_p, &ctx->x_ph, &ctx->x_q, &ctx->x_z, &ctx->x_t, &ctx->x_b,
                      &ctx->x_invD, &ctx->x_dx, &ctx->x_xb})
        BTE_CUDA(b->alloc(sizeof(float) * S * Np));
    BTE_CUDA(ctx->m_part.alloc(sizeof(double) * 2 * S * ctx->nchunk));
    BTE_CUDA(ctx->m_skip.alloc(sizeof(int) * S));
    BTE_CUDA(ctx->m_active.alloc(sizeof(int)));
    ctx->mixed_ready = true;
    return BTE_OK;
}

// ---------------------------------------------------------------------------
// Diffusion-synthetic acceleration: the low-order operator and its solve.

// Weight of the physical second-moment term in the low-order face coefficient
// (0 keeps only the upwind scheme's numerical diffusion).  1/4 came out best
// on 2D squares from thick (Lambda/h ~ 1e-3) to mixed (Lambda/h up to ~8)
// cells: 0.17-0.29 error reduction per outer iteration.
constexpr double kDsaBeta = 0.25;
// BTE_DSA_BETA=x replaces it (a study of the low-order operator; the
// transport iteration and its fixed point do not depend on it).
static double dsa_beta() {
    const char* v = std::getenv("BTE_DSA_BETA");
    if (!v || !*v) return kDsaBeta;
    const double b = std::atof(v);
    return b >= 0.0 && std::isfinite(b) ? b : kDsaBeta;
}
constexpr int kDsaThreads = bte::dsa::THREADS;
// Inner tolerance of the mixed form under the correction (at most).
constexpr double kDsaMixedInnerTol = 1e-11;

// Upload a low-order operator (nb, W as bte_dsa_solve takes them) in its
// symmetrically scaled form, in a locality order of the cells with the
// two-level preconditioner's coarse operator, and size the conjugate-gradient
// work for n cells.
// Host part of the low-order solve's set-up: Jacobi scaling, locality
// order, the permuted operator and the coarse operator.  No CUDA calls, so it
// can run on a host thread while the sweep plan is built.
struct DsaHostPlan {
    int n = 0, F = 0, nblk = 0;
    std::vector<int> order, pos, nbv, agg, nagg;
    std::vector<double> dscp;
    std::vector<float> w;
    bte::DsaCoarse co;
};

// pre_order (optional): a locality order already computed, used as it is
// without pre_cm, and with pre_cm (the coupling pattern it was computed for,
// [n][F]) only when the pattern of W is the same.
// Runs body(i0, i1) over [0, n) split into contiguous ranges on host
// threads (one range below 65,536 items); each i is written by one range.
template <typename Body>
static void host_ranges(int n, Body&& body) {
    const int T = n < 65536 ? 1 : std::max(1, std::min(8, (int)std::thread::hardware_concurrency()));
    if (T == 1) {
        body(0, n);
        return;
    }
    std::vector<std::thread> pool;
    for (int t = 0; t < T; ++t)
        pool.emplace_back(body, (int)((long long)n * t / T), (int)((long long)n * (t + 1) / T));
    for (auto& th : pool) th.join();
}

static void dsa_host_plan(int n, int F, const int* nb, const double* W, int nblk, DsaHostPlan& hp,
                          std::vector<int>* pre_order = nullptr, const std::vector<int>* pre_cm = nullptr) {
    HostTimer tm("dsa_host_plan");
    hp.n = n;
    hp.F = F;
    hp.nblk = nblk;
    std::vector<double> dsc(n, 0.0);
    host_ranges(n, [&](int c0, int c1) {
        for (int c = c0; c < c1; ++c) {
            double diag = 0.0;
            for (int f = 0; f < F; ++f) diag += W[(size_t)f * n + c];
            dsc[c] = diag > 0.0 ? 1.0 / std::sqrt(diag) : 0.0;
        }
    });
    tm.lap("scaling");
    // locality order: contiguous position ranges are compact groups of cells
    const bool given = pre_order && pre_order->size() == (size_t)n;
    if (given && !pre_cm) {
        hp.order.swap(*pre_order);
    } else {
        std::vector<int> cm((size_t)n * F);
        for (int f = 0; f < F; ++f)
            for (int c = 0; c < n; ++c)
                cm[(size_t)c * F + f] = W[(size_t)f * n + c] > 0.0 ? nb[(size_t)f * n + c] : -1;
        const int agg_cells = std::max(1, n / (nblk * bte::dsa::AGG));
        if (given && *pre_cm == cm) hp.order.swap(*pre_order);
        else bte::locality_order(n, F, cm.data(), std::max(8, agg_cells / 2), hp.order);
    }
    tm.lap("locality order");
    const std::vector<int>& order = hp.order;
    std::vector<int>& pos = hp.pos;
    pos.assign(n, 0);
    for (int k = 0; k < n; ++k) pos[order[k]] = k;
    std::vector<double> wd((size_t)F * n, 0.0);
    hp.dscp.assign(n, 0.0);
    hp.w.assign((size_t)F * n, 0.0f);
    hp.nbv.assign((size_t)F * n, -1);
    host_ranges(n, [&](int k0, int k1) {
        for (int k = k0; k < k1; ++k) {
            const int c = order[k];
            hp.dscp[k] = dsc[c];
            for (int f = 0; f < F; ++f) {
                const size_t q = (size_t)f * n + c;
                const int o = nb[q];
                if (o >= 0 && W[q] > 0.0) {
                    const size_t qk = (size_t)f * n + k;
                    wd[qk] = W[q] * dsc[c] * dsc[o];
                    hp.w[qk] = (float)wd[qk];
                    hp.nbv[qk] = pos[o];
                }
            }
        }
    });
    tm.lap("permuted operator");
    bte::dsa_coarse(n, F, hp.nbv.data(), wd.data(), nblk, bte::dsa::AGG, hp.co);
    hp.agg = hp.co.agg;
    hp.nagg.assign((size_t)F * n, -1);
    for (size_t q = 0; q < (size_t)F * n; ++q)
        if (hp.nbv[q] >= 0) hp.nagg[q] = hp.agg[hp.nbv[q]];
    tm.lap("coarse operator");
}

// Blocks of the cooperative low-order kernel for n cells: at most one per SM.
static bte_status dsa_blocks(bte_ctx* ctx, int n, int* nblk) {
    int coop = 0, sms = 0;
    BTE_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device));
    if (!coop) return fail(ctx, BTE_ERR_CUDA, "dsa: the device does not support cooperative launches");
    BTE_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    // enough threads for the cells, few blocks at each barrier
    *nblk = std::max(1, std::min(sms, (n + kDsaThreads - 1) / kDsaThreads));
    return BTE_OK;
}

// Device part: the coarse inverse, the uploads and the work vectors.
static bte_status dsa_upload(bte_ctx* ctx, DsaHostPlan& hp, cudaStream_t st) {
    HostTimer tm("dsa_upload");
    const int n = hp.n, F = hp.F, nblk = hp.nblk;
    int sms = 0, occ = 0;
    BTE_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    ctx->dsa_blocks = nblk;
    ctx->dsa_order = hp.order;
    const bte::DsaCoarse& co = hp.co;
    const std::vector<int>& order = hp.order;
    const std::vector<int>& pos = hp.pos;
    const std::vector<int>& nbv = hp.nbv;
    const std::vector<float>& w = hp.w;
    const std::vector<double>& dscp = hp.dscp;
    // the coarse operator's inverse by Gauss-Jordan steps on the device (FP64),
    // stored in FP32 for the preconditioner
    {
        const int m = co.n_agg;
        DevBuf ga, gb, gbad;
        BTE_CUDA(upload(ga, co.ac, st));
        BTE_CUDA(gb.alloc(sizeof(double) * (size_t)m * m));
        BTE_CUDA(gbad.alloc(sizeof(int) * 2));  // [0] error flag, [1] (as unsigned) grid barrier counter
        BTE_CUDA(cudaMemsetAsync(gbad.p, 0, sizeof(int) * 2, st));
        double* a = ga.as<double>();
        double* b = gb.as<double>();
        // one cooperative launch (one block per SM) when every block fits:
        // kGjBlock pivots per step when the pivot rows fit in shared memory,
        // else one pivot per step; without cooperative launches, one launch per step
        int coop_ok = 0, occ_gj = 0, sms_gj = 0, occ_blk = 0, smem_opt = 0;
        BTE_CUDA(cudaDeviceGetAttribute(&coop_ok, cudaDevAttrCooperativeLaunch, ctx->device));
        BTE_CUDA(cudaDeviceGetAttribute(&sms_gj, cudaDevAttrMultiProcessorCount, ctx->device));
        BTE_CUDA(cudaDeviceGetAttribute(&smem_opt, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device));
        BTE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_gj, bte::dsa::k_gj_all, 1024, 0));
        const int kgb = bte::dsa::kGjBlock;
        const size_t smem_blk = sizeof(double) * (size_t)kgb * (m + kgb + 1);
        if (coop_ok && smem_blk + 1024 <= (size_t)smem_opt) {
            BTE_CUDA(cudaFuncSetAttribute(bte::dsa::k_gj_block_all, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem_blk));
            BTE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_blk, bte::dsa::k_gj_block_all, 1024, smem_blk));
        }
        if (occ_blk >= 1) {
            const int nb = std::min(sms_gj, m);
            int* badp = gbad.as<int>();
            unsigned* barp = reinterpret_cast<unsigned*>(badp + 1);
            int mm = m;
            void* args[] = {&a, &b, &mm, &barp, &badp};
            BTE_CUDA(cudaLaunchCooperativeKernel((const void*)bte::dsa::k_gj_block_all, dim3(nb), dim3(1024), args,
                                                 smem_blk, st));
            if (((m + kgb - 1) / kgb) % 2) std::swap(a, b);  // the inverse is in A after an even number of steps
        } else if (coop_ok && occ_gj >= 1) {
            const int nb = std::min(sms_gj, m);
            int* badp = gbad.as<int>();
            unsigned* barp = reinterpret_cast<unsigned*>(badp + 1);
            int mm = m;
            void* args[] = {&a, &b, &mm, &barp, &badp};
            BTE_CUDA(cudaLaunchCooperativeKernel((const void*)bte::dsa::k_gj_all, dim3(nb), dim3(1024), args, 0, st));
            if (m % 2) std::swap(a, b);  // the inverse is in A after an even number of steps
        } else {
            for (int k = 0; k < m; ++k) {
                bte::dsa::k_gj_step<<<dim3((m + 255) / 256, m), 256, 0, st>>>(a, b, m, k, gbad.as<int>());
                std::swap(a, b);
            }
        }
        BTE_CUDA(ctx->d_co_ainv.alloc(sizeof(float) * (size_t)m * m));
        bte::dsa::k_to_float<<<(unsigned)(((size_t)m * m + 255) / 256), 256, 0, st>>>(
            a, ctx->d_co_ainv.as<float>(), (size_t)m * m);
        BTE_LAUNCHED();
        int bad = 0;
        BTE_CUDA(cudaMemcpyAsync(&bad, gbad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
        BTE_CUDA(cudaStreamSynchronize(st));
        if (bad == 2) return fail(ctx, BTE_ERR_CUDA, "dsa: a grid barrier of the coarse inversion timed out");
        if (bad)
            return fail(ctx, BTE_ERR_INVALID_ARGUMENT,
                        "dsa: the low-order operator is singular (no wall held at a fixed temperature)");
        tm.lap("coarse inverse (device)");
    }
    ctx->dsa_chunk = co.chunk;
    ctx->dsa_seg = co.seg;
    ctx->dsa_n_agg = co.n_agg;
    // the block's rows of the coarse inverse live in shared memory when they fit
    int rows = 0, smem_max = 0;
    for (int k = 0; k < nblk; ++k) rows = std::max(rows, co.need_ptr[k + 1] - co.need_ptr[k]);
    BTE_CUDA(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device));
    const size_t staged = sizeof(float) * (2 + (size_t)rows) * co.n_agg;
    ctx->dsa_stage = staged + 16384 <= (size_t)smem_max;
    ctx->dsa_rows = rows;
    ctx->dsa_smem = ctx->dsa_stage ? staged : sizeof(float) * 2 * (size_t)co.n_agg;
    // and the blocks' couplings after them, when those fit too
    const size_t with_topo = sizeof(float) * (bte::dsa::dsa_topo_offset(co.n_agg, ctx->dsa_stage ? rows : 0) +
                                              bte::dsa::dsa_topo_words(co.chunk, F));
    ctx->dsa_topo = with_topo + 16384 <= (size_t)smem_max;
    if (ctx->dsa_topo) ctx->dsa_smem = with_topo;
    auto pcg = ctx->dsa_topo ? bte::dsa::k_dsa_pcg<true> : bte::dsa::k_dsa_pcg<false>;
    BTE_CUDA(cudaFuncSetAttribute(pcg, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ctx->dsa_smem));
    BTE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, pcg, kDsaThreads, ctx->dsa_smem));
    if (occ < 1 || nblk > occ * sms) return fail(ctx, BTE_ERR_CUDA, "dsa: the low-order kernel cannot be resident");
    BTE_CUDA(upload(ctx->d_lo_nb, nbv, st));
    BTE_CUDA(upload(ctx->d_lo_w, w, st));
    BTE_CUDA(upload(ctx->d_lo_dsc, dscp, st));
    BTE_CUDA(upload(ctx->d_dsa_order, order, st));
    BTE_CUDA(upload(ctx->d_dsa_pos, pos, st));
    BTE_CUDA(upload(ctx->d_co_need_ptr, co.need_ptr, st));
    BTE_CUDA(upload(ctx->d_lo_agg, hp.agg, st));
    BTE_CUDA(upload(ctx->d_lo_nagg, hp.nagg, st));
    BTE_CUDA(upload(ctx->d_co_need, co.need, st));
    BTE_CUDA(ctx->d_co_sums.alloc(sizeof(float) * 6 * (size_t)co.n_agg));
    BTE_CUDA(ctx->d_co_sums0.alloc(sizeof(double) * (size_t)co.n_agg));
    BTE_CUDA(cudaMemsetAsync(ctx->d_co_sums.p, 0, ctx->d_co_sums.bytes, st));
    BTE_CUDA(cudaMemsetAsync(ctx->d_co_sums0.p, 0, ctx->d_co_sums0.bytes, st));
    const size_t nn = (size_t)n;
    BTE_CUDA(ctx->cg_r.alloc(sizeof(float) * 2 * nn));
    BTE_CUDA(ctx->cg_aw.alloc(sizeof(float) * 2 * nn));
    BTE_CUDA(ctx->cg_s.alloc(sizeof(float) * 2 * nn));
    BTE_CUDA(ctx->cg_x.alloc(sizeof(float) * nn));
    BTE_CUDA(ctx->cg_p.alloc(sizeof(float) * nn));
    BTE_CUDA(ctx->cg_u.alloc(sizeof(float) * nn));
    BTE_CUDA(ctx->cg_part.alloc(sizeof(double) * 4 * (size_t)nblk));
    BTE_CUDA(ctx->cg_bar.alloc(sizeof(unsigned) * 2));
    BTE_CUDA(ctx->cg_stat.alloc(sizeof(int) * 4));
    BTE_CUDA(ctx->cg_relres.alloc(sizeof(double)));
    BTE_CUDA(ctx->d_dsa_b.alloc(sizeof(double) * nn));
    BTE_CUDA(ctx->d_dsa_x.alloc(sizeof(double) * nn));
    BTE_CUDA(ctx->d_dsa_xc.alloc(sizeof(double) * nn));
    BTE_CUDA(cudaMemsetAsync(ctx->cg_stat.p, 0, sizeof(int) * 4, st));
    tm.lap("uploads");
    return BTE_OK;
}

// Upload a low-order operator (nb, W as bte_dsa_solve takes them) in its
// symmetrically scaled form, in a locality order of the cells with the
// two-level preconditioner's coarse operator, and size the conjugate-gradient
// work for n cells.
static bte_status dsa_prepare(bte_ctx* ctx, int n, int F, const int* nb, const double* W) {
    int nblk = 0;
    bte_status s = dsa_blocks(ctx, n, &nblk);
    if (s != BTE_OK) return s;
    DsaHostPlan hp;
    dsa_host_plan(n, F, nb, W, nblk, hp);
    return dsa_upload(ctx, hp, ctx->stream);
}

// One low-order solve of d_dsa_b into d_dsa_x, both in the solve's numbering
// (cooperative launch, every block resident).
static bte_status dsa_launch(bte_ctx* ctx, int n, int F, double tol, int maxit) {
    cudaStream_t st = ctx->stream;
    BTE_CUDA(cudaMemsetAsync(ctx->cg_bar.p, 0, sizeof(unsigned) * 2, st));
    bte::dsa::Lo lo{n, F, ctx->d_lo_nb.as<int>(), ctx->d_lo_w.as<float>(), ctx->d_lo_dsc.as<double>(),
                    ctx->d_lo_agg.as<int>(), ctx->d_lo_nagg.as<int>()};
    bte::dsa::Coarse co{ctx->dsa_chunk, ctx->dsa_seg, ctx->dsa_n_agg, ctx->dsa_stage ? 1 : 0, ctx->dsa_rows,
                        ctx->dsa_topo ? 1 : 0, ctx->d_co_ainv.as<float>(),
                        ctx->d_co_need_ptr.as<int>(), ctx->d_co_need.as<int>(), ctx->d_co_sums.as<float>(),
                        ctx->d_co_sums0.as<double>()};
    bte::dsa::CgWork wk{ctx->cg_r.as<float>(), ctx->cg_aw.as<float>(), ctx->cg_s.as<float>(), ctx->cg_x.as<float>(),
                        ctx->cg_p.as<float>(), ctx->cg_u.as<float>(), ctx->cg_part.as<double>(),
                        ctx->cg_bar.as<unsigned>(), ctx->cg_stat.as<int>(), ctx->cg_relres.as<double>()};
    const double* b = ctx->d_dsa_b.as<double>();
    double* x = ctx->d_dsa_x.as<double>();
    void* args[] = {&lo, &co, &wk, &b, &tol, &maxit, &x};
    const void* pcg = ctx->dsa_topo ? (const void*)bte::dsa::k_dsa_pcg<true> : (const void*)bte::dsa::k_dsa_pcg<false>;
    BTE_CUDA(cudaLaunchCooperativeKernel(pcg, dim3(ctx->dsa_blocks), dim3(kDsaThreads), args, ctx->dsa_smem, st));
    BTE_LAUNCHED();
    return BTE_OK;
}

// The low-order operator of the mesh, bands and walls of ctx: the host part
// (coefficients, then dsa_host_plan; it reads only ctx's host-side inputs, so
// it can run on a host thread next to the sweep plan's construction) ...
struct DsaSetupHost {
    int n_dirichlet = 0;
    DsaHostPlan hp;
};

static void setup_dsa_host(const bte_ctx* ctx, int nblk, DsaSetupHost& out) {
    const int n = ctx->n, F = ctx->F;
    // walls held at a fixed temperature: isothermal rows, and boundary faces
    // that no row names (their wall energy stays 0 in the reference)
    std::vector<char> fixed((size_t)n * F, 0);
    for (size_t cf = 0; cf < (size_t)n * F; ++cf) {
        const int code = ctx->nbr[cf];
        if (code >= 0) continue;
        int row = -1;
        for (int i = 0; i < ctx->n_bc; ++i)
            if (ctx->bc_index[i] == code) { row = i; break; }
        fixed[cf] = row < 0 || ctx->bc_type[row] == 1;
    }
    HostTimer tm("setup_dsa_host");
    // The locality order runs on a second thread while the coefficients are
    // computed.  With the centroids (bte_set_centroids) it is the Hilbert
    // curve through them.  Without, it is the bisection of the coupling
    // pattern, which the topology gives (an interior face with positive area
    // that both cells name); that order is used if the coefficients' own
    // pattern is the same (it always is unless a coefficient is zero).
    const bool by_curve = ctx->centroid.size() == (size_t)3 * n;
    std::vector<int> cm_topo, pre_order;
    if (!by_curve) {
        cm_topo.assign((size_t)n * F, -1);
        for (int c = 0; c < n; ++c)
            for (int f = 0; f < F; ++f) {
                const size_t cf = (size_t)c * F + f;
                const int o = ctx->nbr[cf];
                if (o < 0 || o >= n || !(ctx->area[cf] > 0.0)) continue;
                bool back = false;
                for (int g = 0; g < F; ++g) back |= ctx->nbr[(size_t)o * F + g] == c;
                if (back) cm_topo[cf] = o;
            }
    }
    const int agg_cells = std::max(1, n / (nblk * bte::dsa::AGG));
    std::thread order_thread([&] {
        if (by_curve) bte::hilbert_order(ctx->dim, n, ctx->centroid.data(), pre_order);
        else bte::locality_order(n, F, cm_topo.data(), std::max(8, agg_cells / 2), pre_order);
    });
    bte::DsaCoefficients co;
    bte::dsa_coefficients(ctx->dim, n, F, ctx->nbr.data(), ctx->area.data(), ctx->normal.data(), ctx->volume.data(),
                          ctx->n_dir, ctx->s.data(), ctx->S.data(), ctx->solid_angle, ctx->n_band, ctx->vg.data(),
                          ctx->tau.data(), ctx->Lr.data(), fixed, dsa_beta(), co);
    tm.lap("coefficients");
    order_thread.join();
    tm.lap("locality order (joined)");
    out.n_dirichlet = co.n_dirichlet;
    if (co.n_dirichlet > 0)
        dsa_host_plan(n, F, co.nb.data(), co.W.data(), nblk, out.hp, &pre_order, by_curve ? nullptr : &cm_topo);
}

// ... and the device part.
static bte_status setup_dsa_device(bte_ctx* ctx, DsaSetupHost& h, cudaStream_t st) {
    ctx->dsa_walls = h.n_dirichlet;
    if (h.n_dirichlet > 0) {
        bte_status s = dsa_upload(ctx, h.hp, st);
        if (s != BTE_OK) return s;
        BTE_CUDA(cudaStreamSynchronize(st));
    }
    return BTE_OK;
}

// The wall faces held at a fixed temperature that the low-order operator
// couples to (setup_dsa_host's count, without the coefficients): known
// before its set-up ends, so the solve can start while it runs.
static int dsa_wall_faces(const bte_ctx* ctx) {
    int count = 0;
    for (size_t cf = 0; cf < (size_t)ctx->n * ctx->F; ++cf) {
        const int code = ctx->nbr[cf];
        if (code >= 0 || !(ctx->area[cf] > 0.0)) continue;
        int row = -1;
        for (int i = 0; i < ctx->n_bc; ++i)
            if (ctx->bc_index[i] == code) { row = i; break; }
        count += row < 0 || ctx->bc_type[row] == 1;
    }
    return count;
}

// Face slots the sweep is instantiated for (2 in 1D and 2D, 3 in 3D).
static int sweep_slots(const bte_ctx* ctx) { return std::max(2, std::min(ctx->plan_fm, 4)); }

// Build the sweep plan for every direction from the device's inflow coefficients.
// BTE_LEVEL_ORDER=host builds every direction's level order on the host
// (sweep_order.h) instead of on the device (k_level_order_smem, or
// k_level_order when its state does not fit in shared memory), and
// BTE_LEVEL_ORDER=global takes k_level_order even when it would; the order is
// the same either way.
static bool level_order_on_host() {
    const char* v = std::getenv("BTE_LEVEL_ORDER");
    return v && v[0] == 'h';
}
static bool level_order_global() {
    const char* v = std::getenv("BTE_LEVEL_ORDER");
    return v && v[0] == 'g';
}

static bte_status build_sweep_plan(bte_ctx* ctx) {
    HostTimer tm("build_sweep_plan");
    const int n = ctx->n, F = ctx->F, ND = ctx->n_dir;
    const size_t Np = ctx->Np;
    cudaStream_t st = ctx->stream;
    BTE_CUDA(ctx->lo_mask.alloc((size_t)ND * n));
    bte::k_inflow_mask<<<dim3((n + 255) / 256, ND), 256, 0, st>>>(ctx->d_fc.as<double>(), F, n, Np, ND,
                                                                  ctx->lo_mask.as<uint8_t>());
    BTE_LAUNCHED();
    const auto t_order = std::chrono::steady_clock::now();
    // level order: on the device, one block per direction (each wave sorted
    // in shared memory); a direction with a cycle or a wave wider than the
    // block's frontier buffers is ordered on the host
    BTE_CUDA(ctx->lo_perm.alloc(sizeof(int) * (size_t)ND * n));
    BTE_CUDA(ctx->lo_lvl.alloc(sizeof(int) * (size_t)ND * (n + 1)));
    BTE_CUDA(ctx->lo_small.alloc(sizeof(int) * (2 * (size_t)ND + 1)));
    std::vector<int> small(2 * (size_t)ND + 1, 1);  // nlev[ND], status[ND], fmax
    int* d_small = ctx->lo_small.as<int>();
    // the device order packs a cell index and an edge count into one int
    const bool host_all = level_order_on_host() || F > 4 || n >= (1 << 28);
    if (!host_all) {
        BTE_CUDA(ctx->lo_down.alloc(sizeof(int) * (size_t)ND * n * F));
        const size_t nf = (size_t)n * F;
        bte::k_downstream<<<dim3((unsigned)((nf + 255) / 256), ND), 256, 0, st>>>(
            ctx->lo_mask.as<uint8_t>(), ctx->d_nbr.as<int>(), n, F, ctx->lo_down.as<int>());
        BTE_LAUNCHED();
        int smem_max = 0;
        BTE_CUDA(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device));
        BTE_CUDA(cudaMemsetAsync(d_small + 2 * ND, 0, sizeof(int), st));
        // the whole state in shared memory when it fits (in-degree bytes and
        // two cell bitmaps), else the in-degrees in global memory
        // (and the wave list: up to 8,192 cells, at least 2,048)
        const size_t smem_state = sizeof(unsigned) * (((size_t)n + 3) / 4 + 2 * (((size_t)n + 31) / 32));
        const size_t room = (size_t)smem_max - 1024;
        const int wcap = smem_state < room ? (int)std::min<size_t>({(size_t)8192, (size_t)n, (room - smem_state) / 4}) : 0;
        if (!level_order_global() && wcap >= std::min(n, 2048)) {
            const size_t smem = smem_state + sizeof(int) * (size_t)wcap;
            BTE_CUDA(cudaFuncSetAttribute(bte::k_level_order_smem, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
            bte::k_level_order_smem<<<ND, 1024, smem, st>>>(ctx->lo_mask.as<uint8_t>(), ctx->lo_down.as<int>(), n, F,
                                                            wcap, ctx->lo_perm.as<int>(), ctx->lo_lvl.as<int>(),
                                                            d_small, d_small + ND, d_small + 2 * ND);
        } else {
            // frontier capacity: a power of two, two frontiers in at most 128 KB
            int cap = 1;
            while (cap < n && (size_t)cap * 2 * 2 * sizeof(int) <= std::min<size_t>(128 * 1024, smem_max - 1024))
                cap *= 2;
            const size_t smem = (size_t)2 * cap * sizeof(int);
            BTE_CUDA(ctx->lo_indeg.alloc(sizeof(int) * (size_t)ND * n));
            BTE_CUDA(cudaFuncSetAttribute(bte::k_level_order, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            bte::k_level_order<<<ND, 1024, smem, st>>>(ctx->lo_mask.as<uint8_t>(), ctx->lo_down.as<int>(), n, F, cap,
                                                       ctx->lo_indeg.as<int>(), ctx->lo_perm.as<int>(),
                                                       ctx->lo_lvl.as<int>(), d_small, d_small + ND, d_small + 2 * ND);
        }
        BTE_LAUNCHED();
        BTE_CUDA(cudaMemcpyAsync(small.data(), d_small, sizeof(int) * small.size(), cudaMemcpyDeviceToHost, st));
        BTE_CUDA(cudaStreamSynchronize(st));
    }
    std::vector<int> host_dirs;
    for (int d = 0; d < ND; ++d)
        if (host_all || small[ND + d] != 0) host_dirs.push_back(d);
    std::vector<std::vector<int>> lvl(ND), lag(ND);
    std::vector<char> lag_any(ND, 0);
    int fm_all = host_all ? 0 : small[2 * ND];
    if (!host_dirs.empty()) {
        std::vector<uint8_t> mask((size_t)ND * n);
        BTE_CUDA(cudaMemcpyAsync(mask.data(), ctx->lo_mask.p, mask.size(), cudaMemcpyDeviceToHost, st));
        BTE_CUDA(cudaStreamSynchronize(st));
        std::vector<std::vector<int>> perm(ND);
        std::vector<int> fm_dir(ND, 0);
        const int nth = std::max(1, std::min<int>((int)host_dirs.size(), (int)std::thread::hardware_concurrency()));
        std::vector<std::thread> pool;
        for (int t = 0; t < nth; ++t)
            pool.emplace_back([&, t]() {
                for (size_t k = t; k < host_dirs.size(); k += nth) {
                    const int d = host_dirs[k];
                    bte::level_order(n, F, &mask[(size_t)d * n], ctx->nbr.data(), perm[d], lvl[d], lag[d]);
                    lag_any[d] = std::any_of(lag[d].begin(), lag[d].end(), [](int v) { return v != 0; });
                    int fm = 0;
                    const uint8_t* md = &mask[(size_t)d * n];
                    for (int c = 0; c < n; ++c) fm = std::max(fm, bte::inflow_count(md[c]));
                    fm_dir[d] = fm;
                }
            });
        for (auto& th : pool) th.join();
        for (int d : host_dirs) {
            fm_all = std::max(fm_all, fm_dir[d]);
            BTE_CUDA(cudaMemcpyAsync(ctx->lo_perm.as<int>() + (size_t)d * n, perm[d].data(), sizeof(int) * n,
                                     cudaMemcpyHostToDevice, st));
        }
        BTE_CUDA(cudaStreamSynchronize(st));  // perm[] goes out of scope
    }
    // level starts of the device-ordered directions
    for (int d = 0; d < ND; ++d) {
        if (!lvl[d].empty()) continue;
        lvl[d].resize((size_t)small[d] + 1);
        BTE_CUDA(cudaMemcpyAsync(lvl[d].data(), ctx->lo_lvl.as<int>() + (size_t)d * (n + 1),
                                 sizeof(int) * lvl[d].size(), cudaMemcpyDeviceToHost, st));
    }
    BTE_CUDA(cudaStreamSynchronize(st));
    ctx->ms_last_order = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_order).count();
    ctx->plan_host_dirs = (int)host_dirs.size();
    tm.lap("level order");
    // the sweep's face slots: the largest inflow count of a cell
    ctx->plan_fm = fm_all;
    std::vector<int> h_lvl, h_off(ND + 1, 0);
    int lagged_dirs = 0;
    long long levels = 0;
    for (int d = 0; d < ND; ++d) {
        h_off[d] = (int)h_lvl.size();
        h_lvl.insert(h_lvl.end(), lvl[d].begin(), lvl[d].end());
        levels += (long long)lvl[d].size() - 1;
        lagged_dirs += lag_any[d];
    }
    h_off[ND] = (int)h_lvl.size();
    tm.lap("order arrays");
    // cell -> position from the order on the device; the lagged-edge flags
    // only when some direction has a cycle (none on planar meshes)
    DevBuf d_lag;
    BTE_CUDA(ctx->lo_pos.alloc(sizeof(int) * (size_t)ND * n));
    bte::k_inverse_perm<<<dim3((n + 255) / 256, ND), 256, 0, st>>>(ctx->lo_perm.as<int>(), n, ctx->lo_pos.as<int>());
    BTE_LAUNCHED();
    if (lagged_dirs > 0) {
        std::vector<int> h_lag((size_t)ND * F * n, 0);
        for (int d = 0; d < ND; ++d)
            if (!lag[d].empty()) std::copy(lag[d].begin(), lag[d].end(), h_lag.begin() + (size_t)d * F * n);
        BTE_CUDA(upload(d_lag, h_lag, st));
    }
    BTE_CUDA(upload(ctx->p_lvl, h_lvl, st));
    BTE_CUDA(upload(ctx->p_lvl_off, h_off, st));
    BTE_CUDA(ctx->p_cell.alloc(sizeof(int) * ND * n));
    BTE_CUDA(ctx->p_dg.alloc(sizeof(double) * ND * n));
    BTE_CUDA(ctx->p_vo.alloc(sizeof(double) * ND * n));
    BTE_CUDA(ctx->p_nb.alloc(sizeof(int) * ND * F * n));
    BTE_CUDA(ctx->p_fc.alloc(sizeof(double) * ND * F * n));
    BTE_CUDA(ctx->p_bidx.alloc(sizeof(int) * ND * n));
    BTE_CUDA(ctx->d_bsum.alloc(sizeof(double) * (size_t)ctx->nbb * ND * std::max(ctx->nbcell, 1)));
    BTE_CUDA(ctx->p_binvd.alloc(sizeof(double) * (size_t)ctx->n_band * ND * std::max(ctx->nbcell, 1)));
    if (ctx->nbcell > 0) {
        bte::k_bound_invd<<<dim3((ctx->nbcell + 127) / 128, ND), 128, 0, st>>>(
            ctx->d_bcell.as<int>(), ctx->nbcell, ctx->d_kb.as<double>(), ctx->d_dg.as<double>(),
            ctx->d_vo.as<double>(), ctx->n_band, ND, Np, ctx->p_binvd.as<double>());
        BTE_LAUNCHED();
    }
    bte::k_sweep_layout<<<dim3((n + 255) / 256, ND), 256, 0, st>>>(
        ctx->lo_perm.as<int>(), ctx->lo_pos.as<int>(), lagged_dirs > 0 ? d_lag.as<int>() : nullptr, ctx->d_dg.as<double>(), ctx->d_vo.as<double>(), ctx->d_fc.as<double>(),
        ctx->d_nbr.as<int>(), ctx->d_bidx.as<int>(), F, n, Np, ND, ctx->p_cell.as<int>(), ctx->p_bidx.as<int>(),
        ctx->p_dg.as<double>(), ctx->p_vo.as<double>(), ctx->p_nb.as<int>(), ctx->p_fc.as<double>());
    BTE_LAUNCHED();
    ctx->n2 = (n + 1) & ~1;
    tm.lap("layout");
    BTE_CUDA(ctx->p_voi.alloc(sizeof(double) * ctx->n_band * ND * (size_t)ctx->n2));
    BTE_CUDA(ctx->p_kinv.alloc(sizeof(double) * ctx->n_band * ND * (size_t)ctx->n2));
    {
        bte::SweepPlan sp{ctx->p_cell.as<int>(), ctx->p_bidx.as<int>(), ctx->p_dg.as<double>(), ctx->p_vo.as<double>(), ctx->p_nb.as<int>(),
                          ctx->p_fc.as<double>(), ctx->p_lvl.as<int>(), ctx->p_lvl_off.as<int>(), n, F, ctx->n2};
        bte::k_sweep_invd<<<dim3((n + 255) / 256, ND), 256, 0, st>>>(sp, ctx->d_kb.as<double>(), ctx->n_band, ND,
                                                                     ctx->p_voi.as<double>(),
                                                                     ctx->p_kinv.as<double>());
        BTE_LAUNCHED();
    }
    tm.lap("per-system diagonal");
    // staged sweep: one record per (direction, position), the batch's
    // level-ordered right-hand side, the error flag of its bounded waits
    {
        const int fmx = sweep_slots(ctx);
        const int rb = fmx == 2 ? bte::SweepRecLayout<2>::bytes
                                : fmx == 3 ? bte::SweepRecLayout<3>::bytes : bte::SweepRecLayout<4>::bytes;
        BTE_CUDA(ctx->p_rec.alloc((size_t)rb * ND * n));
        const dim3 g((n + 255) / 256, ND);
        if (fmx == 2)
            bte::k_sweep_records<2><<<g, 256, 0, st>>>(ctx->p_cell.as<int>(), ctx->p_bidx.as<int>(), ctx->p_nb.as<int>(),
                                                       ctx->p_fc.as<double>(), n, F, ND,
                                                       ctx->p_rec.as<unsigned char>());
        else if (fmx == 3)
            bte::k_sweep_records<3><<<g, 256, 0, st>>>(ctx->p_cell.as<int>(), ctx->p_bidx.as<int>(), ctx->p_nb.as<int>(),
                                                       ctx->p_fc.as<double>(), n, F, ND,
                                                       ctx->p_rec.as<unsigned char>());
        else
            bte::k_sweep_records<4><<<g, 256, 0, st>>>(ctx->p_cell.as<int>(), ctx->p_bidx.as<int>(), ctx->p_nb.as<int>(),
                                                       ctx->p_fc.as<double>(), n, F, ND,
                                                       ctx->p_rec.as<unsigned char>());
        BTE_LAUNCHED();
        BTE_CUDA(ctx->d_sweep_err.alloc(sizeof(int)));
        BTE_CUDA(cudaMemsetAsync(ctx->d_sweep_err.p, 0, sizeof(int), st));
        int smem_max = 0;
        BTE_CUDA(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device));
        BTE_CUDA(cudaFuncSetAttribute(bte::k_sweep_staged<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_max));
        BTE_CUDA(cudaFuncSetAttribute(bte::k_sweep_staged<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_max));
        BTE_CUDA(cudaFuncSetAttribute(bte::k_sweep_staged<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_max));
        ctx->plan_lvl = h_lvl;
        ctx->plan_lvl_off = h_off;
        ctx->stage_lists.clear();
    }
    tm.lap("records");
    BTE_CUDA(cudaStreamSynchronize(st));  // d_perm / d_lag go out of scope
    tm.lap("sync");
    ctx->sweep_tuned = false;
    ctx->sweep_tune_cand.clear();
    ctx->sweep_tune_ms.clear();
    ctx->plan_lagged_dirs = lagged_dirs;
    ctx->sweep_margin = false;  // decided with the launch shape on the first sweep
    BTE_CUDA(ctx->d_spart.alloc(sizeof(double) * ND * ctx->n_band));
    ctx->plan_levels = levels;
    ctx->plan_ready = true;
    return BTE_OK;
}

// Launch a kernel, optionally bracketed by profiling events.
#define BTE_LAUNCH(kind, iter, bytes_fixed, bytes_per_active, ...)                      \
    do {                                                                                \
        size_t _slot = 0;                                                               \
        BTE_CUDA(prof_begin(ctx, &_slot));                                              \
        __VA_ARGS__;                                                                    \
        BTE_LAUNCHED();                                                                 \
        BTE_CUDA(prof_end(ctx, _slot, (kind), (iter), (bytes_fixed), (bytes_per_active))); \
    } while (0)

// Solve all systems of one batch (bands b0 .. b0+nbb-1, every direction) with
// the plain FP64 BiCGSTAB; x lands in e_curr.

// BTE_KRYLOV=persistent runs the Krylov forms' BiCGSTAB as one persistent
// launch per batch (k_bicg_persistent: one block per system) instead of one
// launch per phase with the host checking every kGroup iterations; x is the
// same to the bit either way.  The phase kernels stay the default: they
// spread every phase over all chunks of all systems, and on GB300 the
// persistent form measured 1.3x (square20k) to 3x (square100k) slower per
// outer iteration -- its per-system parallelism is one block.
static bool krylov_persistent() {
    const char* v = std::getenv("BTE_KRYLOV");
    return v && v[0] == 'p' && v[1] == 'e';
}

static bte_status solve_batch_plain(bte_ctx* ctx, int b0, int nbb, const bte_options& o, bte_report& rep) {
    {
        const size_t bytes = sizeof(double) * (size_t)ctx->nbb * ctx->n_dir * ctx->Np;
        for (DevBuf* b : {&ctx->w_r, &ctx->w_rw, &ctx->w_p, &ctx->w_ph, &ctx->w_q, &ctx->w_z, &ctx->w_t, &ctx->w_b,
                          &ctx->w_invD, &ctx->w_xb})
            BTE_CUDA(b->alloc(bytes));
    }
    cudaStream_t st = ctx->stream;
    const int S = nbb * ctx->n_dir;
    const double N = ctx->n, w = sizeof(double);
    // algorithmic HBM bytes: vector passes per active system, plus the
    // per-direction geometry of an SpMV read once per direction in the launch
    const double geo = N * ((ctx->F + 2) * w + ctx->F * 4.0) * std::min(S, ctx->n_dir);
    bte::FaceFluxOp op{ctx->d_dg.as<double>(), ctx->d_vo.as<double>(), ctx->d_fc.as<double>(),
                       ctx->d_nb.as<int>(), ctx->d_kb.as<double>(), ctx->e_curr, ctx->F, nbb, b0,
                       ctx->n_dir, ctx->Np};
    bte::Boundary bd{ctx->d_bptr.as<int>(), ctx->d_bf_cell.as<int>(), ctx->d_bf_kind.as<int>(),
                     ctx->d_bf_bc.as<int>(), ctx->d_bf_diff.as<int>(), ctx->d_cin.as<double>(),
                     ctx->d_eiso.as<double>(), ctx->d_mirror.as<int>(), ctx->d_ediff.as<double>(),
                     ctx->nbf, std::max(ctx->n_bc, 1)};
    dim3 grid(ctx->nchunk, S);
    BTE_LAUNCH(KK_RHS, -1, S * N * 2 * w + geo / 2, 0,
               bte::k_rhs<<<grid, bte::THREADS, 0, st>>>(
                   op, bte::RhsSrc{bd, ctx->d_ebar.as<double>(), ctx->e_prev, ctx->n_dir, ctx->Np},
                   ctx->w_b.as<double>(), ctx->n));

    const int maxit = o.inner_maxit;
    // The reference stops a system at maxit and keeps its last iterate
    // (cycles = 1, no best-iterate copy).  With plain_cycles = k > 1 a system
    // not converged after maxit iterations goes on up to k x maxit and keeps
    // its best iterate if it still has not.
    const int cycles = std::max(1, o.plain_cycles);
    const int total = maxit * cycles;
    if (ctx->active_cap < total + 2) {
        BTE_CUDA(ctx->s_active.alloc(sizeof(int) * (total + 2)));
        ctx->active_cap = total + 2;
    }
    BTE_CUDA(cudaMemsetAsync(ctx->s_active.p, 0, sizeof(int) * (total + 2), st));
    bte::BicgState bs{ctx->s_done.as<int>(), ctx->s_iters.as<int>(), ctx->s_flagA.as<int>(), ctx->s_flagB.as<int>(),
                      ctx->s_rho.as<double>(), ctx->s_alpha.as<double>(), ctx->s_omega.as<double>(),
                      ctx->s_nrmr.as<double>(), ctx->s_nrm0.as<double>(), ctx->s_best.as<double>(),
                      ctx->s_part.as<double>(), ctx->s_active.as<int>(), S, ctx->nchunk, o.inner_tol, maxit};
    bte::BicgVecs<double> v{ctx->w_r.as<double>(), ctx->w_rw.as<double>(), ctx->w_p.as<double>(),
                            ctx->w_ph.as<double>(), ctx->w_q.as<double>(), ctx->w_z.as<double>(),
                            ctx->w_t.as<double>(), ctx->w_b.as<double>(), ctx->w_invD.as<double>(), ctx->Np};
    if (cycles > 1) {
        v.xb = ctx->w_xb.as<double>();  // the best iterate is kept and returned
        bs.cycles = cycles;
        bs.track_from = maxit / 2;  // systems converging before that never copy x
    }
    BTE_LAUNCH(KK_INIT, -1, S * N * 7 * w + geo / 2, 0, bte::k_bicg_init<<<grid, bte::THREADS, 0, st>>>(op, v, bs));
    BTE_LAUNCH(KK_INIT, -1, 0, 0, bte::k_bicg_init_scalars<<<(S + 127) / 128, 128, 0, st>>>(bs, nullptr));
    int i = 1;
    if (krylov_persistent()) {
        // every iteration of every system in one launch: 25 N w per active
        // system-iteration (the five phases' vector passes) + the geometry
        BTE_LAUNCH(KK_BICG, -2, 0, N * 25 * w, bte::k_bicg_persistent<<<S, bte::THREADS, 0, st>>>(op, v, bs, total + 1));
    }
    for (; !krylov_persistent();) {
        int last = i;
        for (int g = 0; g < kGroup && i <= total + 1; ++g, ++i) {
            BTE_LAUNCH(KK_P, i, 0, N * 6 * w, bte::k_bicg_p<<<grid, bte::THREADS, 0, st>>>(op, v, bs, i));
            last = i;
            if (i > total) break;
            BTE_LAUNCH(KK_SPMV1, i, geo, N * 3 * w, bte::k_bicg_spmv1<<<grid, bte::THREADS, 0, st>>>(op, v, bs, i));
            BTE_LAUNCH(KK_S, i, 0, N * 5 * w, bte::k_bicg_s<<<grid, bte::THREADS, 0, st>>>(op, v, bs, i));
            BTE_LAUNCH(KK_SPMV2, i, geo, N * 3 * w, bte::k_bicg_spmv2<<<grid, bte::THREADS, 0, st>>>(op, v, bs, i));
            BTE_LAUNCH(KK_X, i, 0, N * 8 * w, bte::k_bicg_x<<<grid, bte::THREADS, 0, st>>>(op, v, bs, i));
        }
        BTE_CUDA(cudaMemcpyAsync(ctx->h_pinned_i, ctx->s_active.as<int>() + last, sizeof(int),
                                 cudaMemcpyDeviceToHost, st));
        BTE_CUDA(cudaStreamSynchronize(st));
        if (ctx->h_pinned_i[0] == 0 || last > total) break;
        if (i > total + 1) break;
    }
    BTE_CUDA(cudaMemcpyAsync(ctx->h_done.data(), ctx->s_done.p, sizeof(int) * S, cudaMemcpyDeviceToHost, st));
    BTE_CUDA(cudaMemcpyAsync(ctx->h_iters.data(), ctx->s_iters.p, sizeof(int) * S, cudaMemcpyDeviceToHost, st));
    if (ctx->profile) {
        ctx->h_active.resize(total + 2);
        BTE_CUDA(cudaMemcpyAsync(ctx->h_active.data(), ctx->s_active.p, sizeof(int) * (total + 2),
                                 cudaMemcpyDeviceToHost, st));
    }
    BTE_CUDA(cudaStreamSynchronize(st));
    if (ctx->profile) prof_resolve(ctx, ctx->h_active.data(), total + 2);
    for (int y = 0; y < S; ++y) {
        rep.inner_iterations += ctx->h_iters[y];
        if (ctx->h_done[y] == 3 || ctx->h_done[y] == 0) ++rep.inner_unconverged;
    }
    rep.inner_solves += S;
    return BTE_OK;
}

// Mixed form for one batch: x starts from the previous outer iterate; each
// refinement cycle computes the FP64 residual, stops the systems that meet
// ||b - A x|| <= inner_tol ||b||, solves A dx = r for the others with FP32
// BiCGSTAB (relative tolerance 1e-4) and adds dx in FP64.
static bte_status solve_batch_mixed(bte_ctx* ctx, int b0, int nbb, const bte_options& o, bte_report& rep) {
    BTE_CUDA(ctx->w_b.alloc(sizeof(double) * (size_t)ctx->nbb * ctx->n_dir * ctx->Np));
    cudaStream_t st = ctx->stream;
    const int S = nbb * ctx->n_dir;
    const double N = ctx->n;
    bte::FaceFluxOp op{ctx->d_dg.as<double>(), ctx->d_vo.as<double>(), ctx->d_fc.as<double>(),
                       ctx->d_nb.as<int>(), ctx->d_kb.as<double>(), ctx->e_curr, ctx->F, nbb, b0,
                       ctx->n_dir, ctx->Np};
    bte::FaceFluxOp32 op32{ctx->d_dg32.as<float>(), ctx->d_vo32.as<float>(), ctx->d_fc32.as<float>(),
                           ctx->d_nb.as<int>(), ctx->d_kb32.as<float>(), ctx->x_dx.as<float>(), ctx->F, nbb, b0,
                           ctx->n_dir, ctx->Np};
    bte::Boundary bd{ctx->d_bptr.as<int>(), ctx->d_bf_cell.as<int>(), ctx->d_bf_kind.as<int>(),
                     ctx->d_bf_bc.as<int>(), ctx->d_bf_diff.as<int>(), ctx->d_cin.as<double>(),
                     ctx->d_eiso.as<double>(), ctx->d_mirror.as<int>(), ctx->d_ediff.as<double>(),
                     ctx->nbf, std::max(ctx->n_bc, 1)};
    const double geo = N * ((ctx->F + 2) * 8.0 + ctx->F * 4.0) * std::min(S, ctx->n_dir);
    const double geo32 = N * ((ctx->F + 2) * 4.0 + ctx->F * 4.0) * std::min(S, ctx->n_dir);
    dim3 grid(ctx->nchunk, S);
    BTE_LAUNCH(KK_RHS, -1, S * N * 16.0 + geo / 2, 0,
               bte::k_rhs<<<grid, bte::THREADS, 0, st>>>(
                   op, bte::RhsSrc{bd, ctx->d_ebar.as<double>(), ctx->e_prev, ctx->n_dir, ctx->Np},
                   ctx->w_b.as<double>(), ctx->n));
    BTE_LAUNCH(KK_INIT, -1, S * N * 16.0, 0, bte::k_mixed_start<<<grid, bte::THREADS, 0, st>>>(op, ctx->e_prev));
    const int maxit = o.inner_maxit;
    if (ctx->active_cap < maxit + 2) {
        BTE_CUDA(ctx->s_active.alloc(sizeof(int) * (maxit + 2)));
        ctx->active_cap = maxit + 2;
    }
    bte::BicgState bs{ctx->s_done.as<int>(), ctx->s_iters.as<int>(), ctx->s_flagA.as<int>(), ctx->s_flagB.as<int>(),
                      ctx->s_rho.as<double>(), ctx->s_alpha.as<double>(), ctx->s_omega.as<double>(),
                      ctx->s_nrmr.as<double>(), ctx->s_nrm0.as<double>(), ctx->s_best.as<double>(),
                      ctx->s_part.as<double>(), ctx->s_active.as<int>(), S, ctx->nchunk, 1e-4, maxit};
    bte::BicgVecs<float> v{ctx->x_r.as<float>(), ctx->x_rw.as<float>(), ctx->x_p.as<float>(),
                           ctx->x_ph.as<float>(), ctx->x_q.as<float>(), ctx->x_z.as<float>(),
                           ctx->x_t.as<float>(), ctx->x_b.as<float>(), ctx->x_invD.as<float>(), ctx->Np};
    v.xb = ctx->x_xb.as<float>();
    const double w = 4.0;
    const int max_cycles = 30;
    int cycle = 0;
    for (; cycle < max_cycles; ++cycle) {
        BTE_CUDA(cudaMemsetAsync(ctx->m_active.p, 0, sizeof(int), st));
        BTE_LAUNCH(KK_SWEEP_RES, -1, S * N * (8.0 * 2 + 4.0) + geo, 0,
                   bte::k_mixed_residual<<<grid, bte::THREADS, 0, st>>>(op, ctx->w_b.as<double>(),
                                                                        ctx->d_kappa.as<double>(), ctx->x_b.as<float>(),
                                                                        ctx->m_part.as<double>(), ctx->nchunk, ctx->n));
        bte::k_mixed_check<<<(S + 127) / 128, 128, 0, st>>>(ctx->m_part.as<double>(), S, ctx->nchunk, o.inner_tol,
                                                             ctx->m_skip.as<int>(), ctx->m_active.as<int>());
        BTE_LAUNCHED();
        BTE_CUDA(cudaMemcpyAsync(ctx->h_pinned_i + 1, ctx->m_active.p, sizeof(int), cudaMemcpyDeviceToHost, st));
        BTE_CUDA(cudaStreamSynchronize(st));
        if (ctx->h_pinned_i[1] == 0) break;
        BTE_CUDA(cudaMemsetAsync(ctx->s_active.p, 0, sizeof(int) * (maxit + 2), st));
        BTE_LAUNCH(KK_INIT, -1, S * N * 7 * w + geo32 / 2, 0,
                   bte::k_bicg_init<<<grid, bte::THREADS, 0, st>>>(op32, v, bs));
        BTE_LAUNCH(KK_INIT, -1, 0, 0,
                   bte::k_bicg_init_scalars<<<(S + 127) / 128, 128, 0, st>>>(bs, ctx->m_skip.as<int>()));
        int i = 1;
        if (krylov_persistent())
            BTE_LAUNCH(KK_BICG, -2, 0, N * 25 * w,
                       bte::k_bicg_persistent<<<S, bte::THREADS, 0, st>>>(op32, v, bs, maxit + 1));
        for (; !krylov_persistent();) {
            int last = i;
            for (int g = 0; g < kGroup && i <= maxit + 1; ++g, ++i) {
                BTE_LAUNCH(KK_P, i, 0, N * 6 * w, bte::k_bicg_p<<<grid, bte::THREADS, 0, st>>>(op32, v, bs, i));
                last = i;
                if (i > maxit) break;
                BTE_LAUNCH(KK_SPMV1, i, geo32, N * 3 * w,
                           bte::k_bicg_spmv1<<<grid, bte::THREADS, 0, st>>>(op32, v, bs, i));
                BTE_LAUNCH(KK_S, i, 0, N * 5 * w, bte::k_bicg_s<<<grid, bte::THREADS, 0, st>>>(op32, v, bs, i));
                BTE_LAUNCH(KK_SPMV2, i, geo32, N * 3 * w,
                           bte::k_bicg_spmv2<<<grid, bte::THREADS, 0, st>>>(op32, v, bs, i));
                BTE_LAUNCH(KK_X, i, 0, N * 8 * w, bte::k_bicg_x<<<grid, bte::THREADS, 0, st>>>(op32, v, bs, i));
            }
            BTE_CUDA(cudaMemcpyAsync(ctx->h_pinned_i, ctx->s_active.as<int>() + last, sizeof(int),
                                     cudaMemcpyDeviceToHost, st));
            BTE_CUDA(cudaStreamSynchronize(st));
            if (ctx->h_pinned_i[0] == 0 || last > maxit || i > maxit + 1) break;
        }
        if (ctx->profile) {
            ctx->h_active.resize(maxit + 2);
            BTE_CUDA(cudaMemcpyAsync(ctx->h_active.data(), ctx->s_active.p, sizeof(int) * (maxit + 2),
                                     cudaMemcpyDeviceToHost, st));
            BTE_CUDA(cudaStreamSynchronize(st));
            prof_resolve(ctx, ctx->h_active.data(), maxit + 2);
        }
        BTE_LAUNCH(KK_X, -1, S * N * (8.0 * 2 + 4.0), 0,
                   bte::k_mixed_update<<<grid, bte::THREADS, 0, st>>>(op, ctx->x_dx.as<float>(),
                                                                      ctx->m_skip.as<int>()));
        BTE_CUDA(cudaMemcpyAsync(ctx->h_iters.data(), ctx->s_iters.p, sizeof(int) * S, cudaMemcpyDeviceToHost, st));
        BTE_CUDA(cudaStreamSynchronize(st));
        for (int y = 0; y < S; ++y) rep.inner_iterations += ctx->h_iters[y];
        ++rep.refinements;
    }
    if (cycle == max_cycles) rep.inner_unconverged += ctx->h_pinned_i[1];
    if (ctx->profile) {
        BTE_CUDA(cudaStreamSynchronize(st));
        prof_resolve(ctx, nullptr, 0);
    }
    rep.inner_solves += S;
    return BTE_OK;
}

// Launch shapes chosen by the sweep's autotuner, per (device, cells, faces,
// directions, bands per batch, levels, margin restriction).
using SweepTuneKey = std::tuple<int, int, int, int, int, long long, int, int, int>;

// BTE_SWEEP_MARGIN=1 (in the sweep) or 0 (in k_reduce) fixes where the margin
// of an acyclic plan is summed instead of timing both (the temperatures are
// the same to the bit either way; the margins differ by summation order).
static int sweep_margin_restriction() {
    const char* v = std::getenv("BTE_SWEEP_MARGIN");
    if (!v || !*v) return -1;
    return v[0] == '0' ? 0 : v[0] == '1' ? 1 : -1;
}
// BTE_SWEEP_KERNEL=level (k_sweep), split (k_sweep over levels split into
// slices of one position per thread) or staged (k_sweep_staged) restricts the
// autotuner to one sweep kernel (x is the same to the bit either way).
static int sweep_kernel_restriction() {
    const char* v = std::getenv("BTE_SWEEP_KERNEL");
    if (!v || !*v) return -1;
    return v[0] == 'l' ? 0 : v[0] == 's' && v[1] == 't' ? 1 : v[0] == 's' && v[1] == 'p' ? 2 : -1;
}
// BTE_SWEEP_SHAPE=G,T restricts the autotuner to G bands and T threads per
// block (a test of a particular shape, e.g. stages narrower than a level);
// returns G * 10000 + T, or -1.
static int sweep_shape_restriction() {
    const char* v = std::getenv("BTE_SWEEP_SHAPE");
    int g = 0, t = 0;
    if (!v || std::sscanf(v, "%d,%d", &g, &t) != 2 || g <= 0 || t <= 0) return -1;
    return g * 10000 + t;
}
static std::mutex g_sweep_tune_mutex;
static std::map<SweepTuneKey, SweepShape> g_sweep_tune;

// Shared-memory ring of k_sweep: W (a power of two) positions per band, 32 KB per block.
static int sweep_ring(int G) {
    int w = 4096;
    while (w > 256 && w * std::max(G, 1) > 4096) w >>= 1;
    return w;
}

// Candidates of the autotuner for batches of nbb bands: (bands per block,
// threads); k_sweep takes at most 128 threads.
// Shared memory of a staged candidate (face slots fm).
static size_t staged_smem(int fm, int cap, int G, int W) {
    return fm == 2 ? bte::staged_smem_bytes<2>(cap, G, W)
                   : fm == 3 ? bte::staged_smem_bytes<3>(cap, G, W) : bte::staged_smem_bytes<4>(cap, G, W);
}

// Candidates of the autotuner for batches of nbb bands: k_sweep (bands per
// block, threads; at most 128 threads) over the levels as they are and over
// the levels split into slices of one position per thread (a thread's items
// are then all loaded a level ahead; a wider level costs one more barrier per
// slice instead), and k_sweep_staged (at most 256 threads; two rounds of the
// block's positions per stage, a ring of 2048 / G positions per band).
static std::vector<SweepShape> sweep_candidates(const bte_ctx* ctx, int nbb, int only_kernel, int only_margin,
                                                int only_shape) {
    static const int cand[][2] = {{1, 64}, {1, 128}, {2, 64}, {2, 128}, {4, 64}, {4, 128}, {8, 128}, {16, 128}};
    static const int staged[][2] = {{1, 128}, {1, 256}, {2, 128}, {2, 256}, {4, 64},
                                    {4, 128}, {4, 256}, {8, 256}};
    std::vector<SweepShape> out;
    for (int split = 0; split < 2; ++split)
        for (const auto& c : cand) {
            if (only_kernel == 1 || only_kernel == (split ? 0 : 2)) break;
            if (only_shape >= 0 && only_shape != c[0] * 10000 + c[1]) continue;
            // split levels only in the 128-thread shapes of up to 4 bands (the
            // others were never faster unsplit)
            if (split && only_shape < 0 && (c[1] != 128 || c[0] > 4)) continue;
            SweepShape sh;
            sh.G = std::max(1, std::min(c[0], nbb));
            sh.threads = c[1];
            sh.W = sweep_ring(sh.G);
            sh.smem = sizeof(double) * (size_t)sh.G * sh.W;
            if (split) {
                int gp = 1;
                while (gp < sh.G) gp <<= 1;
                sh.split = true;
                sh.cap = sh.threads / gp;
            }
            bool dup = false;
            for (const SweepShape& o : out)
                dup |= !o.staged && o.split == sh.split && o.G == sh.G && o.threads == sh.threads;
            if (!dup) out.push_back(sh);
        }
    int smem_max = 0;
    cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
    for (const auto& c : staged) {
        // the staged kernel leaves the margin to k_reduce
        if ((only_kernel >= 0 && only_kernel != 1) || only_margin == 1) break;
        if (only_shape >= 0 && only_shape != c[0] * 10000 + c[1]) continue;
        SweepShape sh;
        sh.staged = true;
        sh.G = std::max(1, std::min(c[0], nbb));
        sh.threads = c[1];
        int gp = 1;
        while (gp < sh.G) gp <<= 1;
        sh.cap = 2 * (sh.threads / gp);
        sh.W = std::max(256, 2048 / gp);
        sh.smem = staged_smem(sweep_slots(ctx), sh.cap, sh.G, sh.W);
        if (sh.smem > (size_t)smem_max) continue;
        bool dup = false;
        for (const SweepShape& o : out) dup |= o.staged && o.G == sh.G && o.threads == sh.threads;
        if (!dup) out.push_back(sh);
    }
    return out;
}

// Stage bounds for stages of at most cap positions (built once per width).
static bte_status stage_list(bte_ctx* ctx, int cap, const StageList** out) {
    auto it = ctx->stage_lists.find(cap);
    if (it == ctx->stage_lists.end()) {
        std::vector<int> stages, off(ctx->n_dir + 1, 0);
        for (int d = 0; d < ctx->n_dir; ++d) {
            off[d] = (int)stages.size();
            const int l0 = ctx->plan_lvl_off[d], l1 = ctx->plan_lvl_off[d + 1];  // level starts, then n
            for (int l = l0; l + 1 < l1; ++l)
                for (int j = ctx->plan_lvl[l]; j < ctx->plan_lvl[l + 1]; j += cap) stages.push_back(j);
            stages.push_back(ctx->n);
        }
        off[ctx->n_dir] = (int)stages.size();
        auto sl = std::make_unique<StageList>();
        BTE_CUDA(upload(sl->stages, stages, ctx->stream));
        BTE_CUDA(upload(sl->off, off, ctx->stream));
        it = ctx->stage_lists.emplace(cap, std::move(sl)).first;
    }
    *out = it->second.get();
    return BTE_OK;
}

// One sweep of bands b0 .. b0+nbb-1 in every direction with shape sh, for the
// plan's face slots (2 in 1D and 2D, 3 in 3D).
template <bool MARGIN>
static void launch_sweep(const bte_ctx* ctx, const SweepShape& sh, int nbb, int b0, cudaStream_t st,
                         const bte::SweepPlan& sp, const bte::SweepSrc& src, int first_sweep, double* mpart) {
    const dim3 grid((nbb + sh.G - 1) / sh.G, ctx->n_dir);
    const double* voi = ctx->p_voi.as<double>();
    const double* kinv = ctx->p_kinv.as<double>();
    const int fm = sweep_slots(ctx);
    if (sh.staged) {  // MARGIN is false here: the staged kernel leaves the margin to k_reduce
        const StageList* sl = ctx->stage_lists.find(sh.cap)->second.get();
        const bte::StagedPlan pl{ctx->p_rec.as<unsigned char>(), sl->stages.as<int>(), sl->off.as<int>(),
                                 ctx->p_cell.as<int>(), ctx->n, ctx->n2, sh.cap};
#define BTE_STAGED_FM(FM)                                                                                          \
    bte::k_sweep_staged<FM><<<grid, sh.threads, sh.smem, st>>>(pl, kinv, voi, src, src.x_old, ctx->e_curr,          \
                                                               first_sweep, sh.G, sh.W, nbb, b0, ctx->n_dir,        \
                                                               ctx->Np, ctx->d_sweep_err.as<int>())
        if (fm == 2) BTE_STAGED_FM(2);
        else if (fm == 3) BTE_STAGED_FM(3);
        else BTE_STAGED_FM(4);
#undef BTE_STAGED_FM
        return;
    }
    bte::SweepPlan spl = sp;
    if (sh.split) {  // the same kernel over the levels split into slices of cap positions
        const StageList* sl = ctx->stage_lists.find(sh.cap)->second.get();
        spl.lvl = sl->stages.as<int>();
        spl.lvl_off = sl->off.as<int>();
    }
#define BTE_SWEEP_FM(FM)                                                                                          \
    bte::k_sweep<MARGIN, FM><<<grid, sh.threads, sh.smem, st>>>(spl, voi, kinv, src, ctx->e_curr, first_sweep, sh.G, \
                                                                sh.W, nbb, b0, ctx->n_band, ctx->n_dir, ctx->Np, mpart)
    if (fm == 2) BTE_SWEEP_FM(2);
    else if (fm == 3) BTE_SWEEP_FM(3);
    else BTE_SWEEP_FM(4);
#undef BTE_SWEEP_FM
}

// Solve all systems of one batch by upwind sweeps (exact in one sweep when no
// edge is lagged; otherwise Gauss-Seidel sweeps until ||R - A x|| <= inner_tol ||R||).
static bte_status solve_batch_sweep(bte_ctx* ctx, int b0, int nbb, const bte_options& o, bte_report& rep) {
    cudaStream_t st = ctx->stream;
    const int S = nbb * ctx->n_dir;
    const double N = ctx->n, w = sizeof(double);
    bte::FaceFluxOp op{ctx->d_dg.as<double>(), ctx->d_vo.as<double>(), ctx->d_fc.as<double>(),
                       ctx->d_nb.as<int>(), ctx->d_kb.as<double>(), ctx->e_curr, ctx->F, nbb, b0,
                       ctx->n_dir, ctx->Np};
    bte::Boundary bd{ctx->d_bptr.as<int>(), ctx->d_bf_cell.as<int>(), ctx->d_bf_kind.as<int>(),
                     ctx->d_bf_bc.as<int>(), ctx->d_bf_diff.as<int>(), ctx->d_cin.as<double>(),
                     ctx->d_eiso.as<double>(), ctx->d_mirror.as<int>(), ctx->d_ediff.as<double>(),
                     ctx->nbf, std::max(ctx->n_bc, 1)};
    const double geo = N * ((ctx->F + 2) * w + ctx->F * 4.0) * ctx->n_dir;
    dim3 grid(ctx->nchunk, S);
    const bte::RhsSrc src{bd, ctx->d_ebar.as<double>(), ctx->e_prev, ctx->n_dir, ctx->Np};
    if (ctx->nbcell > 0) {
        BTE_LAUNCH(KK_RHS, -1, (double)S * ctx->nbcell * 2 * w, 0,
                   bte::k_bound_rhs<<<dim3((ctx->nbcell + 127) / 128, S), 128, 0, st>>>(
                       src, ctx->d_bcell.as<int>(), ctx->nbcell, ctx->d_kb.as<double>(), ctx->p_binvd.as<double>(),
                       nbb, b0, ctx->d_bsum.as<double>()));
    }
    const bte::SweepSrc ssrc{ctx->d_ebar.as<double>(), ctx->d_bsum.as<double>(), ctx->e_prev, ctx->nbcell};
    bte::SweepPlan sp{ctx->p_cell.as<int>(), ctx->p_bidx.as<int>(), ctx->p_dg.as<double>(), ctx->p_vo.as<double>(), ctx->p_nb.as<int>(),
                      ctx->p_fc.as<double>(), ctx->p_lvl.as<int>(), ctx->p_lvl_off.as<int>(), ctx->n, ctx->F,
                      ctx->n2};
    // launch-shape autotuning on the first sweep of this plan (each candidate
    // computes the same x from the same inputs); the choice is kept per
    // process for the same device and plan shape, so a new context on the
    // same mesh does not time the candidates again
    const int only_margin = sweep_margin_restriction();
    const int only_kernel = sweep_kernel_restriction();
    const int only_shape = sweep_shape_restriction();
    const SweepTuneKey tkey{ctx->device, ctx->n, ctx->F, ctx->n_dir, nbb, ctx->plan_levels, only_margin, only_kernel,
                            only_shape};
    if (!ctx->sweep_tuned) {
        std::lock_guard<std::mutex> lock(g_sweep_tune_mutex);
        auto hit = g_sweep_tune.find(tkey);
        if (hit != g_sweep_tune.end()) {
            ctx->sweep_shape = hit->second;
            ctx->sweep_tuned = true;
        }
    }
    if (!ctx->sweep_tuned) {
        const std::vector<SweepShape> cand = sweep_candidates(ctx, nbb, only_kernel, only_margin, only_shape);
        if (cand.empty())
            return fail(ctx, BTE_ERR_INVALID_ARGUMENT,
                        "sweep: no launch shape left by BTE_SWEEP_KERNEL / BTE_SWEEP_SHAPE / BTE_SWEEP_MARGIN");
        ctx->sweep_tune_cand = cand;
        ctx->sweep_tune_ms.assign(cand.size(), 0.f);
        cudaEvent_t e0, e1;
        BTE_CUDA(cudaEventCreate(&e0));
        BTE_CUDA(cudaEventCreate(&e1));
        float best = 1e30f;
        for (size_t k = 0; k < cand.size(); ++k) {
            if (cand[k].staged || cand[k].split) {
                const StageList* sl = nullptr;
                bte_status s2 = stage_list(ctx, cand[k].cap, &sl);
                if (s2 != BTE_OK) return s2;
            }
            BTE_CUDA(cudaEventRecord(e0, st));
            launch_sweep<false>(ctx, cand[k], nbb, b0, st, sp, ssrc, 1, nullptr);
            BTE_LAUNCHED();
            BTE_CUDA(cudaEventRecord(e1, st));
            BTE_CUDA(cudaEventSynchronize(e1));
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            ctx->sweep_tune_ms[k] = ms;
            if (ms < best) { best = ms; ctx->sweep_shape = cand[k]; }
        }
        // where an acyclic plan sums the margin: in the sweep (one more load
        // and two FP64 operations per cell-system, k_reduce<false>) or in
        // k_reduce<true> (e_prev read again).  Both are timed with the chosen
        // shape -- best of two launches each -- per outer iteration (batches x
        // sweep difference against reduce difference); the sweep takes the
        // margin only when that saves 3 % of the sweeps and reduction, so a
        // near tie (2D meshes) does not flip between runs.
        bool fuse = false;
        if (ctx->plan_lagged_dirs == 0 && !ctx->sweep_shape.staged) {  // (the staged kernel leaves it to k_reduce)
            if (only_margin >= 0) fuse = only_margin == 1;
            else {
                auto time_best = [&](auto&& launch) -> float {
                    float t = 1e30f;
                    for (int r = 0; r < 2; ++r) {
                        cudaEventRecord(e0, st);
                        launch();
                        cudaEventRecord(e1, st);
                        cudaEventSynchronize(e1);
                        float ms = 0;
                        cudaEventElapsedTime(&ms, e0, e1);
                        t = std::min(t, ms);
                    }
                    return t;
                };
                const SweepShape sh = ctx->sweep_shape;
                const int NB = ctx->n_band, nred = (int)(ctx->Np / bte::THREADS);
                const float sf = time_best([&] { launch_sweep<false>(ctx, sh, nbb, b0, st, sp, ssrc, 1, nullptr); });
                const float sm = time_best(
                    [&] { launch_sweep<true>(ctx, sh, nbb, b0, st, sp, ssrc, 1, ctx->d_spart.as<double>()); });
                auto reduce = [&](bool with_margin) {
                    if (with_margin)
                        bte::k_reduce<true><<<dim3(nred, NB), bte::THREADS, 0, st>>>(
                            ctx->e_curr, ctx->e_prev, ctx->d_omega.as<double>(), ctx->d_Cb.as<double>(), ctx->T_ref,
                            ctx->n, ctx->n_dir, ctx->Np, ctx->d_Tb.as<double>(), ctx->d_mpart.as<double>());
                    else
                        bte::k_reduce<false><<<dim3(nred, NB), bte::THREADS, 0, st>>>(
                            ctx->e_curr, ctx->e_prev, ctx->d_omega.as<double>(), ctx->d_Cb.as<double>(), ctx->T_ref,
                            ctx->n, ctx->n_dir, ctx->Np, ctx->d_Tb.as<double>(), nullptr);
                };
                const float rm = time_best([&] { reduce(true); });
                const float rf = time_best([&] { reduce(false); });
                BTE_LAUNCHED();
                const int batches = (NB + ctx->nbb - 1) / ctx->nbb;
                fuse = batches * (sm - sf) < (rm - rf) - 0.03f * (batches * sf + rf);
            }
        }
        ctx->sweep_shape.margin = fuse;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        ctx->sweep_tuned = true;
        std::lock_guard<std::mutex> lock(g_sweep_tune_mutex);
        g_sweep_tune[tkey] = ctx->sweep_shape;
    }
    const SweepShape shape = ctx->sweep_shape;
    if (shape.staged || shape.split) {  // a shape from the per-process cache: this plan's stage list may not exist yet
        const StageList* sl = nullptr;
        bte_status s2 = stage_list(ctx, shape.cap, &sl);
        if (s2 != BTE_OK) return s2;
    }
    ctx->sweep_margin = shape.margin && !shape.staged && ctx->plan_lagged_dirs == 0;
    // algorithmic HBM bytes of a sweep per system and cell: V Omega / D and
    // k / D read, x written (and, with the fused margin, the previous iterate
    // read), plus the level-ordered geometry per direction; ebar and the
    // boundary values come from L2
    const bool margin = ctx->sweep_margin;
    const double sweep_bytes = S * N * (margin ? 4 : 3) * w + geo;
    int sweeps = 0;
    for (;;) {
        if (margin) {
            BTE_LAUNCH(KK_SWEEP, -1, sweep_bytes, 0,
                       launch_sweep<true>(ctx, shape, nbb, b0, st, sp, ssrc, 1, ctx->d_spart.as<double>()));
        } else {
            BTE_LAUNCH(KK_SWEEP, -1, sweep_bytes, 0,
                       launch_sweep<false>(ctx, shape, nbb, b0, st, sp, ssrc, sweeps == 0, nullptr));
        }
        ++sweeps;
        if (ctx->plan_lagged_dirs == 0) break;
        BTE_CUDA(ctx->p_part.alloc(sizeof(double) * 2 * (size_t)S * ctx->nchunk));
        BTE_CUDA(ctx->p_bad.alloc(sizeof(int)));
        BTE_CUDA(cudaMemsetAsync(ctx->p_bad.p, 0, sizeof(int), st));
        BTE_LAUNCH(KK_SWEEP_RES, -1, S * N * 2 * w + geo, 0,
                   bte::k_sweep_residual<<<grid, bte::THREADS, 0, st>>>(op, src, ctx->p_cell.as<int>(),
                                                                        ctx->p_part.as<double>(), ctx->nchunk, ctx->n));
        bte::k_sweep_check<<<(S + 127) / 128, 128, 0, st>>>(ctx->p_part.as<double>(), S, ctx->nchunk, o.inner_tol,
                                                             ctx->p_bad.as<int>());
        BTE_LAUNCHED();
        BTE_CUDA(cudaMemcpyAsync(ctx->h_pinned_i, ctx->p_bad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
        BTE_CUDA(cudaStreamSynchronize(st));
        if (ctx->h_pinned_i[0] == 0) break;
        if (sweeps >= o.inner_maxit) {
            rep.inner_unconverged += ctx->h_pinned_i[0];
            break;
        }
    }
    if (ctx->profile) {
        BTE_CUDA(cudaStreamSynchronize(st));
        prof_resolve(ctx, nullptr, 0);
    }
    rep.inner_iterations += (long long)S * sweeps;
    rep.inner_solves += S;
    return BTE_OK;
}

// Anderson state: T and the intensities at the cells with boundary faces.
static bte::mlp::AaState aa_state(const bte_ctx* ctx) {
    return bte::mlp::AaState{ctx->d_bcell.as<int>(), ctx->n, ctx->nbcell, ctx->n_band, ctx->n_dir, ctx->Np,
                             ctx->d_Cb.as<double>(), ctx->solid_angle};
}
static size_t aa_len(const bte_ctx* ctx) { return (size_t)ctx->n + (size_t)ctx->n_band * ctx->n_dir * ctx->nbcell; }

// One Anderson step after outer iteration it (it >= 1): store (g, f) of this
// iteration, form the Gram matrix of the stored f, solve for alpha and set
// T = sum alpha_i g_i (and ebar).  The history restarts when the margin grew
// tenfold or the weights blow up.
static bte_status anderson_step(bte_ctx* ctx, int slots, int& count, int& next, std::vector<int>& order, double m,
                                bte_report& rep) {
    namespace M = bte::mlp;
    cudaStream_t st = ctx->stream;
    const int n = ctx->n;
    if (count > 0 && m > 10.0 * ctx->aa_prev_margin) {  // diverging: keep only this iteration
        count = 0;
        order.clear();
    }
    ctx->aa_prev_margin = m;
    const int slot = next;
    next = (next + 1) % slots;
    if (count == slots) order.erase(order.begin());
    else ++count;
    order.push_back(slot);
    const M::AaState as = aa_state(ctx);
    const size_t L = aa_len(ctx);
    const unsigned gl = (unsigned)((L + 255) / 256);
    M::AaMix mx{};
    mx.k = count;
    for (int i = 0; i < count; ++i) mx.slot[i] = order[i];
    const int nblk = M::AA_BLOCKS;
    BTE_LAUNCH(KK_REDUCE, -1, (3.0 + count) * L * 8.0, 0,
               M::k_aa_push<<<nblk, M::AA_THREADS, 0, st>>>(as, ctx->d_T.as<double>(), ctx->e_curr,
                                                           ctx->d_aa_x.as<double>(), L, slot, mx,
                                                           ctx->d_aa_g.as<double>(), ctx->d_aa_f.as<double>(),
                                                           ctx->d_aa_part.as<double>()));
    M::k_aa_row<<<1, 32 * M::AA_MAX, 0, st>>>(ctx->d_aa_part.as<double>(), nblk, slot, mx,
                                               ctx->d_aa_gram.as<double>());
    BTE_LAUNCHED();
    const int k = count;
    if (k < 2) return BTE_OK;  // nothing to mix yet
    // the small least-squares system on the device: no host round trip; an
    // ill-conditioned history sets the flag the host reads with the next margin
    M::k_aa_solve<<<1, 32, 0, st>>>(ctx->d_aa_gram.as<double>(), mx, ctx->d_aa_alpha.as<double>(),
                                   ctx->d_aa_flag.as<double>());
    BTE_LAUNCHED();
    BTE_LAUNCH(KK_REDUCE, -1, ((double)k + 1) * L * 8.0, 0,
               M::k_aa_mix<<<gl, 256, 0, st>>>(as, ctx->d_aa_g.as<double>(), L, mx, ctx->d_aa_alpha.as<double>(),
                                                ctx->T_ref, ctx->d_T.as<double>(), ctx->d_ebar.as<double>(),
                                                ctx->e_curr));
    BTE_LAUNCH(KK_REDUCE, -1, (double)(ctx->n_band + 1) * n * 8.0, 0,
               M::k_ebar_from_T<<<dim3((n + 255) / 256, ctx->n_band), 256, 0, st>>>(
                   ctx->d_T.as<double>(), ctx->d_Cb.as<double>(), ctx->solid_angle, ctx->T_ref, n, ctx->Np,
                   ctx->d_ebar.as<double>()));
    ++rep.accel_steps;
    return BTE_OK;
}

extern "C" bte_status bte_solve(bte_ctx* ctx, const bte_options* opts, bte_report* report) {
    if (!ctx) return BTE_ERR_INVALID_ARGUMENT;
    if (!(ctx->has_geom && ctx->has_quad && ctx->has_bands && ctx->has_bcs))
        return fail(ctx, BTE_ERR_STATE, "bte_solve: set geometry, quadrature, bands and boundary conditions first");
    bte_options o;
    if (opts) o = *opts;
    else bte_default_options(&o);
    if (o.max_iter < 0 || o.inner_maxit <= 0 || !(o.inner_tol > 0))
        return fail(ctx, BTE_ERR_INVALID_ARGUMENT, "bte_solve: bad options");
    if (o.form != BTE_FORM_PLAIN && o.form != BTE_FORM_SWEEP && o.form != BTE_FORM_MIXED)
        return fail(ctx, BTE_ERR_INVALID_ARGUMENT, "bte_solve: unknown form");
    if (ctx->dim == 1 && ctx->F != 2) return fail(ctx, BTE_ERR_INVALID_ARGUMENT, "1D mesh needs 2 faces");
    if (o.dsa && ctx->dim == 1) return fail(ctx, BTE_ERR_INVALID_ARGUMENT, "bte_solve: dsa needs a 2D or 3D mesh");
    if (o.dsa && (o.dsa_tol < 0 || o.dsa_maxit < 0))
        return fail(ctx, BTE_ERR_INVALID_ARGUMENT, "bte_solve: bad dsa_tol / dsa_maxit");
    const double dsa_tol = o.dsa_tol > 0 ? o.dsa_tol : 1e-3;
    const int dsa_maxit = o.dsa_maxit > 0 ? o.dsa_maxit : 4000;
    // The correction amplifies an inner solve's error by up to 1 / (1 - rho),
    // rho the source iteration's contraction (~1e5 on a 1e-4 m square).  The
    // mixed form's refinement stops just under inner_tol, and at 1e-9 its
    // margins then cycle between 1e-2 and 20 on that square; at 1e-11 it
    // stops in the 9 outer iterations of the FP64 forms.
    if (o.dsa && o.form == BTE_FORM_MIXED) o.inner_tol = std::min(o.inner_tol, kDsaMixedInnerTol);
    BTE_CUDA(cudaSetDevice(ctx->device));
    bte_report rep;
    std::memset(&rep, 0, sizeof(rep));
    ctx->launches = 0;
    ctx->profile = o.profile != 0;
    ctx->pending.clear();
    ctx->ev_next = 0;
    for (int k = 0; k < kNumKinds; ++k) {
        std::memset(&ctx->stats[k], 0, sizeof(bte_kernel_stat));
        std::snprintf(ctx->stats[k].name, sizeof(ctx->stats[k].name), "%s", kKindNames[k]);
    }
    const auto wall0 = std::chrono::steady_clock::now();
    auto since = [](std::chrono::steady_clock::time_point t) {
        return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t).count();
    };
    if (ctx->dirty) {
        const auto t = std::chrono::steady_clock::now();
        bte_status s = setup(ctx, o.batch_systems);
        if (s != BTE_OK) return s;
        rep.ms_host_setup = since(t);
    }
    // new geometry with dsa: the low-order operator's host work runs on a
    // host thread while the sweep plan is built
    const bool need_plan = o.form == BTE_FORM_SWEEP && !ctx->plan_ready;
    const bool need_dsa = o.dsa && !ctx->dsa_ready;
    DsaSetupHost dsa_host;
    std::thread dsa_thread;
    struct Joiner {
        std::thread& t;
        ~Joiner() {
            if (t.joinable()) t.join();
        }
    } joiner{dsa_thread};
    const auto t_dsa = std::chrono::steady_clock::now();
    bte_status dsa_status = BTE_OK;
    if (need_dsa) {
        int nblk = 0;
        bte_status s = dsa_blocks(ctx, ctx->n, &nblk);
        if (s != BTE_OK) return s;
        if (need_plan) {
            // host part and device part (on its own stream) on a host thread
            if (!ctx->setup_stream) BTE_CUDA(cudaStreamCreateWithFlags(&ctx->setup_stream, cudaStreamNonBlocking));
            dsa_thread = std::thread([ctx, nblk, &dsa_host, &dsa_status] {
                if (cudaSetDevice(ctx->device) != cudaSuccess) {
                    dsa_status = fail(ctx, BTE_ERR_CUDA, "dsa: cudaSetDevice on the set-up thread failed");
                    return;
                }
                setup_dsa_host(ctx, nblk, dsa_host);
                dsa_status = setup_dsa_device(ctx, dsa_host, ctx->setup_stream);
            });
        } else {
            setup_dsa_host(ctx, nblk, dsa_host);
            dsa_status = setup_dsa_device(ctx, dsa_host, ctx->stream);
        }
    }
    if (need_plan) {
        const auto t = std::chrono::steady_clock::now();
        bte_status s = build_sweep_plan(ctx);
        if (s != BTE_OK) return s;
        rep.ms_host_plan = since(t);
        rep.ms_host_order = ctx->ms_last_order;
    }
    if (o.form == BTE_FORM_MIXED && !ctx->mixed_ready) {
        bte_status s = setup_mixed(ctx);
        if (s != BTE_OK) return s;
    }
    // The low-order set-up on its thread may still run: the solve starts, and
    // the thread is joined before the first correction (after the first
    // outer iteration), or after the loop.  Its device part is complete when
    // it returns (it synchronises its stream).
    bool dsa_pending = dsa_thread.joinable();
    auto join_dsa = [&]() -> bte_status {
        if (!dsa_pending) return BTE_OK;
        dsa_thread.join();
        dsa_pending = false;
        rep.ms_host_dsa = since(t_dsa);  // (overlaps the plan's time and the first iteration's)
        if (dsa_status != BTE_OK) return dsa_status;
        ctx->dsa_ready = true;
        return BTE_OK;
    };
    if (need_dsa && !dsa_pending) {
        if (dsa_status != BTE_OK) return dsa_status;
        ctx->dsa_ready = true;
        rep.ms_host_dsa = since(t_dsa);
    }
    // without a wall held at a fixed temperature the low-order operator is singular: dsa is ignored
    const int dsa_walls = dsa_pending ? dsa_wall_faces(ctx) : ctx->dsa_walls;
    const bool dsa_on = o.dsa && dsa_walls > 0;
    if (dsa_on) BTE_CUDA(ctx->d_Tsrc.alloc(sizeof(double) * ctx->Np));
    cudaStream_t st = ctx->stream;
    const int NB = ctx->n_band, ND = ctx->n_dir;
    const size_t Np = ctx->Np;
    ctx->e_curr = ctx->d_e0.as<double>();
    ctx->e_prev = ctx->d_e1.as<double>();
    BTE_CUDA(cudaMemsetAsync(ctx->e_curr, 0, sizeof(double) * NB * ND * Np, st));
    BTE_CUDA(cudaMemsetAsync(ctx->d_ebar.p, 0, sizeof(double) * NB * Np, st));  // cell_band_density = 0 (:92)
    if (dsa_on) {
        // the source of the first outer iteration is ebar = 0, i.e. T = T_ref
        bte::dsa::k_fill<<<(unsigned)((Np + 255) / 256), 256, 0, st>>>(ctx->d_T.as<double>(), ctx->T_ref, (int)Np);
        BTE_LAUNCHED();
        // (the low-order work memory exists once its set-up is joined)
        if (!dsa_pending) BTE_CUDA(cudaMemsetAsync(ctx->cg_stat.p, 0, sizeof(int) * 4, st));
    }
    ctx->margins.clear();
    double Lr_sum = 0;
    for (int b = 0; b < NB; ++b) Lr_sum += ctx->Lr[b];
    // [0..3] the phases of an outer iteration, [5..6] the accelerator step
    // after it (the dsa correction included), [7..8] the dsa correction
    cudaEvent_t ev[9];
    for (auto& e : ev) BTE_CUDA(cudaEventCreate(&e));
    struct EvGuard { cudaEvent_t* e; ~EvGuard() { for (int k = 0; k < 9; ++k) cudaEventDestroy(e[k]); } } guard{ev};
    bool accel_timed = false;  // ev[5..6] hold an accelerator step not yet added to the report
    bool dsa_timed = false;    // ev[7..8] hold a dsa correction not yet added
    auto add_accel_time = [&]() {
        if (dsa_timed) {
            float t = 0;
            cudaEventElapsedTime(&t, ev[7], ev[8]);
            rep.ms_dsa += t;
            dsa_timed = false;
        }
        if (!accel_timed) return;
        float t = 0;
        cudaEventElapsedTime(&t, ev[5], ev[6]);
        rep.ms_reduce += t;
        rep.ms_total += t;
        accel_timed = false;
    };
    const bool post_step = o.accel != 0 || dsa_on;  // kernels after the margin read-back
    bte_status result = BTE_ERR_NOT_CONVERGED;
    const int nred = (int)(Np / bte::THREADS);
    // the sweep of an acyclic plan may sum the margin itself (k_reduce then
    // reads e_curr only); the choice is made with the launch shape, on the
    // first sweep, so it is read after the sweeps of an iteration
    auto fused_margin = [&]() { return o.form == BTE_FORM_SWEEP && ctx->sweep_margin; };
    const bool acyclic_sweep = o.form == BTE_FORM_SWEEP && ctx->plan_lagged_dirs == 0;
    // accelerator set-up
    bool accel_on = o.accel != 0;
    int accel_last = -1;
    double accel_margin = 0.0;
    bte::mlp::FeatureGeom fg{};
    if (o.accel < 0 || o.accel > 3) return fail(ctx, BTE_ERR_INVALID_ARGUMENT, "bte_solve: accel must be 0..3");
    // Anderson mixing (accel = 3): depth m = accel_every, slots m + 1
    const int aa_slots = o.accel == 3 ? o.accel_every + 1 : 0;
    int aa_count = 0, aa_next = 0;  // stored pairs, next slot
    std::vector<int> aa_order;      // stored slots, oldest first
    if (o.accel == 3) {
        if (o.accel_every < 1 || aa_slots > bte::mlp::AA_MAX)
            return fail(ctx, BTE_ERR_INVALID_ARGUMENT, "bte_solve: Anderson depth (accel_every) must be 1..8");
        const size_t L = aa_len(ctx);
        const int nblk = bte::mlp::AA_BLOCKS;
        BTE_CUDA(ctx->d_aa_x.alloc(sizeof(double) * L));
        BTE_CUDA(ctx->d_aa_g.alloc(sizeof(double) * aa_slots * L));
        BTE_CUDA(ctx->d_aa_f.alloc(sizeof(double) * aa_slots * L));
        BTE_CUDA(ctx->d_aa_part.alloc(sizeof(double) * bte::mlp::AA_MAX * nblk));
        BTE_CUDA(ctx->d_aa_gram.alloc(sizeof(double) * bte::mlp::AA_MAX * bte::mlp::AA_MAX));
        BTE_CUDA(ctx->d_aa_alpha.alloc(sizeof(double) * bte::mlp::AA_MAX));
        BTE_CUDA(ctx->d_aa_flag.alloc(sizeof(double)));
        BTE_CUDA(cudaMemsetAsync(ctx->d_aa_flag.p, 0, sizeof(double), st));
    }
    if (o.accel == 1 || o.accel == 2) {
        if (o.accel_every < 4) return fail(ctx, BTE_ERR_INVALID_ARGUMENT, "bte_solve: accel_every must be >= 4");
        if (o.accel == 1 && !ctx->has_mlp) return fail(ctx, BTE_ERR_STATE, "bte_solve: accel = 1 needs bte_set_mlp");
        if ((int)ctx->centroid.size() != 3 * ctx->n)
            return fail(ctx, BTE_ERR_STATE, "bte_solve: the accelerator needs bte_set_centroids");
        BTE_CUDA(upload(ctx->d_centroid, ctx->centroid, st));
        BTE_CUDA(ctx->d_ring.alloc(sizeof(double) * 4 * Np));
        // the state before the last jump, restored when the jump does not pay off
        BTE_CUDA(ctx->d_snap_e.alloc(sizeof(double) * (size_t)NB * ND * Np));
        BTE_CUDA(ctx->d_snap_T.alloc(sizeof(double) * Np));
        BTE_CUDA(ctx->d_snap_ebar.alloc(sizeof(double) * (size_t)NB * Np));
        BTE_CUDA(ctx->d_feat.alloc(sizeof(__nv_bfloat16) * bte::mlp::IN_PAD * ctx->n));
        BTE_CUDA(ctx->d_scale.alloc(sizeof(double) * ctx->n));
        BTE_CUDA(ctx->d_y.alloc(sizeof(float) * ctx->n));
        BTE_CUDA(cudaFuncSetAttribute(bte::mlp::k_forward, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)bte::mlp::FWD_SMEM));
        double vmean = 0, xmin = 1e300, xmax = -1e300, ymin = 1e300, ymax = -1e300, lrs = 0, lrk = 0, dT = 0;
        for (int c = 0; c < ctx->n; ++c) {
            vmean += ctx->volume[c];
            xmin = std::min(xmin, ctx->centroid[3 * c]); xmax = std::max(xmax, ctx->centroid[3 * c]);
            ymin = std::min(ymin, ctx->centroid[3 * c + 1]); ymax = std::max(ymax, ctx->centroid[3 * c + 1]);
        }
        for (int b = 0; b < NB; ++b) { lrs += ctx->Lr[b]; lrk += ctx->Lr[b] * ctx->vg[b] * ctx->tau[b]; }
        for (int i = 0; i < ctx->n_bc; ++i) dT = std::max(dT, std::fabs(ctx->bc_T[i] - ctx->T_ref));
        fg = bte::mlp::FeatureGeom{ctx->d_centroid.as<double>(), ctx->d_volume.as<double>(), vmean / ctx->n, xmin,
                                   xmax - xmin, ymin, ymax - ymin, lrk / lrs, 1.0 / ctx->dim, ctx->T_ref,
                                   dT > 0 ? dT : 1.0};
    }
    ctx->history.clear();
    ctx->history_rows = 0;
    // CUDA graphs of the sweep form's outer iteration (not with the profiler,
    // which times each launch, nor with lagged edges, whose sweeps repeat
    // under host control)
    const bool use_graph = o.form == BTE_FORM_SWEEP && ctx->plan_lagged_dirs == 0 && !ctx->profile;
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    struct GraphGuard {
        cudaGraphExec_t* g;
        ~GraphGuard() {
            for (int k = 0; k < 2; ++k)
                if (g[k]) cudaGraphExecDestroy(g[k]);
        }
    } graph_guard{gexec};
    long long graph_solves[2] = {0, 0}, graph_inner[2] = {0, 0}, graph_launches[2] = {0, 0};
    for (int it = 0; it < o.max_iter; ++it) {
        std::swap(ctx->e_curr, ctx->e_prev);
        BTE_CUDA(cudaEventRecord(ev[0], st));
        if (dsa_on)  // the temperature this iteration's source comes from
            BTE_CUDA(cudaMemcpyAsync(ctx->d_Tsrc.p, ctx->d_T.p, sizeof(double) * ctx->n, cudaMemcpyDeviceToDevice, st));
        if (aa_slots && it > 0) {  // the state this iteration starts from (iteration 0 starts from T_ref, e = 0)
            const bte::mlp::AaState as = aa_state(ctx);
            const size_t L = aa_len(ctx);
            BTE_LAUNCH(KK_REDUCE, -1, 2.0 * L * 8.0, 0,
                       bte::mlp::k_aa_gather<<<(unsigned)((L + 255) / 256), 256, 0, st>>>(
                           as, ctx->d_T.as<double>(), ctx->e_prev, ctx->d_aa_x.as<double>()));
        }
        // the kernels of one outer iteration (ev[1], ev[2] mark its phases when
        // launched one by one; a captured CUDA graph is timed as a whole)
        auto enqueue_iteration = [&](bool timed) -> bte_status {
            if (ctx->ndiff > 0) {
                const int nt = ctx->ndiff * NB;
                BTE_LAUNCH(KK_DIFFUSE, -1, (double)nt * (ND + 1) * 8.0, 0,
                           bte::k_diffuse_wall<<<(nt + 3) / 4, 128, 0, st>>>(
                               ctx->e_prev, ctx->d_dlist.as<int>(), ctx->d_bf_cell.as<int>(), ctx->d_wdiff.as<double>(),
                               ctx->d_wden.as<double>(), ctx->ndiff, NB, ND, Np, ctx->nbf, ctx->d_ediff.as<double>()));
            }
            if (acyclic_sweep) BTE_CUDA(cudaMemsetAsync(ctx->d_spart.p, 0, sizeof(double) * ND * NB, st));
            if (timed) BTE_CUDA(cudaEventRecord(ev[1], st));
            for (int b0 = 0; b0 < NB; b0 += ctx->nbb) {
                const int nbb = std::min(ctx->nbb, NB - b0);
                bte_status s = o.form == BTE_FORM_SWEEP   ? solve_batch_sweep(ctx, b0, nbb, o, rep)
                               : o.form == BTE_FORM_MIXED ? solve_batch_mixed(ctx, b0, nbb, o, rep)
                                                          : solve_batch_plain(ctx, b0, nbb, o, rep);
                if (s != BTE_OK) return s;
            }
            if (timed) BTE_CUDA(cudaEventRecord(ev[2], st));
            const bool fused = fused_margin();
            if (fused) {
                BTE_LAUNCH(KK_REDUCE, -1, (1.0 * NB * ND + NB) * ctx->n * 8.0, 0,
                           bte::k_reduce<false><<<dim3(nred, NB), bte::THREADS, 0, st>>>(
                               ctx->e_curr, ctx->e_prev, ctx->d_omega.as<double>(), ctx->d_Cb.as<double>(), ctx->T_ref,
                               ctx->n, ND, Np, ctx->d_Tb.as<double>(), nullptr));
            } else {
                BTE_LAUNCH(KK_REDUCE, -1, (2.0 * NB * ND + NB) * ctx->n * 8.0, 0,
                           bte::k_reduce<true><<<dim3(nred, NB), bte::THREADS, 0, st>>>(
                               ctx->e_curr, ctx->e_prev, ctx->d_omega.as<double>(), ctx->d_Cb.as<double>(), ctx->T_ref,
                               ctx->n, ND, Np, ctx->d_Tb.as<double>(), ctx->d_mpart.as<double>()));
            }
            BTE_LAUNCH(KK_REDUCE, -1, (2.0 * NB + 1) * ctx->n * 8.0, 0,
                       bte::k_recover<<<(ctx->n + bte::RC_CELLS - 1) / bte::RC_CELLS, bte::RC_CELLS * bte::RC_SLICES,
                                        0, st>>>(
                           ctx->d_Tb.as<double>(), ctx->d_Cb.as<double>(), ctx->d_Lr.as<double>(), Lr_sum, ctx->T_ref,
                           ctx->solid_angle, ctx->n, NB, Np, ctx->d_T.as<double>(), ctx->d_ebar.as<double>()));
            // margin = sum of the partials / (n_band n_cell), fixed order
            bte::k_margin_final<<<1, bte::THREADS, 0, st>>>(fused ? ctx->d_spart.as<double>() : ctx->d_mpart.as<double>(),
                                                            fused ? ND * NB : nred * NB, (double)NB * ctx->n,
                                                            ctx->d_margin.as<double>());
            BTE_LAUNCHED();
            return BTE_OK;
        };
        if (use_graph && it >= 1) {
            // from the second outer iteration on (the first times the sweep's
            // launch shapes), the iteration is one CUDA graph per parity of it
            // (e_curr and e_prev alternate), captured once and replayed
            const int par = it & 1;
            if (!gexec[par]) {
                const bte_report before = rep;
                const long long launches_before = ctx->launches;
                BTE_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
                const bte_status cs = enqueue_iteration(false);
                cudaGraph_t graph = nullptr;
                const cudaError_t ce = cudaStreamEndCapture(st, &graph);
                if (cs != BTE_OK) {
                    if (graph) cudaGraphDestroy(graph);
                    return cs;
                }
                BTE_CUDA(ce);
                const cudaError_t ie = cudaGraphInstantiate(&gexec[par], graph, 0);
                cudaGraphDestroy(graph);
                BTE_CUDA(ie);
                // host-side counters the capture advanced: added on every replay instead
                graph_solves[par] = rep.inner_solves - before.inner_solves;
                graph_inner[par] = rep.inner_iterations - before.inner_iterations;
                graph_launches[par] = ctx->launches - launches_before;
                rep.inner_solves = before.inner_solves;
                rep.inner_iterations = before.inner_iterations;
                ctx->launches = launches_before;
            }
            BTE_CUDA(cudaEventRecord(ev[1], st));
            BTE_CUDA(cudaGraphLaunch(gexec[par], st));
            BTE_CUDA(cudaEventRecord(ev[2], st));
            rep.inner_solves += graph_solves[par];
            rep.inner_iterations += graph_inner[par];
            ctx->launches += graph_launches[par];
        } else {
            bte_status es = enqueue_iteration(true);
            if (es != BTE_OK) return es;
        }
        BTE_CUDA(cudaEventRecord(ev[3], st));
        BTE_CUDA(cudaMemcpyAsync(ctx->h_pinned, ctx->d_margin.p, sizeof(double), cudaMemcpyDeviceToHost, st));
        if (aa_slots)
            BTE_CUDA(cudaMemcpyAsync(ctx->h_pinned + 1, ctx->d_aa_flag.p, sizeof(double), cudaMemcpyDeviceToHost, st));
        BTE_CUDA(cudaStreamSynchronize(st));
        if (ctx->profile) prof_resolve(ctx, nullptr, 0);
        add_accel_time();
        const double m = ctx->h_pinned[0];
        if (aa_slots && ctx->h_pinned[1] != 0.0) {  // the last Anderson weights blew up: restart the history
            if (!aa_order.empty()) aa_order.erase(aa_order.begin(), aa_order.end() - 1);
            aa_count = (int)aa_order.size();
            BTE_CUDA(cudaMemsetAsync(ctx->d_aa_flag.p, 0, sizeof(double), st));
        }
        // the last four temperature fields (accelerator) and the history
        if (o.accel == 1 || o.accel == 2) {
            BTE_CUDA(cudaMemcpyAsync(ctx->d_ring.as<double>() + (size_t)(it % 4) * Np, ctx->d_T.p,
                                     sizeof(double) * Np, cudaMemcpyDeviceToDevice, st));
        }
        if (o.keep_history) {
            ctx->history.resize((size_t)(it + 1) * ctx->n);
            BTE_CUDA(cudaMemcpyAsync(ctx->history.data() + (size_t)it * ctx->n, ctx->d_T.p, sizeof(double) * ctx->n,
                                     cudaMemcpyDeviceToHost, st));
            BTE_CUDA(cudaStreamSynchronize(st));
            ctx->history_rows = it + 1;
        }
        float t01 = 0, t12 = 0, t23 = 0;
        cudaEventElapsedTime(&t01, ev[0], ev[1]);
        cudaEventElapsedTime(&t12, ev[1], ev[2]);
        cudaEventElapsedTime(&t23, ev[2], ev[3]);
        rep.ms_rhs += t01;
        rep.ms_inner += t12;
        rep.ms_reduce += t23;
        rep.ms_total += t01 + t12 + t23;
        ctx->margins.push_back(m);
        rep.n_iter = it + 1;
        rep.final_margin = m;
        if (o.on_iteration) o.on_iteration(o.user, it, m, (double)(t01 + t12 + t23));
        if (!std::isfinite(m)) {
            result = BTE_ERR_NUMERICAL;
            ctx->err = "non-finite margin in outer iteration " + std::to_string(it);
            break;
        }
        if (m <= o.tol) {
            rep.converged = 1;
            result = BTE_OK;
            break;
        }
        // outer-iteration extrapolation (accel): stop for good when the margin
        // accel_every-1 iterations after a jump is not below the margin at it
        // accel_every-1 iterations after a jump: keep it if the margin is below
        // the margin at the jump (right after a jump the margin rises while the
        // intensities follow the new source, so it is judged once they have);
        // otherwise restore the state before the jump and stop extrapolating
        if (post_step) {
            BTE_CUDA(cudaEventRecord(ev[5], st));
            accel_timed = true;
        }
        if (dsa_on) {
            // low-order correction: solve for the remaining error x of T from
            // this iteration's change, then T += x (and ebar, and the boundary
            // cells' intensities the walls reflect next)
            const int n = ctx->n;
            if (dsa_pending) {
                bte_status js = join_dsa();
                if (js != BTE_OK) return js;
                if (ctx->dsa_walls != dsa_walls)
                    return fail(ctx, BTE_ERR_STATE, "dsa: the set-up found another count of fixed-temperature faces");
                BTE_CUDA(cudaMemsetAsync(ctx->cg_stat.p, 0, sizeof(int) * 4, st));
            }
            BTE_CUDA(cudaEventRecord(ev[7], st));
            BTE_LAUNCH(KK_DSA, -1, 3.0 * n * 8.0, 0,
                       bte::dsa::k_dsa_rhs<<<(n + 255) / 256, 256, 0, st>>>(
                           ctx->d_T.as<double>(), ctx->d_Tsrc.as<double>(), ctx->d_volume.as<double>(),
                           ctx->d_dsa_order.as<int>(), n, ctx->d_dsa_b.as<double>()));
            {
                size_t slot = 0;
                BTE_CUDA(prof_begin(ctx, &slot));
                bte_status ls = dsa_launch(ctx, n, ctx->F, dsa_tol, dsa_maxit);
                if (ls != BTE_OK) return ls;
                BTE_CUDA(prof_end(ctx, slot, KK_DSA, -1, 0, 0));
            }
            BTE_LAUNCH(KK_DSA, -1, (2.0 + NB) * n * 8.0, 0,
                       bte::dsa::k_dsa_apply<<<(n + 255) / 256, 256, 0, st>>>(
                           ctx->d_dsa_x.as<double>(), ctx->d_dsa_pos.as<int>(), ctx->d_Cb.as<double>(),
                           ctx->solid_angle, ctx->T_ref, n, NB, Np, ctx->d_T.as<double>(), ctx->d_ebar.as<double>(),
                           ctx->d_dsa_xc.as<double>()));
            if (ctx->nbcell > 0) {
                const int nt = ctx->nbcell * ND;
                BTE_LAUNCH(KK_DSA, -1, 2.0 * nt * NB * 8.0, 0,
                           bte::dsa::k_dsa_shift_boundary<<<dim3((nt + 255) / 256, NB), 256, 0, st>>>(
                               ctx->d_dsa_xc.as<double>(), ctx->d_bcell.as<int>(), ctx->nbcell, ctx->d_Cb.as<double>(),
                               ctx->solid_angle, ND, Np, ctx->e_curr));
            }
            BTE_CUDA(cudaEventRecord(ev[8], st));
            dsa_timed = true;
            ++rep.dsa_solves;
        }
        if (aa_slots && it > 0) {
            bte_status s = anderson_step(ctx, aa_slots, aa_count, aa_next, aa_order, m, rep);
            if (s != BTE_OK) return s;
        }
        if ((o.accel == 1 || o.accel == 2) && accel_on && accel_last >= 0 && it == accel_last + o.accel_every - 1 &&
            !(m < accel_margin)) {
            accel_on = false;
            const size_t ne = (size_t)NB * ND * Np;
            BTE_CUDA(cudaMemcpyAsync(ctx->e_curr, ctx->d_snap_e.p, sizeof(double) * ne, cudaMemcpyDeviceToDevice, st));
            BTE_CUDA(cudaMemcpyAsync(ctx->d_T.p, ctx->d_snap_T.p, sizeof(double) * Np, cudaMemcpyDeviceToDevice, st));
            BTE_CUDA(cudaMemcpyAsync(ctx->d_ebar.p, ctx->d_snap_ebar.p, sizeof(double) * NB * Np,
                                     cudaMemcpyDeviceToDevice, st));
            ++rep.accel_reverts;
        }
        if ((o.accel == 1 || o.accel == 2) && accel_on && it >= 3 &&
            (accel_last < 0 || it - accel_last >= o.accel_every)) {
            const int n = ctx->n;
            const int s0 = it % 4, s1 = (it + 3) % 4, s2 = (it + 2) % 4, s3 = (it + 1) % 4;
            BTE_CUDA(cudaMemcpyAsync(ctx->d_snap_e.p, ctx->e_curr, sizeof(double) * (size_t)NB * ND * Np,
                                     cudaMemcpyDeviceToDevice, st));
            BTE_CUDA(cudaMemcpyAsync(ctx->d_snap_T.p, ctx->d_T.p, sizeof(double) * Np, cudaMemcpyDeviceToDevice, st));
            BTE_CUDA(cudaMemcpyAsync(ctx->d_snap_ebar.p, ctx->d_ebar.p, sizeof(double) * NB * Np,
                                     cudaMemcpyDeviceToDevice, st));
            BTE_LAUNCH(KK_REDUCE, -1, 0, 0,
                       bte::mlp::k_accel_features<<<(n + 255) / 256, 256, 0, st>>>(
                           ctx->d_ring.as<double>(), s0, s1, s2, s3, Np, n, fg, ctx->d_feat.as<__nv_bfloat16>(),
                           ctx->d_scale.as<double>()));
            if (o.accel == 1) {
                BTE_LAUNCH(KK_REDUCE, -1, 0, 0,
                           bte::mlp::k_forward<<<std::max(1, std::min(1024, (n + 63) / 64)), 128, bte::mlp::FWD_SMEM, st>>>(
                               ctx->d_feat.as<__nv_bfloat16>(), n, ctx->d_wpack.as<__nv_bfloat16>(),
                               ctx->d_params.as<float>(), ctx->d_y.as<float>(), nullptr));
            }
            BTE_LAUNCH(KK_REDUCE, -1, 0, 0,
                       bte::mlp::k_accel_apply<<<(n + 255) / 256, 256, 0, st>>>(
                           ctx->d_ring.as<double>(), s0, s1, s2, Np, n, ctx->d_scale.as<double>(),
                           ctx->d_y.as<float>(), o.accel == 1, ctx->d_Cb.as<double>(), NB, ctx->solid_angle,
                           ctx->T_ref, ctx->d_T.as<double>(), ctx->d_ebar.as<double>()));
            accel_last = it;
            accel_margin = m;
            ++rep.accel_steps;
        }
        // the accelerator's kernels and copies run after ev[3]: timed by
        // ev[5..6], read after the next synchronisation
        if (post_step) BTE_CUDA(cudaEventRecord(ev[6], st));
    }
    if (accel_timed) {
        BTE_CUDA(cudaEventSynchronize(ev[6]));
        add_accel_time();
    }
    // a low-order set-up that no correction needed (the solve stopped first)
    if (dsa_pending) (void)join_dsa();
    if (o.max_iter == 0) result = BTE_OK;
    // heat flux (src/StaticBTESolver.cpp:323-370)
    if (ctx->nbf > 0) {
        const int nt = ctx->nbf * NB;
        BTE_LAUNCH(KK_HEAT, -1, (double)nt * ND * 16.0, 0,
                   bte::k_heat_face<<<(nt + 127) / 128, 128, 0, st>>>(ctx->e_curr, ctx->d_bf_cell.as<int>(),
                                                                    ctx->d_hw.as<double>(), ctx->nbf, NB, ND, Np,
                                                                    ctx->d_hpart.as<double>()));
    }
    bte::k_heat_final<<<1, 256, 0, st>>>(ctx->d_hpart.as<double>(), ctx->d_bf_bc.as<int>(),
                                        ctx->d_bf_area.as<double>(), ctx->d_vg.as<double>(), ctx->nbf, NB,
                                        ctx->n_bc, ctx->dim, ctx->d_qband.as<double>(), ctx->d_q.as<double>());
    BTE_LAUNCHED();
    int dsa_stat[4] = {0, 0, 0, 0};
    if (dsa_on && rep.dsa_solves > 0)
        BTE_CUDA(cudaMemcpyAsync(dsa_stat, ctx->cg_stat.p, sizeof(dsa_stat), cudaMemcpyDeviceToHost, st));
    int sweep_err = 0;
    if (o.form == BTE_FORM_SWEEP && ctx->d_sweep_err.p)
        BTE_CUDA(cudaMemcpyAsync(&sweep_err, ctx->d_sweep_err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    BTE_CUDA(cudaStreamSynchronize(st));
    if (ctx->profile) prof_resolve(ctx, nullptr, 0);
    if (sweep_err) {
        BTE_CUDA(cudaMemsetAsync(ctx->d_sweep_err.p, 0, sizeof(int), st));
        BTE_CUDA(cudaStreamSynchronize(st));
        if (report) *report = rep;
        return fail(ctx, BTE_ERR_CUDA, "sweep: a stage's copies did not complete in time (the fields are not valid)");
    }
    if (dsa_on) {
        rep.dsa_iterations = dsa_stat[2];
        if (dsa_stat[1]) {
            if (report) *report = rep;
            return fail(ctx, BTE_ERR_CUDA, "dsa: a grid barrier of the low-order solve timed out");
        }
    }
    rep.kernel_launches = ctx->launches;
    rep.sweep_group = o.form == BTE_FORM_SWEEP ? ctx->sweep_shape.G : 0;
    rep.sweep_threads = o.form == BTE_FORM_SWEEP ? ctx->sweep_shape.threads : 0;
    rep.sweep_ring = o.form == BTE_FORM_SWEEP ? ctx->sweep_shape.W : 0;
    rep.sweep_margin = o.form == BTE_FORM_SWEEP && ctx->sweep_margin ? 1 : 0;
    rep.sweep_kernel = o.form == BTE_FORM_SWEEP ? ctx->sweep_shape.kind() : 0;
    rep.ms_wall = since(wall0);
    rep.sweep_host_dirs = o.form == BTE_FORM_SWEEP ? ctx->plan_host_dirs : 0;
    ctx->solved = true;
    if (report) *report = rep;
    if (result == BTE_ERR_NOT_CONVERGED && ctx->err.empty()) ctx->err = "max_iter reached";
    return result;
}

extern "C" {

bte_status bte_get_temperature(bte_ctx* ctx, double* T) {
    if (!ctx || !T) return BTE_ERR_INVALID_ARGUMENT;
    if (!ctx->solved) return fail(ctx, BTE_ERR_STATE, "no solution yet");
    BTE_CUDA(cudaSetDevice(ctx->device));
    BTE_CUDA(cudaMemcpyAsync(T, ctx->d_T.p, sizeof(double) * ctx->n, cudaMemcpyDeviceToHost, ctx->stream));
    BTE_CUDA(cudaStreamSynchronize(ctx->stream));
    return BTE_OK;
}

bte_status bte_get_band_temperature(bte_ctx* ctx, double* Tb) {
    if (!ctx || !Tb) return BTE_ERR_INVALID_ARGUMENT;
    if (!ctx->solved) return fail(ctx, BTE_ERR_STATE, "no solution yet");
    BTE_CUDA(cudaSetDevice(ctx->device));
    std::vector<double> tmp((size_t)ctx->n_band * ctx->n);
    BTE_CUDA(cudaMemcpy2DAsync(tmp.data(), sizeof(double) * ctx->n, ctx->d_Tb.p, sizeof(double) * ctx->Np,
                               sizeof(double) * ctx->n, ctx->n_band, cudaMemcpyDeviceToHost, ctx->stream));
    BTE_CUDA(cudaStreamSynchronize(ctx->stream));
    for (int c = 0; c < ctx->n; ++c)
        for (int b = 0; b < ctx->n_band; ++b) Tb[(size_t)c * ctx->n_band + b] = tmp[(size_t)b * ctx->n + c];
    return BTE_OK;
}

bte_status bte_get_heat_flux(bte_ctx* ctx, double* q_bc, double* q_bc_band) {
    if (!ctx || !q_bc) return BTE_ERR_INVALID_ARGUMENT;
    if (!ctx->solved) return fail(ctx, BTE_ERR_STATE, "no solution yet");
    BTE_CUDA(cudaSetDevice(ctx->device));
    if (ctx->n_bc > 0) {
        BTE_CUDA(cudaMemcpyAsync(q_bc, ctx->d_q.p, sizeof(double) * ctx->n_bc, cudaMemcpyDeviceToHost, ctx->stream));
        if (q_bc_band)
            BTE_CUDA(cudaMemcpyAsync(q_bc_band, ctx->d_qband.p, sizeof(double) * ctx->n_bc * ctx->n_band,
                                     cudaMemcpyDeviceToHost, ctx->stream));
    }
    BTE_CUDA(cudaStreamSynchronize(ctx->stream));
    return BTE_OK;
}

bte_status bte_get_energy(bte_ctx* ctx, double* e) {
    if (!ctx || !e) return BTE_ERR_INVALID_ARGUMENT;
    if (!ctx->solved) return fail(ctx, BTE_ERR_STATE, "no solution yet");
    BTE_CUDA(cudaSetDevice(ctx->device));
    BTE_CUDA(cudaMemcpy2DAsync(e, sizeof(double) * ctx->n, ctx->e_curr, sizeof(double) * ctx->Np,
                               sizeof(double) * ctx->n, (size_t)ctx->n_band * ctx->n_dir, cudaMemcpyDeviceToHost,
                               ctx->stream));
    BTE_CUDA(cudaStreamSynchronize(ctx->stream));
    return BTE_OK;
}

bte_status bte_get_margins(bte_ctx* ctx, double* m, int cap, int* n) {
    if (!ctx) return BTE_ERR_INVALID_ARGUMENT;
    int k = (int)ctx->margins.size();
    for (int i = 0; i < k && i < cap && m; ++i) m[i] = ctx->margins[i];
    if (n) *n = k;
    return BTE_OK;
}

bte_status bte_get_kernel_stats(bte_ctx* ctx, bte_kernel_stat* stats, int cap, int* n) {
    if (!ctx) return BTE_ERR_INVALID_ARGUMENT;
    for (int k = 0; k < kNumKinds && k < cap && stats; ++k) stats[k] = ctx->stats[k];
    if (n) *n = kNumKinds;
    return BTE_OK;
}

bte_status bte_get_level_order(bte_ctx* ctx, int d, int* perm, int* lvl, int cap_lvl, int* nlev) {
    if (!ctx || !perm || cap_lvl < 0 || (cap_lvl > 0 && !lvl)) return BTE_ERR_INVALID_ARGUMENT;
    if (!ctx->plan_ready) return fail(ctx, BTE_ERR_STATE, "bte_get_level_order: no sweep plan (solve in the sweep form first)");
    if (d < 0 || d >= ctx->n_dir) return fail(ctx, BTE_ERR_INVALID_ARGUMENT, "bte_get_level_order: direction out of range");
    BTE_CUDA(cudaSetDevice(ctx->device));
    BTE_CUDA(cudaMemcpy(perm, ctx->p_cell.as<int>() + (size_t)d * ctx->n, sizeof(int) * ctx->n,
                        cudaMemcpyDeviceToHost));
    const int l0 = ctx->plan_lvl_off[d], l1 = ctx->plan_lvl_off[d + 1];
    for (int k = 0; k < l1 - l0 && k < cap_lvl; ++k) lvl[k] = ctx->plan_lvl[l0 + k];
    if (nlev) *nlev = l1 - l0 - 1;
    return BTE_OK;
}

bte_status bte_get_sweep_tuning(bte_ctx* ctx, int* group, int* threads, int* ring, int* kernel, float* ms, int cap,
                                int* n) {
    if (!ctx || cap < 0) return BTE_ERR_INVALID_ARGUMENT;
    const int m = (int)ctx->sweep_tune_cand.size();
    if (cap > 0 && (!group || !threads || !ring || !kernel || !ms)) return BTE_ERR_INVALID_ARGUMENT;
    for (int k = 0; k < m && k < cap; ++k) {
        const SweepShape& c = ctx->sweep_tune_cand[k];
        group[k] = c.G;
        threads[k] = c.threads;
        ring[k] = c.W;
        kernel[k] = c.kind();
        ms[k] = ctx->sweep_tune_ms[k];
    }
    if (n) *n = m;
    return BTE_OK;
}

// Single CSR system (the reference's BICGSTAB::init + solve), host buffers.
bte_status bte_bicgstab_csr(int n, const int* rowptr, const int* colind, const double* val, int nnz,
                            const double* b, double* x, int maxit, double tol, int* iterations,
                            int* converged) {
    if (n <= 0 || !rowptr || !colind || !val || !b || !x || nnz < 0 || maxit <= 0 || !(tol > 0))
        return BTE_ERR_INVALID_ARGUMENT;
    if (rowptr[0] != 0 || rowptr[n] != nnz) return BTE_ERR_INVALID_ARGUMENT;
    for (int i = 0; i < n; ++i)
        if (rowptr[i + 1] < rowptr[i]) return BTE_ERR_INVALID_ARGUMENT;
    for (int k = 0; k < nnz; ++k)
        if (colind[k] < 0 || colind[k] >= n) return BTE_ERR_INVALID_ARGUMENT;
    bte_ctx tmp;  // scratch holder for error text and buffers
    bte_ctx* ctx = &tmp;
    int dev = 0;
    BTE_CUDA(cudaGetDevice(&dev));
    BTE_CUDA(cudaStreamCreateWithFlags(&tmp.stream, cudaStreamNonBlocking));
    struct StreamGuard { cudaStream_t s; ~StreamGuard() { cudaStreamSynchronize(s); cudaStreamDestroy(s); } } sg{tmp.stream};
    cudaStream_t st = tmp.stream;
    const size_t Np = (size_t)((n + bte::CH - 1) / bte::CH) * bte::CH;
    const int nchunk = (int)(Np / bte::CH);
    DevBuf d_rp, d_ci, d_v, d_x;
    BTE_CUDA(d_rp.alloc(sizeof(int) * (n + 1)));
    BTE_CUDA(d_ci.alloc(sizeof(int) * std::max(nnz, 1)));
    BTE_CUDA(d_v.alloc(sizeof(double) * std::max(nnz, 1)));
    BTE_CUDA(d_x.alloc(sizeof(double) * Np));
    for (DevBuf* w : {&tmp.w_r, &tmp.w_rw, &tmp.w_p, &tmp.w_ph, &tmp.w_q, &tmp.w_z, &tmp.w_t, &tmp.w_b, &tmp.w_invD})
        BTE_CUDA(w->alloc(sizeof(double) * Np));
    BTE_CUDA(tmp.s_done.alloc(sizeof(int)));
    BTE_CUDA(tmp.s_iters.alloc(sizeof(int)));
    BTE_CUDA(tmp.s_flagA.alloc(sizeof(int) * 2));
    BTE_CUDA(tmp.s_flagB.alloc(sizeof(int) * 2));
    BTE_CUDA(tmp.s_rho.alloc(sizeof(double) * 2));
    BTE_CUDA(tmp.s_alpha.alloc(sizeof(double)));
    BTE_CUDA(tmp.s_omega.alloc(sizeof(double)));
    BTE_CUDA(tmp.s_nrmr.alloc(sizeof(double)));
    BTE_CUDA(tmp.s_nrm0.alloc(sizeof(double)));
    BTE_CUDA(tmp.s_part.alloc(sizeof(double) * 7 * nchunk));
    BTE_CUDA(tmp.s_active.alloc(sizeof(int) * (maxit + 2)));
    BTE_CUDA(cudaMemcpyAsync(d_rp.p, rowptr, sizeof(int) * (n + 1), cudaMemcpyHostToDevice, st));
    if (nnz > 0) {
        BTE_CUDA(cudaMemcpyAsync(d_ci.p, colind, sizeof(int) * nnz, cudaMemcpyHostToDevice, st));
        BTE_CUDA(cudaMemcpyAsync(d_v.p, val, sizeof(double) * nnz, cudaMemcpyHostToDevice, st));
    }
    BTE_CUDA(cudaMemsetAsync(tmp.w_b.p, 0, sizeof(double) * Np, st));
    BTE_CUDA(cudaMemcpyAsync(tmp.w_b.p, b, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    BTE_CUDA(cudaMemsetAsync(tmp.s_active.p, 0, sizeof(int) * (maxit + 2), st));
    bte::CsrOp op{d_rp.as<int>(), d_ci.as<int>(), d_v.as<double>(), d_x.as<double>(), n, Np};
    bte::BicgState bs{tmp.s_done.as<int>(), tmp.s_iters.as<int>(), tmp.s_flagA.as<int>(), tmp.s_flagB.as<int>(),
                      tmp.s_rho.as<double>(), tmp.s_alpha.as<double>(), tmp.s_omega.as<double>(),
                      tmp.s_nrmr.as<double>(), tmp.s_nrm0.as<double>(), nullptr, tmp.s_part.as<double>(),
                      tmp.s_active.as<int>(), 1, nchunk, tol, maxit};
    bte::BicgVecs<double> v{tmp.w_r.as<double>(), tmp.w_rw.as<double>(), tmp.w_p.as<double>(),
                            tmp.w_ph.as<double>(), tmp.w_q.as<double>(), tmp.w_z.as<double>(),
                            tmp.w_t.as<double>(), tmp.w_b.as<double>(), tmp.w_invD.as<double>(), Np};
    dim3 grid(nchunk, 1);
    bte::k_bicg_init<<<grid, bte::THREADS, 0, st>>>(op, v, bs);
    BTE_LAUNCHED();
    bte::k_bicg_init_scalars<<<1, 32, 0, st>>>(bs, nullptr);
    BTE_LAUNCHED();
    int i = 1;
    for (;;) {
        int last = i;
        for (int g = 0; g < kGroup && i <= maxit + 1; ++g, ++i) {
            bte::k_bicg_p<<<grid, bte::THREADS, 0, st>>>(op, v, bs, i);
            BTE_LAUNCHED();
            last = i;
            if (i > maxit) break;
            bte::k_bicg_spmv1<<<grid, bte::THREADS, 0, st>>>(op, v, bs, i);
            BTE_LAUNCHED();
            bte::k_bicg_s<<<grid, bte::THREADS, 0, st>>>(op, v, bs, i);
            BTE_LAUNCHED();
            bte::k_bicg_spmv2<<<grid, bte::THREADS, 0, st>>>(op, v, bs, i);
            BTE_LAUNCHED();
            bte::k_bicg_x<<<grid, bte::THREADS, 0, st>>>(op, v, bs, i);
            BTE_LAUNCHED();
        }
        BTE_CUDA(cudaMemcpyAsync(&tmp.h_done.emplace_back(0), bs.active + last, sizeof(int),
                                 cudaMemcpyDeviceToHost, st));
        BTE_CUDA(cudaStreamSynchronize(st));
        if (tmp.h_done.back() == 0 || last > maxit || i > maxit + 1) break;
    }
    int done = 0, its = 0;
    BTE_CUDA(cudaMemcpyAsync(x, d_x.p, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    BTE_CUDA(cudaMemcpyAsync(&done, bs.done, sizeof(int), cudaMemcpyDeviceToHost, st));
    BTE_CUDA(cudaMemcpyAsync(&its, bs.iters, sizeof(int), cudaMemcpyDeviceToHost, st));
    BTE_CUDA(cudaStreamSynchronize(st));
    if (iterations) *iterations = its;
    if (converged) *converged = (done == 1 || done == 2) ? 1 : 0;
    return BTE_OK;
}

static bte_status dsa_solve_impl(bte_ctx* ctx, int n, int F, const int* nb, const double* W, const double* b,
                                 double* x, double tol, int maxit, int* iterations, double* relres) {
    BTE_CUDA(cudaGetDevice(&ctx->device));
    BTE_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    bte_status s = dsa_prepare(ctx, n, F, nb, W);
    if (s != BTE_OK) return s;
    std::vector<double> bp(n), xp(n);
    for (int k = 0; k < n; ++k) bp[k] = b[ctx->dsa_order[k]];
    BTE_CUDA(cudaMemcpyAsync(ctx->d_dsa_b.p, bp.data(), sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    s = dsa_launch(ctx, n, F, tol, maxit);
    if (s != BTE_OK) return s;
    int stat[4] = {0, 0, 0, 0};
    double rr = 0.0;
    BTE_CUDA(cudaMemcpyAsync(xp.data(), ctx->d_dsa_x.p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    BTE_CUDA(cudaMemcpyAsync(stat, ctx->cg_stat.p, sizeof(stat), cudaMemcpyDeviceToHost, ctx->stream));
    BTE_CUDA(cudaMemcpyAsync(&rr, ctx->cg_relres.p, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    BTE_CUDA(cudaStreamSynchronize(ctx->stream));
    if (stat[1]) return fail(ctx, BTE_ERR_CUDA, "a grid barrier of the low-order solve timed out");
    for (int k = 0; k < n; ++k) x[ctx->dsa_order[k]] = xp[k];
    if (iterations) *iterations = stat[0];
    if (relres) *relres = rr;
    return BTE_OK;
}

bte_status bte_dsa_solve(int n, int n_face, const int* nb, const double* W, const double* b, double* x, double tol,
                         int maxit, int* iterations, double* relres) {
    if (n <= 0 || n_face <= 0 || !nb || !W || !b || !x || !(tol > 0) || maxit <= 0) {
        g_create_error = "bte_dsa_solve: bad size, tolerance, iteration limit or null pointer";
        return BTE_ERR_INVALID_ARGUMENT;
    }
    const size_t nf = (size_t)n * n_face;
    for (size_t q = 0; q < nf; ++q) {
        if (nb[q] < -1 || nb[q] >= n || !(W[q] >= 0.0) || !std::isfinite(W[q]) || !std::isfinite(b[q % n])) {
            g_create_error = "bte_dsa_solve: neighbour index out of range or negative / non-finite value";
            return BTE_ERR_INVALID_ARGUMENT;
        }
    }
    for (int f = 0; f < n_face; ++f)
        for (int c = 0; c < n; ++c) {
            const size_t q = (size_t)f * n + c;
            const int o = nb[q];
            if (o < 0 || W[q] == 0.0) continue;
            bool back = false;
            for (int g = 0; g < n_face && !back; ++g) back = nb[(size_t)g * n + o] == c && W[(size_t)g * n + o] == W[q];
            if (!back || o == c) {
                g_create_error = "bte_dsa_solve: the operator is not symmetric (no matching slot in the neighbour)";
                return BTE_ERR_INVALID_ARGUMENT;
            }
        }
    bte_ctx tmp;
    struct StreamGuard {
        bte_ctx* c;
        ~StreamGuard() {
            if (c->stream) {
                cudaStreamSynchronize(c->stream);
                cudaStreamDestroy(c->stream);
            }
        }
    } guard{&tmp};
    const bte_status s = dsa_solve_impl(&tmp, n, n_face, nb, W, b, x, tol, maxit, iterations, relres);
    if (s != BTE_OK) g_create_error = "bte_dsa_solve: " + tmp.err;
    return s;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free CSR BiCGSTAB (bte_bicgstab_csr_noalloc).
//
// For callers that cannot allocate device memory themselves: code whose
// device memory is owned by another allocator with a fixed budget (a
// framework's caching pool, an embedding application), and code that must not
// trigger the implicit device-wide synchronisation of cudaMalloc/cudaFree in
// the middle of its stream work.  The caller passes device inputs and outputs;
// every work vector, per-system scalar and partial dot product lives in the
// file-scope array below, which every GPU that loads this library holds until
// the process exits (kNoAllocScratchBytes, about 21 MB).
//
// Host code must not pass g_noalloc_scratch itself to a kernel: in host code
// the name is a host-side stand-in, not a device address.  Every call looks up
// the device address with cudaGetSymbolAddress on the current device, so a
// context that was torn down and created again (cudaDeviceReset) is followed;
// the first call on a device also loads this module's device code there and
// should therefore come before any stream capture.  All calls share the one
// array and leave their contents in it: each call clears what must start at
// zero, and calls that overlap on the GPU (different streams or threads at the
// same time) race.
namespace {
constexpr int kNoAllocMaxN = 1 << 18;     // unknowns
constexpr int kNoAllocMaxIt = 10000;      // BiCGSTAB iterations
constexpr size_t kNoAllocNp = ((size_t)kNoAllocMaxN + bte::CH - 1) / bte::CH * bte::CH;
constexpr int kNoAllocChunks = (int)(kNoAllocNp / bte::CH);
// doubles: 10 vectors of kNoAllocNp (r, r_hat, p, p_hat, q, z, t, b, 1/D, x),
// 7 x kNoAllocChunks partials, 8 scalars; then ints (done, iters, flagA[2],
// flagB[2], error flag, spare, active[kNoAllocMaxIt + 2]) packed two per double.
constexpr size_t kNoAllocDoubles = 10 * kNoAllocNp + 7 * (size_t)kNoAllocChunks + 8;
constexpr size_t kNoAllocInts = 8 + (size_t)kNoAllocMaxIt + 2;
constexpr size_t kNoAllocScratch = kNoAllocDoubles + (kNoAllocInts + 1) / 2;
constexpr size_t kNoAllocScratchBytes = kNoAllocScratch * sizeof(double);
static_assert(kNoAllocScratchBytes < (size_t)24 << 20, "the static scratch is documented as about 21 MB");
}  // namespace

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratch];

// Checks a caller's device CSR (row pointers non-decreasing from 0 to nnz,
// column indices in range) before any kernel dereferences it.
__global__ void k_noalloc_check_csr(const int* __restrict__ rowptr, const int* __restrict__ col, int n, int nnz,
                                    int* bad) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t == 0 && (rowptr[0] != 0 || rowptr[n] != nnz)) atomicOr(bad, 1);
    if (t < n && rowptr[t + 1] < rowptr[t]) atomicOr(bad, 1);
    for (int k = t; k < nnz; k += gridDim.x * blockDim.x)
        if (col[k] < 0 || col[k] >= n) atomicOr(bad, 1);
}

// Device address of g_noalloc_scratch in the current device's context.
static cudaError_t noalloc_scratch_address(double** out) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    *out = static_cast<double*>(p);
    return cudaSuccess;
}

// On a failure after kernels were queued on the caller's stream, wait for them
// (ignoring the status) so that no kernel of this call still uses the shared
// array when the call returns.
#define NOALLOC_CUDA(call)                                                            \
    do {                                                                              \
        cudaError_t _e = (call);                                                      \
        if (_e != cudaSuccess) {                                                      \
            g_create_error = std::string("bte_bicgstab_csr_noalloc: ") + #call + ": " + \
                             cudaGetErrorString(_e);                                  \
            if (launched) cudaStreamSynchronize(st);                                  \
            return BTE_ERR_CUDA;                                                      \
        }                                                                             \
    } while (0)

extern "C" bte_status bte_bicgstab_csr_noalloc(int n, const int* rowptr, const int* colind, const double* val,
                                               int nnz, const double* b, double* x, int maxit, double tol,
                                               void* stream, int* iterations, int* converged) {
    if (n <= 0 || n > kNoAllocMaxN) {
        g_create_error = "bte_bicgstab_csr_noalloc: n must be in 1.." + std::to_string(kNoAllocMaxN);
        return BTE_ERR_INVALID_ARGUMENT;
    }
    if (maxit <= 0 || maxit > kNoAllocMaxIt) {
        g_create_error = "bte_bicgstab_csr_noalloc: maxit must be in 1.." + std::to_string(kNoAllocMaxIt);
        return BTE_ERR_INVALID_ARGUMENT;
    }
    if (!rowptr || !colind || !val || !b || !x || nnz < 0 || !(tol > 0)) {
        g_create_error = "bte_bicgstab_csr_noalloc: null pointer, negative nnz or tol <= 0";
        return BTE_ERR_INVALID_ARGUMENT;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    bool launched = false;  // work of this call is queued on st
    double* base = nullptr;
    NOALLOC_CUDA(noalloc_scratch_address(&base));
    const size_t Np = (size_t)((n + bte::CH - 1) / bte::CH) * bte::CH;
    const int nchunk = (int)(Np / bte::CH);
    double* vec[10];
    for (int k = 0; k < 10; ++k) vec[k] = base + (size_t)k * kNoAllocNp;
    double* part = base + 10 * kNoAllocNp;
    double* sc = part + 7 * (size_t)kNoAllocChunks;  // rho[2], alpha, omega, nrmr, nrm0
    int* iv = reinterpret_cast<int*>(base + kNoAllocDoubles);
    int* done = iv;
    int* iters = iv + 1;
    int* flagA = iv + 2;
    int* flagB = iv + 4;
    int* bad = iv + 6;
    int* active = iv + 8;
    // what must start at zero: the error flag, the per-iteration counters and
    // the right-hand side padding (the kernels rewrite everything else)
    launched = true;
    NOALLOC_CUDA(cudaMemsetAsync(iv, 0, sizeof(int) * (8 + (size_t)maxit + 2), st));
    NOALLOC_CUDA(cudaMemsetAsync(vec[7], 0, sizeof(double) * Np, st));
    k_noalloc_check_csr<<<(n + 255) / 256, 256, 0, st>>>(rowptr, colind, n, nnz, bad);
    NOALLOC_CUDA(cudaGetLastError());
    int h_bad = 0;
    NOALLOC_CUDA(cudaMemcpyAsync(&h_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
    NOALLOC_CUDA(cudaStreamSynchronize(st));
    if (h_bad) {
        g_create_error = "bte_bicgstab_csr_noalloc: malformed CSR (row pointers or column indices)";
        return BTE_ERR_INVALID_ARGUMENT;
    }
    NOALLOC_CUDA(cudaMemcpyAsync(vec[7], b, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    bte::CsrOp op{rowptr, colind, val, vec[9], n, Np};
    bte::BicgState bs{done, iters, flagA, flagB, sc, sc + 2, sc + 3, sc + 4, sc + 5, nullptr, part, active, 1, nchunk,
                      tol, maxit};
    bte::BicgVecs<double> v{vec[0], vec[1], vec[2], vec[3], vec[4], vec[5], vec[6], vec[7], vec[8], Np};
    dim3 grid(nchunk, 1);
    bte::k_bicg_init<<<grid, bte::THREADS, 0, st>>>(op, v, bs);
    bte::k_bicg_init_scalars<<<1, 32, 0, st>>>(bs, nullptr);
    NOALLOC_CUDA(cudaGetLastError());
    int i = 1;
    for (;;) {
        int last = i;
        for (int g = 0; g < kGroup && i <= maxit + 1; ++g, ++i) {
            bte::k_bicg_p<<<grid, bte::THREADS, 0, st>>>(op, v, bs, i);
            last = i;
            if (i > maxit) break;
            bte::k_bicg_spmv1<<<grid, bte::THREADS, 0, st>>>(op, v, bs, i);
            bte::k_bicg_s<<<grid, bte::THREADS, 0, st>>>(op, v, bs, i);
            bte::k_bicg_spmv2<<<grid, bte::THREADS, 0, st>>>(op, v, bs, i);
            bte::k_bicg_x<<<grid, bte::THREADS, 0, st>>>(op, v, bs, i);
        }
        NOALLOC_CUDA(cudaGetLastError());
        int h_active = 0;
        NOALLOC_CUDA(cudaMemcpyAsync(&h_active, active + last, sizeof(int), cudaMemcpyDeviceToHost, st));
        NOALLOC_CUDA(cudaStreamSynchronize(st));
        if (h_active == 0 || last > maxit || i > maxit + 1) break;
    }
    NOALLOC_CUDA(cudaMemcpyAsync(x, vec[9], sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    int h_state[2] = {0, 0};
    NOALLOC_CUDA(cudaMemcpyAsync(h_state, done, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
    NOALLOC_CUDA(cudaStreamSynchronize(st));
    if (iterations) *iterations = h_state[1];
    if (converged) *converged = (h_state[0] == 1 || h_state[0] == 2) ? 1 : 0;
    return BTE_OK;
}

// ---------------------------------------------------------------------------
// MLP of the learned accelerator: parameters, inference, gradient, training.

namespace {

// Device buffers of one MLP computation on M rows (batch).
struct MlpWork {
    DevBuf x, y, t, dy, act, dh, p1, p2, p3, part, params, wpack, wi, grad, m, v, idx, xall, yall;
    int M = 0, nslices = 0;
};
constexpr int kRowsPerSlice = 256;

#define MLP_CUDA(call)                                                                          \
    do {                                                                                        \
        cudaError_t _e = (call);                                                                \
        if (_e != cudaSuccess) {                                                                \
            g_create_error = std::string("mlp: ") + #call + ": " + cudaGetErrorString(_e);      \
            return _e == cudaErrorMemoryAllocation ? BTE_ERR_OUT_OF_MEMORY : BTE_ERR_CUDA;      \
        }                                                                                       \
    } while (0)

bte_status mlp_alloc(MlpWork& w, int M) {
    using bf = __nv_bfloat16;
    namespace ml = bte::mlp;
    w.M = M;
    w.nslices = (M + kRowsPerSlice - 1) / kRowsPerSlice;
    MLP_CUDA(w.x.alloc(sizeof(bf) * (size_t)M * ml::IN_PAD));
    MLP_CUDA(w.y.alloc(sizeof(float) * M));
    MLP_CUDA(w.t.alloc(sizeof(float) * M));
    MLP_CUDA(w.dy.alloc(sizeof(float) * M));
    MLP_CUDA(w.act.alloc(sizeof(bf) * 3 * (size_t)M * ml::H));
    MLP_CUDA(w.dh.alloc(sizeof(bf) * 3 * (size_t)M * ml::H));
    MLP_CUDA(w.p1.alloc(sizeof(float) * (size_t)w.nslices * ml::IN_PAD * ml::H));
    MLP_CUDA(w.p2.alloc(sizeof(float) * (size_t)w.nslices * ml::H * ml::H));
    MLP_CUDA(w.p3.alloc(sizeof(float) * (size_t)w.nslices * ml::H * ml::H));
    MLP_CUDA(w.part.alloc(sizeof(double) * 256));
    MLP_CUDA(w.params.alloc(sizeof(float) * ml::NPARAM));
    MLP_CUDA(w.wpack.alloc(sizeof(bf) * ml::PK_N));
    MLP_CUDA(w.wi.alloc(sizeof(bf) * 2 * ml::H * ml::H));
    MLP_CUDA(w.grad.alloc(sizeof(float) * ml::NPARAM));
    MLP_CUDA(cudaFuncSetAttribute(ml::k_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ml::FWD_SMEM));
    MLP_CUDA(cudaFuncSetAttribute(ml::k_backward_data, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)ml::BWD_SMEM));
    return BTE_OK;
}

int mlp_blocks(int M) { return std::max(1, std::min(1024, (M + 63) / 64)); }

// Pack the FP32 parameters in w.params into the kernels' BF16 layouts.
bte_status mlp_pack(MlpWork& w, cudaStream_t st) {
    namespace ml = bte::mlp;
    ml::k_pack<<<(ml::H * ml::H + 255) / 256, 256, 0, st>>>(w.params.as<float>(), w.wpack.as<__nv_bfloat16>());
    ml::k_pack_in_major<<<(ml::H * ml::H + 255) / 256, 256, 0, st>>>(w.params.as<float>(), w.wi.as<__nv_bfloat16>());
    MLP_CUDA(cudaGetLastError());
    return BTE_OK;
}

// Loss and gradient of the rows already in w.x / w.t (M rows) into w.grad; loss to *loss.
bte_status mlp_loss_grad(MlpWork& w, int M, cudaStream_t st, double* loss) {
    namespace ml = bte::mlp;
    using bf = __nv_bfloat16;
    ml::k_forward<<<mlp_blocks(M), 128, ml::FWD_SMEM, st>>>(w.x.as<bf>(), M, w.wpack.as<bf>(), w.params.as<float>(),
                                                          w.y.as<float>(), w.act.as<bf>());
    const int lb = std::min(256, (M + 255) / 256);
    ml::k_loss<<<lb, 256, 0, st>>>(w.y.as<float>(), w.t.as<float>(), M, w.dy.as<float>(), w.part.as<double>());
    ml::k_backward_data<<<mlp_blocks(M), 128, ml::BWD_SMEM, st>>>(w.dy.as<float>(), M, w.act.as<bf>(),
                                                                 w.wi.as<bf>(), w.params.as<float>(), w.dh.as<bf>());
    const int ns = (M + kRowsPerSlice - 1) / kRowsPerSlice;
    ml::k_weight_grad<ml::IN_PAD><<<ns, 256, 0, st>>>(w.x.as<bf>(), ml::IN_PAD, w.dh.as<bf>(), M, kRowsPerSlice,
                                                       w.p1.as<float>());
    ml::k_weight_grad<ml::H><<<ns, 256, 0, st>>>(w.act.as<bf>(), ml::H, w.dh.as<bf>() + (size_t)M * ml::H, M,
                                                 kRowsPerSlice, w.p2.as<float>());
    ml::k_weight_grad<ml::H><<<ns, 256, 0, st>>>(w.act.as<bf>() + (size_t)M * ml::H, ml::H,
                                                 w.dh.as<bf>() + (size_t)2 * M * ml::H, M, kRowsPerSlice,
                                                 w.p3.as<float>());
    ml::k_grad_assemble<<<(ml::NPARAM + 255) / 256, 256, 0, st>>>(w.p1.as<float>(), w.p2.as<float>(),
                                                                   w.p3.as<float>(), ns, w.act.as<bf>(),
                                                                   w.dh.as<bf>(), w.dy.as<float>(), M,
                                                                   w.grad.as<float>());
    MLP_CUDA(cudaGetLastError());
    if (loss) {
        std::vector<double> part(lb);
        MLP_CUDA(cudaMemcpyAsync(part.data(), w.part.p, sizeof(double) * lb, cudaMemcpyDeviceToHost, st));
        MLP_CUDA(cudaStreamSynchronize(st));
        double s = 0;
        for (double v : part) s += v;
        *loss = s;
    }
    return BTE_OK;
}

struct ScopedStream {
    cudaStream_t s = nullptr;
    ~ScopedStream() {
        if (s) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    }
};

}  // namespace

extern "C" {

int bte_mlp_param_count(void) { return bte::mlp::NPARAM; }

bte_status bte_set_centroids(bte_ctx* ctx, const double* centroid) {
    if (!ctx || !centroid) return BTE_ERR_INVALID_ARGUMENT;
    if (!ctx->has_geom) return fail(ctx, BTE_ERR_STATE, "bte_set_centroids: set the geometry first");
    ctx->centroid.assign(centroid, centroid + 3 * (size_t)ctx->n);
    for (double v : ctx->centroid)
        if (!std::isfinite(v)) return fail(ctx, BTE_ERR_INVALID_ARGUMENT, "bte_set_centroids: non-finite value");
    return BTE_OK;
}

bte_status bte_set_mlp(bte_ctx* ctx, const float* params) {
    if (!ctx || !params) return BTE_ERR_INVALID_ARGUMENT;
    namespace ml = bte::mlp;
    for (int i = 0; i < ml::NPARAM; ++i)
        if (!std::isfinite(params[i])) return fail(ctx, BTE_ERR_INVALID_ARGUMENT, "bte_set_mlp: non-finite parameter");
    BTE_CUDA(cudaSetDevice(ctx->device));
    BTE_CUDA(ctx->d_params.alloc(sizeof(float) * ml::NPARAM));
    BTE_CUDA(ctx->d_wpack.alloc(sizeof(__nv_bfloat16) * ml::PK_N));
    BTE_CUDA(cudaMemcpyAsync(ctx->d_params.p, params, sizeof(float) * ml::NPARAM, cudaMemcpyHostToDevice, ctx->stream));
    ml::k_pack<<<(ml::H * ml::H + 255) / 256, 256, 0, ctx->stream>>>(ctx->d_params.as<float>(),
                                                                     ctx->d_wpack.as<__nv_bfloat16>());
    BTE_LAUNCHED();
    BTE_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->has_mlp = true;
    return BTE_OK;
}

bte_status bte_get_history(bte_ctx* ctx, double* T, int cap_iters, int* n_iters) {
    if (!ctx) return BTE_ERR_INVALID_ARGUMENT;
    if (n_iters) *n_iters = ctx->history_rows;
    if (T && cap_iters > 0) {
        const size_t rows = (size_t)std::min(cap_iters, ctx->history_rows);
        std::memcpy(T, ctx->history.data(), sizeof(double) * rows * ctx->n);
    }
    return BTE_OK;
}

bte_status bte_mlp_predict(const float* X, int M, const float* params, float* y) {
    namespace ml = bte::mlp;
    if (!X || !params || !y || M <= 0) return BTE_ERR_INVALID_ARGUMENT;
    ScopedStream ss;
    MLP_CUDA(cudaStreamCreateWithFlags(&ss.s, cudaStreamNonBlocking));
    MlpWork w;
    bte_status rc = mlp_alloc(w, M);
    if (rc) return rc;
    DevBuf xf;
    MLP_CUDA(xf.alloc(sizeof(float) * (size_t)M * ml::IN));
    MLP_CUDA(cudaMemcpyAsync(xf.p, X, sizeof(float) * (size_t)M * ml::IN, cudaMemcpyHostToDevice, ss.s));
    MLP_CUDA(cudaMemcpyAsync(w.params.p, params, sizeof(float) * ml::NPARAM, cudaMemcpyHostToDevice, ss.s));
    ml::k_features_bf16<<<(M * ml::IN_PAD + 255) / 256, 256, 0, ss.s>>>(xf.as<float>(), M, w.x.as<__nv_bfloat16>());
    rc = mlp_pack(w, ss.s);
    if (rc) return rc;
    ml::k_forward<<<mlp_blocks(M), 128, ml::FWD_SMEM, ss.s>>>(w.x.as<__nv_bfloat16>(), M, w.wpack.as<__nv_bfloat16>(),
                                                            w.params.as<float>(), w.y.as<float>(), nullptr);
    MLP_CUDA(cudaGetLastError());
    MLP_CUDA(cudaMemcpyAsync(y, w.y.p, sizeof(float) * M, cudaMemcpyDeviceToHost, ss.s));
    MLP_CUDA(cudaStreamSynchronize(ss.s));
    return BTE_OK;
}

bte_status bte_mlp_gradient(const float* X, const float* Y, int M, const float* params, float* grad, double* loss) {
    namespace ml = bte::mlp;
    if (!X || !Y || !params || !grad || M <= 0) return BTE_ERR_INVALID_ARGUMENT;
    ScopedStream ss;
    MLP_CUDA(cudaStreamCreateWithFlags(&ss.s, cudaStreamNonBlocking));
    MlpWork w;
    bte_status rc = mlp_alloc(w, M);
    if (rc) return rc;
    DevBuf xf;
    MLP_CUDA(xf.alloc(sizeof(float) * (size_t)M * ml::IN));
    MLP_CUDA(cudaMemcpyAsync(xf.p, X, sizeof(float) * (size_t)M * ml::IN, cudaMemcpyHostToDevice, ss.s));
    MLP_CUDA(cudaMemcpyAsync(w.t.p, Y, sizeof(float) * M, cudaMemcpyHostToDevice, ss.s));
    MLP_CUDA(cudaMemcpyAsync(w.params.p, params, sizeof(float) * ml::NPARAM, cudaMemcpyHostToDevice, ss.s));
    ml::k_features_bf16<<<(M * ml::IN_PAD + 255) / 256, 256, 0, ss.s>>>(xf.as<float>(), M, w.x.as<__nv_bfloat16>());
    rc = mlp_pack(w, ss.s);
    if (rc) return rc;
    rc = mlp_loss_grad(w, M, ss.s, loss);
    if (rc) return rc;
    MLP_CUDA(cudaMemcpyAsync(grad, w.grad.p, sizeof(float) * ml::NPARAM, cudaMemcpyDeviceToHost, ss.s));
    MLP_CUDA(cudaStreamSynchronize(ss.s));
    return BTE_OK;
}

bte_status bte_mlp_train(const float* X, const float* Y, int M, int steps, int batch, float lr, unsigned seed,
                         float* params, float* loss_hist) {
    namespace ml = bte::mlp;
    using bf = __nv_bfloat16;
    if (!X || !Y || !params || M <= 0 || steps <= 0 || batch <= 0 || !(lr > 0)) return BTE_ERR_INVALID_ARGUMENT;
    batch = std::min(batch, M);
    ScopedStream ss;
    MLP_CUDA(cudaStreamCreateWithFlags(&ss.s, cudaStreamNonBlocking));
    cudaStream_t st = ss.s;
    MlpWork w;
    bte_status rc = mlp_alloc(w, batch);
    if (rc) return rc;
    DevBuf xf;
    MLP_CUDA(xf.alloc(sizeof(float) * (size_t)M * ml::IN));
    MLP_CUDA(w.xall.alloc(sizeof(bf) * (size_t)M * ml::IN_PAD));
    MLP_CUDA(w.yall.alloc(sizeof(float) * M));
    MLP_CUDA(w.idx.alloc(sizeof(int) * M));
    MLP_CUDA(w.m.alloc(sizeof(float) * ml::NPARAM));
    MLP_CUDA(w.v.alloc(sizeof(float) * ml::NPARAM));
    MLP_CUDA(cudaMemsetAsync(w.m.p, 0, sizeof(float) * ml::NPARAM, st));
    MLP_CUDA(cudaMemsetAsync(w.v.p, 0, sizeof(float) * ml::NPARAM, st));
    MLP_CUDA(cudaMemcpyAsync(xf.p, X, sizeof(float) * (size_t)M * ml::IN, cudaMemcpyHostToDevice, st));
    MLP_CUDA(cudaMemcpyAsync(w.yall.p, Y, sizeof(float) * M, cudaMemcpyHostToDevice, st));
    MLP_CUDA(cudaMemcpyAsync(w.params.p, params, sizeof(float) * ml::NPARAM, cudaMemcpyHostToDevice, st));
    ml::k_features_bf16<<<(M * ml::IN_PAD + 255) / 256, 256, 0, st>>>(xf.as<float>(), M, w.xall.as<bf>());
    MLP_CUDA(cudaGetLastError());
    std::mt19937 rng(seed);
    std::vector<int> perm(M);
    for (int i = 0; i < M; ++i) perm[i] = i;
    int pos = M;  // force a shuffle on the first step
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    float c1 = 1.f, c2 = 1.f;
    for (int step = 0; step < steps; ++step) {
        if (pos + batch > M) {
            std::shuffle(perm.begin(), perm.end(), rng);
            MLP_CUDA(cudaMemcpyAsync(w.idx.p, perm.data(), sizeof(int) * M, cudaMemcpyHostToDevice, st));
            MLP_CUDA(cudaStreamSynchronize(st));  // perm is reshuffled on the host next time
            pos = 0;
        }
        ml::k_gather<<<(batch * ml::IN_PAD + 255) / 256, 256, 0, st>>>(w.xall.as<bf>(), w.yall.as<float>(),
                                                                       w.idx.as<int>() + pos, batch, w.x.as<bf>(),
                                                                       w.t.as<float>());
        pos += batch;
        rc = mlp_pack(w, st);
        if (rc) return rc;
        double loss = 0;
        rc = mlp_loss_grad(w, batch, st, loss_hist ? &loss : nullptr);
        if (rc) return rc;
        if (loss_hist) loss_hist[step] = (float)loss;
        c1 *= b1;
        c2 *= b2;
        ml::k_adam<<<(ml::NPARAM + 255) / 256, 256, 0, st>>>(w.params.as<float>(), w.grad.as<float>(), w.m.as<float>(),
                                                              w.v.as<float>(), lr, b1, b2, eps, 1.f - c1, 1.f - c2);
        MLP_CUDA(cudaGetLastError());
    }
    MLP_CUDA(cudaMemcpyAsync(params, w.params.p, sizeof(float) * ml::NPARAM, cudaMemcpyDeviceToHost, st));
    MLP_CUDA(cudaStreamSynchronize(st));
    return BTE_OK;
}

}  // extern "C"
