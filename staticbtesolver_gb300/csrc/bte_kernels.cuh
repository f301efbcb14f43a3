// bte_kernels.cuh -- sm_103a kernels of the batched DOM-FVM phonon BTE solve.
//
// Data layout in HBM (Np = n_cell rounded up to CH; padded cells carry an
// identity row and a zero right-hand side, so they stay zero and never enter
// a dot product):
//   e_curr/e_prev   [n_band][n_dir][Np]  FP64, the reference's ee_curr/ee_prev
//                                        (src/StaticBTESolver.cpp:702-717)
//   dg, vo          [n_dir][Np]          per-direction diagonal geometry
//   fc              [n_dir][n_face][Np]  per-direction inflow face coefficients
//   nb              [n_face][Np]         neighbour cell (self when none)
//   BiCGSTAB work   [batch systems][Np]  one row per (band, direction) system
//
// A (band b, direction d) system of the reference (_get_Ke, :122-160) is
//   A[c][c]      = k_b * sum_{outflow f} A_cf g_dcf + V_c Omega_d      (1D: + V_c)
//   A[c][nb(c,f)] = k_b * A_cf g_dcf            for inflow faces with a neighbour
// with k_b = v_g,b tau_b and g_dcf = S_d . n_cf (1D: s_d . n_cf), so it is
// applied matrix-free from band-independent per-direction geometry:
//   (A x)[c] = (k_b dg[d][c] + vo[d][c]) x[c] + k_b sum_f fc[d][f][c] x[nb[f][c]].
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace bte {

constexpr int THREADS = 256;
constexpr int CPT = 8;                 // cells per thread per chunk
constexpr int CH = THREADS * CPT;      // cells per block ("chunk")
constexpr int NWARP = THREADS / 32;

// ----------------------------------------------------------------------------
// Deterministic block reductions (fixed shuffle tree + fixed warp order).
template <int K>
__device__ __forceinline__ void block_sum(double (&v)[K], double (*smem)[NWARP]) {
#pragma unroll
    for (int k = 0; k < K; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < K; ++k) smem[k][warp] = v[k];
    __syncthreads();
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < K; ++k) {
            double s = 0;
#pragma unroll
            for (int w = 0; w < NWARP; ++w) s += smem[k][w];
            v[k] = s;
        }
}

// Serial sum of the per-chunk partials (for kernels with one thread per system).
__device__ __forceinline__ double sum_parts_serial(const double* p, int n) {
    double s = 0;
    for (int i = 0; i < n; ++i) s += p[i];
    return s;
}

// Fused multiply-add in the vector type: fmaf for float, fma for double
// (a plain fma() on floats would promote them to FP64).
__device__ __forceinline__ float fmat(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fmat(double a, double b, double c) { return fma(a, b, c); }

// Sum of the per-chunk partials of one system.  Each warp loads them in
// parallel (lane l sums partials l, l+32, ... in order) and combines the lanes
// with a fixed butterfly, so every warp of every block gets the same value
// and the order never depends on timing.  Must be called by whole warps.
__device__ __forceinline__ double sum_parts(const double* p, int n) {
    const int lane = threadIdx.x & 31;
    double s = 0;
    for (int i = lane; i < n; i += 32) s += p[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return s;
}

// ----------------------------------------------------------------------------
// Batched BiCGSTAB state.  One row per system y of the batch.
struct BicgState {
    int* done;        // 0 active, 1 converged, 2 zero residual, 3 iteration limit
    int* iters;       // iterations used (set when done)
    int* flagA;       // [2][S] restart in the p-update phase of iteration parity
    int* flagB;       // [2][S] restart in the s-update phase
    double* rho;      // [2][S]
    double* alpha;    // [S]
    double* omega;    // [S]
    double* nrmr;     // [S] last ||r||
    double* nrm0;     // [S] ||b||
    double* bestr;    // [2][S] smallest ||r|| so far (used when BicgVecs::xb is set)
    double* part;     // [7][S][nchunk] partial dot products
    int* active;      // [maxit + 2] number of active systems at each iteration
    int S, nchunk;
    double tol;
    int maxit;
    int cycles = 1;   // with BicgVecs::xb: the iteration limit is cycles x maxit
    int track_from = 0;  // with BicgVecs::xb: iterations before this are not candidates
    __device__ double* P(int kind, int y) const { return part + ((size_t)kind * S + y) * nchunk; }
};
enum { PK_RR0 = 0, PK_RR1 = 1, PK_RWR0 = 2, PK_RWR1 = 3, PK_RWQ = 4, PK_TS = 5, PK_TT = 6 };

// xb (optional, nullptr to follow the reference exactly): the iterate with the
// smallest residual norm after iteration BicgState::track_from (x = 0 before),
// returned instead of the last one when the iteration limit (cycles x maxit)
// is reached or the residual stops being finite.
template <typename T>
struct BicgVecs {
    T* r; T* rw; T* p; T* ph; T* q; T* z; T* t; const T* b; T* invD;
    size_t Np;
    T* xb = nullptr;
};

// Matrix-free upwind operator of all (band, direction) systems of a batch.
// Batch row y -> direction y / nbb, band b0 + y % nbb (the bands of one
// direction are adjacent so they share that direction's geometry in L2).
struct FaceFluxOp {
    const double* dg;
    const double* vo;
    const double* fc;
    const int* nb;
    const double* kb;  // k_b = v_g tau per band
    double* x_out;     // e_curr base [n_band][n_dir][Np]
    int F, nbb, b0, n_dir;
    size_t Np;
    __device__ __forceinline__ void bd(int y, int& b, int& d) const {
        d = y / nbb;
        b = b0 + y % nbb;
    }
    __device__ __forceinline__ double* x_of(int y) const {
        int b, d;
        bd(y, b, d);
        return x_out + ((size_t)b * n_dir + d) * Np;
    }
    __device__ __forceinline__ double inv_diag(int y, int c) const {
        int b, d;
        bd(y, b, d);
        return 1.0 / fma(kb[b], dg[(size_t)d * Np + c], vo[(size_t)d * Np + c]);
    }
    template <typename T>
    __device__ __forceinline__ T apply(int y, int c, const T* __restrict__ xs) const {
        int b, d;
        bd(y, b, d);
        const double k = kb[b];
        const size_t dc = (size_t)d * Np + c;
        double acc = fma(k, dg[dc], vo[dc]) * (double)xs[c];
        double off = 0.0;
        for (int f = 0; f < F; ++f)
            off = fma(fc[((size_t)d * F + f) * Np + c], (double)xs[nb[(size_t)f * Np + c]], off);
        return (T)fma(k, off, acc);
    }
    // (A M v)[c] with M = 1/D (the Jacobi preconditioner) and ph = M v: the
    // diagonal term D (M v)[c] is v[c] itself, so only the inflow coupling is
    // computed -- 2 FP64 operations per cell fewer than apply(ph), which
    // matters on GB300's FP64 pipe.  Equal to apply(ph) up to rounding.
    template <typename T>
    __device__ __forceinline__ T apply_pc(int y, int c, const T* __restrict__ ph, const T* __restrict__ v) const {
        int b, d;
        bd(y, b, d);
        double off = 0.0;
        for (int f = 0; f < F; ++f)
            off = fma(fc[((size_t)d * F + f) * Np + c], (double)ph[nb[(size_t)f * Np + c]], off);
        return (T)fma(kb[b], off, (double)v[c]);
    }
};

// One or more independent CSR systems (the reference's BICGSTAB boundary).
struct CsrOp {
    const int* rowptr;
    const int* col;
    const double* val;
    double* x_out;
    int n;
    size_t Np;
    __device__ __forceinline__ double* x_of(int) const { return x_out; }
    // src/bicgstab.hpp:122-131: 1 / (last stored diagonal entry), 0 for a row
    // without one
    __device__ __forceinline__ double inv_diag(int, int c) const {
        if (c >= n) return 1.0;
        double inv = 0.0;
        for (int k = rowptr[c]; k < rowptr[c + 1]; ++k)
            if (col[k] == c) inv = 1.0 / val[k];
        return inv;
    }
    template <typename T>
    __device__ __forceinline__ T apply(int, int c, const T* __restrict__ xs) const {
        if (c >= n) return xs[c];
        double s = 0.0;
        for (int k = rowptr[c]; k < rowptr[c + 1]; ++k) s = fma(val[k], (double)xs[col[k]], s);
        return (T)s;
    }
    // a general CSR matrix: A (M v) computed as A ph (the reference's SpMV)
    template <typename T>
    __device__ __forceinline__ T apply_pc(int y, int c, const T* __restrict__ ph, const T* __restrict__) const {
        return apply<T>(y, c, ph);
    }
};

#define BTE_CELL_LOOP_K(c, chunk)                                            \
    _Pragma("unroll") for (int _k = 0, c = (chunk) * CH + threadIdx.x; _k < CPT; ++_k, c += THREADS)
#define BTE_CELL_LOOP(c) BTE_CELL_LOOP_K(c, blockIdx.x)

// The vector-update kernels load a group of GRP cells' operands into registers
// before computing and storing any of them, so each thread keeps GRP x (number
// of operands) loads in flight.
constexpr int GRP = 4;
#define BTE_GROUP_LOOP_K(c0, chunk)                                          \
    _Pragma("unroll") for (int c0 = (chunk) * CH + threadIdx.x; c0 < ((chunk) + 1) * CH; c0 += GRP * THREADS)
#define BTE_GROUP_LOOP(c0) BTE_GROUP_LOOP_K(c0, (int)blockIdx.x)

// FP32 counterpart of FaceFluxOp for the mixed form: per-direction geometry
// stored in FP32 and pre-scaled by kappa_d = 1 / mean(V Omega_d), so the
// scaled operator's entries are O(1..1e3) and no FP32 product under- or
// overflows.  The unknown is the batch-local correction dx[y][Np].
struct FaceFluxOp32 {
    const float* dg;
    const float* vo;
    const float* fc;
    const int* nb;
    const float* kb;
    float* dx;
    int F, nbb, b0, n_dir;
    size_t Np;
    __device__ __forceinline__ void bd(int y, int& b, int& d) const {
        d = y / nbb;
        b = b0 + y % nbb;
    }
    __device__ __forceinline__ float* x_of(int y) const { return dx + (size_t)y * Np; }
    __device__ __forceinline__ float inv_diag(int y, int c) const {
        int b, d;
        bd(y, b, d);
        return 1.0f / fmaf(kb[b], dg[(size_t)d * Np + c], vo[(size_t)d * Np + c]);
    }
    template <typename T>
    __device__ __forceinline__ T apply(int y, int c, const T* __restrict__ xs) const {
        int b, d;
        bd(y, b, d);
        const float k = kb[b];
        const size_t dc = (size_t)d * Np + c;
        const float acc = fmaf(k, dg[dc], vo[dc]) * (float)xs[c];
        float off = 0.0f;
        for (int f = 0; f < F; ++f) off = fmaf(fc[((size_t)d * F + f) * Np + c], (float)xs[nb[(size_t)f * Np + c]], off);
        return (T)fmaf(k, off, acc);
    }
    template <typename T>
    __device__ __forceinline__ T apply_pc(int y, int c, const T* __restrict__ ph, const T* __restrict__ v) const {
        int b, d;
        bd(y, b, d);
        float off = 0.0f;
        for (int f = 0; f < F; ++f) off = fmaf(fc[((size_t)d * F + f) * Np + c], (float)ph[nb[(size_t)f * Np + c]], off);
        return (T)fmaf(kb[b], off, (float)v[c]);
    }
};

// K0: x = 0, r = p = r_hat = b, q = 0, invD; partial ||b||^2 (src/bicgstab.hpp:146-162).
// With rho_0 = alpha = omega = 1 the reference's first update is
// p_1 = r + ||b||^2 b: the same direction scaled by 1 + ||b||^2, harmless in
// FP64 but an FP32 overflow once ||b||^2 exceeds ~1e19 (t.t and r_hat.q become
// inf - inf).  The FP32 solve therefore starts from p_0 = 0, so p_1 = r.
template <typename Op, typename T>
__global__ void __launch_bounds__(THREADS) k_bicg_init(Op op, BicgVecs<T> v, BicgState st) {
    __shared__ double sm[2][NWARP];
    const int y = blockIdx.y;
    const size_t o = (size_t)y * v.Np;
    T* x = op.x_of(y);
    T acc_t = 0;
    BTE_CELL_LOOP(c) {
        const T bb = v.b[o + c];
        v.invD[o + c] = (T)op.inv_diag(y, c);
        v.r[o + c] = bb; v.rw[o + c] = bb; v.q[o + c] = 0;
        if constexpr (sizeof(T) == sizeof(float)) v.p[o + c] = 0;
        else v.p[o + c] = bb;
        if (v.xb) v.xb[o + c] = 0;
        x[c] = 0;
        acc_t = fmat(bb, bb, acc_t);
    }
    double acc[2] = {(double)acc_t, (double)acc_t};
    block_sum<2>(acc, sm);
    if (threadIdx.x == 0) {
        st.P(PK_RR0, y)[blockIdx.x] = acc[0];
        st.P(PK_RWR0, y)[blockIdx.x] = acc[1];
    }
}

// One thread per system: scalars after K0.  skip[y] != 0 (optional) marks a
// system that needs no solve this time (done = 4).
__global__ void k_bicg_init_scalars(BicgState st, const int* skip) {
    int y = blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= st.S) return;
    double n0 = sqrt(sum_parts_serial(st.P(PK_RR0, y), st.nchunk));
    st.nrm0[y] = n0;
    st.nrmr[y] = n0;
    if (st.bestr) st.bestr[y] = st.bestr[st.S + y] = n0;  // x0 = 0 has ||r|| = ||b||
    st.rho[y] = 1.0; st.rho[st.S + y] = 1.0;
    st.alpha[y] = 1.0; st.omega[y] = 1.0;
    st.done[y] = (skip && skip[y]) ? 4 : 0;
    st.iters[y] = 0;
    st.flagA[y] = st.flagA[st.S + y] = 0;
    st.flagB[y] = st.flagB[st.S + y] = 0;
}

// Breakdown restart on this block's chunk (src/bicgstab.hpp:170-179, :224-234):
// x = q = p = 0, r = b, r_hat = 6.8 b + 0.6; partial r_hat.r for the next rho.
template <typename Op, typename T>
__device__ __forceinline__ void bicg_restart_chunk(const Op& op, const BicgVecs<T>& v, const BicgState& st, int y,
                                                   int par, int chunk, double (*sm)[NWARP]) {
    const size_t o = (size_t)y * v.Np;
    T* x = op.x_of(y);
    T acc_t = 0;
    BTE_CELL_LOOP_K(c, chunk) {
        // Padded cells get r_hat = 0.6 but keep r = p = q = 0, so they add
        // nothing to any dot product.
        const T bb = v.b[o + c];
        const T rh = bb * (T)6.8 + (T)0.6;
        x[c] = 0; v.q[o + c] = 0; v.p[o + c] = 0; v.r[o + c] = bb;
        v.rw[o + c] = rh;
        acc_t = fmat(rh, bb, acc_t);
    }
    double acc[1] = {(double)acc_t};
    block_sum<1>(acc, sm);
    if (threadIdx.x == 0) st.P(par ? PK_RWR1 : PK_RWR0, y)[chunk] = acc[0];
}

// K1 (iteration i): convergence bookkeeping, rho, beta; p = r + beta (p - omega q); ph = M p.
template <typename Op, typename T>
__device__ __forceinline__ void bicg_p_body(const Op& op, const BicgVecs<T>& v, const BicgState& st, int i, int y,
                                          int chunk, double (*sm)[NWARP]) {
    if (st.done[y]) return;
    const int par = i & 1, pp = par ^ 1;
    const bool lead = chunk == 0 && threadIdx.x == 0;
    double nr;
    bool fresh = false;  // nr is the residual norm of the current x
    if (i > 1 && !(st.flagA[pp * st.S + y] | st.flagB[pp * st.S + y])) {
        nr = sqrt(sum_parts(st.P(pp ? PK_RR1 : PK_RR0, y), st.nchunk));
        if (nr / st.nrm0[y] < st.tol) {  // src/bicgstab.hpp:295
            if (lead) { st.done[y] = 1; st.iters[y] = i - 1; }
            return;
        }
        if (lead) st.nrmr[y] = nr;
        fresh = true;
    } else {
        nr = st.nrmr[y];
    }
    const size_t ox = (size_t)y * v.Np;
    T* __restrict__ xcur = op.x_of(y);
    if (v.xb) {
        const double best = st.bestr[pp * st.S + y];
        const bool improved = fresh && i > st.track_from && nr < best;  // false for NaN
        const double best_now = improved ? nr : best;
        if (lead) st.bestr[par * st.S + y] = best_now;
        if (i > st.maxit * st.cycles || !(nr <= 1.0e300)) {  // limit reached or the iteration blew up
            if (!improved)
                BTE_CELL_LOOP_K(c, chunk) { xcur[c] = v.xb[ox + c]; }
            if (lead) { st.done[y] = 3; st.iters[y] = i - 1; }
            return;
        }
        if (improved)
            BTE_CELL_LOOP_K(c, chunk) { v.xb[ox + c] = xcur[c]; }
    } else if (i > st.maxit) {
        if (lead) { st.done[y] = 3; st.iters[y] = st.maxit; }
        return;
    }
    if (nr < 1e-50) {  // src/bicgstab.hpp:166
        if (lead) { st.done[y] = 2; st.iters[y] = i - 1; }
        return;
    }
    if (lead) atomicAdd(&st.active[i], 1);
    const double rho_new = sum_parts(st.P(pp ? PK_RWR1 : PK_RWR0, y), st.nchunk);
    if (rho_new < 1e-200 && rho_new > -1e-200) {
        if (lead) {
            st.rho[par * st.S + y] = 1.0; st.alpha[y] = 1.0; st.omega[y] = 1.0;
            st.flagA[par * st.S + y] = 1; st.flagB[par * st.S + y] = 0;
        }
        bicg_restart_chunk(op, v, st, y, par, chunk, sm);
        return;
    }
    const double beta = (rho_new / st.rho[pp * st.S + y]) * (st.alpha[y] / st.omega[y]);
    const T om = (T)st.omega[y], bt = (T)beta;
    if (lead) {
        st.rho[par * st.S + y] = rho_new;
        st.flagA[par * st.S + y] = 0; st.flagB[par * st.S + y] = 0;
    }
    const size_t o = (size_t)y * v.Np;
    // restrict-qualified row pointers: the unrolled cell loop may issue all
    // its loads before the first store
    const T* __restrict__ q = v.q + o;
    const T* __restrict__ r = v.r + o;
    const T* __restrict__ iD = v.invD + o;
    T* __restrict__ p = v.p + o;
    T* __restrict__ ph = v.ph + o;
    BTE_GROUP_LOOP_K(c0, chunk) {
        T qv[GRP], pv[GRP], rv[GRP], dv[GRP];
#pragma unroll
        for (int k = 0; k < GRP; ++k) {
            const int c = c0 + k * THREADS;
            qv[k] = q[c]; pv[k] = p[c]; rv[k] = r[c]; dv[k] = iD[c];
        }
#pragma unroll
        for (int k = 0; k < GRP; ++k) {
            const int c = c0 + k * THREADS;
            // cublasDaxpy(-omega, q, p); cublasDscal(beta, p); cublasDaxpy(1, r, p)
            T u = fmat(-om, qv[k], pv[k]);
            u = fmat(bt, u, rv[k]);
            p[c] = u;
            ph[c] = dv[k] * u;
        }
    }
}

template <typename Op, typename T>
__global__ void __launch_bounds__(THREADS) k_bicg_p(Op op, BicgVecs<T> v, BicgState st, int i) {
    __shared__ double sm[2][NWARP];
    bicg_p_body(op, v, st, i, (int)blockIdx.y, (int)blockIdx.x, sm);
}

// K2: q = A ph (= A M p); partial r_hat . q
template <typename Op, typename T>
__device__ __forceinline__ void bicg_spmv1_body(const Op& op, const BicgVecs<T>& v, const BicgState& st, int i, int y,
                                          int chunk, double (*sm)[NWARP]) {
    const int par = i & 1;
    if (st.done[y] | st.flagA[par * st.S + y]) return;
    const size_t o = (size_t)y * v.Np;
    const T* __restrict__ ph = v.ph + o;
    const T* __restrict__ pv = v.p + o;
    const T* __restrict__ rw = v.rw + o;
    T* __restrict__ q = v.q + o;
    T acc_t = 0;
    BTE_CELL_LOOP_K(c, chunk) {
        const T qv = op.template apply_pc<T>(y, c, ph, pv);
        q[c] = qv;
        acc_t = fmat(rw[c], qv, acc_t);
    }
    double acc[1] = {(double)acc_t};
    block_sum<1>(acc, sm);
    if (threadIdx.x == 0) st.P(PK_RWQ, y)[chunk] = acc[0];
}

template <typename Op, typename T>
__global__ void __launch_bounds__(THREADS) k_bicg_spmv1(Op op, BicgVecs<T> v, BicgState st, int i) {
    __shared__ double sm[1][NWARP];
    bicg_spmv1_body(op, v, st, i, (int)blockIdx.y, (int)blockIdx.x, sm);
}

// K3: alpha; s = r - alpha q (in place in r); z = M s
template <typename Op, typename T>
__device__ __forceinline__ void bicg_s_body(const Op& op, const BicgVecs<T>& v, const BicgState& st, int i, int y,
                                          int chunk, double (*sm)[NWARP]) {
    const int par = i & 1;
    if (st.done[y] | st.flagA[par * st.S + y]) return;
    const bool lead = chunk == 0 && threadIdx.x == 0;
    const double temp = sum_parts(st.P(PK_RWQ, y), st.nchunk);
    if (temp < 1e-200 && temp > -1e-200) {
        if (lead) {
            st.rho[par * st.S + y] = 1.0; st.alpha[y] = 1.0; st.omega[y] = 1.0;
            st.flagB[par * st.S + y] = 1;
        }
        bicg_restart_chunk(op, v, st, y, par, chunk, sm);
        return;
    }
    const double alpha = st.rho[par * st.S + y] / temp;
    if (lead) st.alpha[y] = alpha;
    const T al = (T)alpha;
    const size_t o = (size_t)y * v.Np;
    const T* __restrict__ q = v.q + o;
    const T* __restrict__ iD = v.invD + o;
    T* __restrict__ r = v.r + o;
    T* __restrict__ z = v.z + o;
    BTE_GROUP_LOOP_K(c0, chunk) {
        T qv[GRP], rv[GRP], dv[GRP];
#pragma unroll
        for (int k = 0; k < GRP; ++k) {
            const int c = c0 + k * THREADS;
            qv[k] = q[c]; rv[k] = r[c]; dv[k] = iD[c];
        }
#pragma unroll
        for (int k = 0; k < GRP; ++k) {
            const int c = c0 + k * THREADS;
            const T sv = fmat(-al, qv[k], rv[k]);
            r[c] = sv;
            z[c] = dv[k] * sv;
        }
    }
}

template <typename Op, typename T>
__global__ void __launch_bounds__(THREADS) k_bicg_s(Op op, BicgVecs<T> v, BicgState st, int i) {
    __shared__ double sm[1][NWARP];
    bicg_s_body(op, v, st, i, (int)blockIdx.y, (int)blockIdx.x, sm);
}

// K4: t = A z (= A M s); partials t.s, t.t
template <typename Op, typename T>
__device__ __forceinline__ void bicg_spmv2_body(const Op& op, const BicgVecs<T>& v, const BicgState& st, int i, int y,
                                          int chunk, double (*sm)[NWARP]) {
    const int par = i & 1;
    if (st.done[y] | st.flagA[par * st.S + y] | st.flagB[par * st.S + y]) return;
    const size_t o = (size_t)y * v.Np;
    const T* __restrict__ z = v.z + o;
    const T* __restrict__ sv = v.r + o;  // s, stored in r by K3
    T* __restrict__ t = v.t + o;
    T a0 = 0, a1 = 0;
    BTE_CELL_LOOP_K(c, chunk) {
        const T tv = op.template apply_pc<T>(y, c, z, sv);
        t[c] = tv;
        a0 = fmat(tv, sv[c], a0);
        a1 = fmat(tv, tv, a1);
    }
    double acc[2] = {(double)a0, (double)a1};
    block_sum<2>(acc, sm);
    if (threadIdx.x == 0) {
        st.P(PK_TS, y)[chunk] = acc[0];
        st.P(PK_TT, y)[chunk] = acc[1];
    }
}

template <typename Op, typename T>
__global__ void __launch_bounds__(THREADS) k_bicg_spmv2(Op op, BicgVecs<T> v, BicgState st, int i) {
    __shared__ double sm[2][NWARP];
    bicg_spmv2_body(op, v, st, i, (int)blockIdx.y, (int)blockIdx.x, sm);
}

// K5: omega; x += alpha ph; x += omega z; r = s - omega t; partials r.r, r_hat.r
template <typename Op, typename T>
__device__ __forceinline__ void bicg_x_body(const Op& op, const BicgVecs<T>& v, const BicgState& st, int i, int y,
                                          int chunk, double (*sm)[NWARP]) {
    const int par = i & 1;
    if (st.done[y] | st.flagA[par * st.S + y] | st.flagB[par * st.S + y]) return;
    const bool lead = chunk == 0 && threadIdx.x == 0;
    // t.t == 0 means s == 0: the half step already solved the system.  The
    // reference would divide 0 by 0 here (src/bicgstab.hpp:280); omega = 0
    // keeps x += alpha ph, r = s = 0, and the next p-update retires the system.
    const double tt = sum_parts(st.P(PK_TT, y), st.nchunk);
    const double omega = tt > 0.0 ? sum_parts(st.P(PK_TS, y), st.nchunk) / tt : 0.0;
    const double alpha = st.alpha[y];
    if (lead) st.omega[y] = omega;
    const T al = (T)alpha, om = (T)omega;
    const size_t o = (size_t)y * v.Np;
    T* __restrict__ x = op.x_of(y);
    const T* __restrict__ ph = v.ph + o;
    const T* __restrict__ z = v.z + o;
    const T* __restrict__ t = v.t + o;
    const T* __restrict__ rw = v.rw + o;
    T* __restrict__ r = v.r + o;
    T a0 = 0, a1 = 0;
    BTE_GROUP_LOOP_K(c0, chunk) {
        T xv[GRP], phv[GRP], zv[GRP], tv[GRP], rv[GRP], wv[GRP];
#pragma unroll
        for (int k = 0; k < GRP; ++k) {
            const int c = c0 + k * THREADS;
            xv[k] = x[c]; phv[k] = ph[c]; zv[k] = z[c]; tv[k] = t[c]; rv[k] = r[c]; wv[k] = rw[c];
        }
#pragma unroll
        for (int k = 0; k < GRP; ++k) {
            const int c = c0 + k * THREADS;
            T u = fmat(al, phv[k], xv[k]);
            u = fmat(om, zv[k], u);
            x[c] = u;
            const T rn = fmat(-om, tv[k], rv[k]);
            r[c] = rn;
            a0 = fmat(rn, rn, a0);
            a1 = fmat(wv[k], rn, a1);
        }
    }
    double acc[2] = {(double)a0, (double)a1};
    block_sum<2>(acc, sm);
    if (threadIdx.x == 0) {
        st.P(par ? PK_RR1 : PK_RR0, y)[chunk] = acc[0];
        st.P(par ? PK_RWR1 : PK_RWR0, y)[chunk] = acc[1];
    }
}

template <typename Op, typename T>
__global__ void __launch_bounds__(THREADS) k_bicg_x(Op op, BicgVecs<T> v, BicgState st, int i) {
    __shared__ double sm[2][NWARP];
    bicg_x_body(op, v, st, i, (int)blockIdx.y, (int)blockIdx.x, sm);
}

// Whole BiCGSTAB solves in one launch, one block per system of the batch
// (blockIdx.x = y): the phase bodies above run chunk by chunk, with a block
// barrier after each chunk, so a decision the lead thread records in one chunk
// (converged, restarted, limit reached) is seen by every thread of the block
// in the next.  Each chunk then computes exactly what the phase kernels'
// block for that chunk computes -- none of them depends on another block of
// the same launch -- so x is the same to the bit.  No host round trip between
// iterations, a converged system's block just ends.  i_last = the iteration
// limit + 1 (the p-update of that iteration retires what is left).
template <typename Op, typename T>
__global__ void __launch_bounds__(THREADS) k_bicg_persistent(Op op, BicgVecs<T> v, BicgState st, int i_last) {
    __shared__ double sm[2][NWARP];
    const int y = blockIdx.x;
    for (int i = 1; i <= i_last; ++i) {
        for (int k = 0; k < st.nchunk; ++k) {
            bicg_p_body(op, v, st, i, y, k, sm);
            __syncthreads();
        }
        if (*(volatile const int*)(st.done + y) || i >= i_last) break;
        for (int k = 0; k < st.nchunk; ++k) {
            bicg_spmv1_body(op, v, st, i, y, k, sm);
            __syncthreads();
        }
        for (int k = 0; k < st.nchunk; ++k) {
            bicg_s_body(op, v, st, i, y, k, sm);
            __syncthreads();
        }
        for (int k = 0; k < st.nchunk; ++k) {
            bicg_spmv2_body(op, v, st, i, y, k, sm);
            __syncthreads();
        }
        for (int k = 0; k < st.nchunk; ++k) {
            bicg_x_body(op, v, st, i, y, k, sm);
            __syncthreads();
        }
    }
}

}  // namespace bte
