// bte_dsa.cuh -- diffusion-synthetic acceleration (DSA) of the outer iteration.
//
// No counterpart in the reference: its source iteration (src/StaticBTESolver.cpp:
// 690-808) is kept as it is, and after each outer iteration the change
// r = T_new - T_old of the equilibrium temperature drives a low-order diffusion
// solve on the same cells (face coefficients from dsa_setup.h):
//   sum_f W_f (x_c - x_nb) + sum_{walls} W_f x_c = V_c r_c,
// and T_new + x becomes the source of the next outer iteration (with the
// boundary cells' intensities shifted by C_b / Omega_tot x, the isotropic part
// of the same correction).  The reference's margin between consecutive
// transport iterates still decides convergence, and the result is the last
// transport iterate, never a corrected field.
//
// The diffusion solve is one persistent cooperative kernel: preconditioned
// conjugate gradients in the Chronopoulos-Gear form on the symmetrically
// Jacobi-scaled operator (unit diagonal), with a two-level preconditioner
// (the identity plus a coarse correction on aggregates of cells), FP32
// vectors, dot products summed in FP64 over the block and the grid (each
// thread's one or two cells in FP32), and one grid barrier per iteration, which also
// completes the iteration's two dot products.  One barrier suffices because r,
// w = A u and s are kept in two parity copies: after a barrier every block
// recomputes the new residual of its cells' neighbours from the previous
// iteration's r, w and s with the same fused operations as the neighbours'
// owners, so the values agree to the bit, and the coarse correction of the
// new residual follows from aggregate sums published with the dot products.
#pragma once
#include <cuda_runtime.h>

#include "bte_kernels.cuh"

namespace bte {
namespace dsa {

constexpr int THREADS = 512;
// polls of the barrier flag before a block gives up (~a second)
constexpr long long kBarrierPolls = 1ll << 22;

// The low-order operator in the solve's cell numbering (a locality order of
// the mesh's cells, dsa_setup.h), symmetrically scaled: unit diagonal,
// off-diagonal -w[f][c] coupling c to nb[f][c]; dsc[c] = 1 / sqrt(diagonal)
// (0 for a cell with no coupling at all).
struct Lo {
    int n, F;
    const int* nb;     // [F][n]
    const float* w;    // [F][n]
    const double* dsc; // [n]
    const int* agg;    // [n] aggregate of each cell (Coarse::agg_of)
    const int* nagg;   // [F][n] aggregate of the neighbour nb[f][c] (-1 none)
};

// Aggregates per block of the coarse correction (dsa_setup.h dsa_coarse).
constexpr int AGG = 4;

// The coarse correction of the preconditioner M^-1 = I + P A_c^-1 P^T: block
// k owns cells [k chunk, (k+1) chunk), split into AGG aggregates of seg cells.
struct Coarse {
    int chunk, seg, n_agg;
    int stage;             // nonzero: the block's rows of ainv are copied to shared memory once
    int rows;              // the longest need list (rows of ainv a block stages)
    int topo;              // nonzero: each block's cells' nb, nagg, w and agg are copied to shared memory once
    const float* ainv;     // [n_agg][n_agg]
    const int* need_ptr;   // [nblk+1]
    const int* need;       // aggregates of a block's cells and of their neighbours
    float* sums;           // [2][n_agg][3] published aggregate sums of (r, A u, s), two parity copies
    double* sums0;         // [n_agg] aggregate sums of the scaled right-hand side
    __device__ __forceinline__ int agg_of(int c) const {
        const int k = c / chunk;
        return k * AGG + (c - k * chunk) / seg;
    }
};

// Work and control of one solve (all device memory, 16-byte aligned).
struct CgWork {
    float* r;          // [2][n] residual, two parity copies
    float* aw;         // [2][n] A u
    float* s;          // [2][n] A p
    float* x;          // [n]
    float* p;          // [n]
    float* u;          // [n] preconditioned residual
    double* part;      // [2][nblk][2] per-block partial dot products, by round parity
    unsigned* bar;     // [2] barrier arrivals in this launch (zero before the launch), spare
    int* stat;         // [0] iterations of the last solve, [1] error flag (barrier timeout),
                       // [2] iterations summed over solves
    double* relres;    // [1] final sqrt(r.M r / r0.M r0)
};

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
// Counts the calling block in on a barrier counter: a release at GPU scope,
// so every write the block made before its last __syncthreads is visible to
// a block that reads the new count with ld_acquire.
__device__ __forceinline__ void red_release_add(unsigned* p, unsigned v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Block sum of two doubles in a fixed order; valid in thread 0.
__device__ __forceinline__ void block_sum2(double& a, double& b) {
    __shared__ double wa[32], wb[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0) { wa[warp] = a; wb[warp] = b; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double x = 0.0, y = 0.0;
        for (int w = 0; w < nw; ++w) { x += wa[w]; y += wb[w]; }
        a = x;
        b = y;
    }
    __syncthreads();
}

// Grid-wide sum of two doubles with one barrier (cooperative launch: every
// block is resident).  Each block sums its threads' values (fixed order),
// publishes the pair in the partials of this round's parity and counts itself
// in on a counter that only grows during the launch; once the counter reaches
// round x nblk every block adds the nblk pairs itself, in block order (lane l
// takes blocks l, l+32, ..., then a fixed butterfly), so every block gets the
// same sums, independent of timing, without a second hop through a reducing
// block.  A block can publish round r+1 while another still reads round r
// (other parity), never round r+2 (that needs every block past round r+1).
// The wait is bounded: after kBarrierPolls polls a block records an error and
// the call reports failure, so a kernel never spins forever.
// after(): run by every thread once the barrier is passed, before the sums
// are read (loads of other published values overlap those of the partials);
// fin(a, b): run by thread 0 with the sums, before the block's final barrier.
template <typename After, typename Fin>
__device__ __forceinline__ bool grid_sum2(double& a, double& b, const CgWork& wk, unsigned nblk, unsigned& round,
                                          After&& after, Fin&& fin) {
    __shared__ int s_ok;
    __shared__ double s_a, s_b;
    block_sum2(a, b);
    ++round;
    double* part = wk.part + (size_t)(round & 1u) * 2 * nblk;
    if (threadIdx.x == 0) {
        __stcg(part + 2 * blockIdx.x, a);
        __stcg(part + 2 * blockIdx.x + 1, b);
        red_release_add(wk.bar, 1u);
        const unsigned target = round * nblk;
        s_ok = 1;
        long long k = 0;
        // the error flag is read every 64th poll only: a load after the
        // acquire load waits for it, and would double every poll's latency
        while (ld_acquire(wk.bar) < target) {
            if ((++k & 63) == 0 && (k > kBarrierPolls || *(volatile int*)(wk.stat + 1))) {
                atomicExch(wk.stat + 1, 1);
                s_ok = 0;
                break;
            }
            __nanosleep(20);
        }
    }
    __syncthreads();
    after();
    if (threadIdx.x < 32) {
        double x = 0.0, y = 0.0;
#pragma unroll 4
        for (unsigned i = threadIdx.x; i < nblk; i += 32) {
            x += __ldcg(part + 2 * i);
            y += __ldcg(part + 2 * i + 1);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            x += __shfl_xor_sync(0xffffffffu, x, o);
            y += __shfl_xor_sync(0xffffffffu, y, o);
        }
        if (threadIdx.x == 0) {
            s_a = x;
            s_b = y;
            fin(x, y);
        }
    }
    __syncthreads();
    a = s_a;
    b = s_b;
    return s_ok != 0;
}
__device__ __forceinline__ bool grid_sum2(double& a, double& b, const CgWork& wk, unsigned nblk, unsigned& round) {
    return grid_sum2(a, b, wk, nblk, round, [] {}, [](double, double) {});
}

// r_{i+1} of cell c from the previous iteration's parity copies: the one
// formula every block uses for it.
__device__ __forceinline__ float next_residual(const CgWork& wk, int P, int c, float malpha, float beta, int n) {
    const float so = __ldcg(wk.s + (size_t)(P ^ 1) * n + c);
    const float wi = __ldcg(wk.aw + (size_t)P * n + c);
    const float ri = __ldcg(wk.r + (size_t)P * n + c);
    return __fmaf_rn(malpha, __fmaf_rn(beta, so, wi), ri);
}

// Block sum of the per-thread aggregate partials acc[AGG][3] in a fixed
// order; thread t < 3 AGG holds sum number t afterwards (in out).
__device__ __forceinline__ float block_sum_aggs(const float (&acc)[AGG][3], float* red /* [32][3 AGG] */) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int a = 0; a < AGG; ++a)
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            float v = acc[a][q];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if (lane == 0) red[warp * 3 * AGG + a * 3 + q] = v;
        }
    __syncthreads();
    float t = 0.0f;
    if (threadIdx.x < 3 * AGG)
        for (int w = 0; w < nw; ++w) t += red[w * 3 * AGG + threadIdx.x];
    __syncthreads();
    return t;
}

// sX[J] = (A_c^-1 R)[J] for the aggregates J this block needs, R = sR (all
// aggregates): one warp per row, lanes over the columns (four running sums
// per lane, added in a fixed order), fixed butterfly.  rows: the block's rows
// of A_c^-1 in shared memory (stage) or in global memory.
__device__ __forceinline__ void coarse_rows(const Coarse& co, const float* rows, const float* sR, float* sX) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int j0 = co.need_ptr[blockIdx.x], j1 = co.need_ptr[blockIdx.x + 1];
    const int m = co.n_agg;
    for (int j = j0 + warp; j < j1; j += nw) {
        const int J = co.need[j];
        const float* row = co.stage ? rows + (size_t)(j - j0) * m : co.ainv + (size_t)J * m;
        float v0 = 0.0f, v1 = 0.0f, v2 = 0.0f, v3 = 0.0f;
        int K = lane;
        for (; K + 96 < m; K += 128) {
            v0 = __fmaf_rn(row[K], sR[K], v0);
            v1 = __fmaf_rn(row[K + 32], sR[K + 32], v1);
            v2 = __fmaf_rn(row[K + 64], sR[K + 64], v2);
            v3 = __fmaf_rn(row[K + 96], sR[K + 96], v3);
        }
        for (; K < m; K += 32) v0 = __fmaf_rn(row[K], sR[K], v0);
        float v = (v0 + v1) + (v2 + v3);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) sX[J] = v;
    }
}

// Shared-memory layout of k_dsa_pcg: the couplings start after (2 + rows)
// n_agg floats, rounded up to 16 bytes, and take 3 F + 1 words per cell of
// a block's range.
__host__ __device__ constexpr size_t dsa_topo_offset(int n_agg, int rows) {
    return (((size_t)(2 + rows) * n_agg + 3) / 4) * 4;
}
__host__ __device__ constexpr size_t dsa_topo_words(int chunk, int F) { return (size_t)(3 * F + 1) * chunk; }

// Solve A x = b (A = the low-order operator before scaling, both in the
// solve's numbering) for b[n] (FP64) into xout[n] (FP64): preconditioned
// conjugate gradients, M^-1 = I + P A_c^-1 P^T on the scaled operator,
// relative tolerance tol on sqrt(r.M r), at most maxit iterations.  Launched
// cooperatively with one block per cell range of the coarse set-up, every
// block resident.  Dynamic shared memory: (2 + rows) n_agg floats, rows = the
// longest need list when co.stage, else 0; with co.topo then
// dsa_topo_words(chunk, F) words, the block's cells' couplings (neighbour
// position, its aggregate, weight) and aggregates, so a cell's neighbour
// values are one dependent load away instead of two.
//
// The coarse correction needs P^T r_{i+1} of every aggregate before any block
// can form u_{i+1} = M^-1 r_{i+1}; it follows without another barrier from
// the aggregate sums the owners published with the last dot products:
//   P^T r_{i+1} = P^T r_i - alpha_i (P^T w_i + beta_i P^T s_{i-1}).
template <bool TOPO>
__global__ void __launch_bounds__(THREADS) k_dsa_pcg(Lo lo, Coarse co, CgWork wk, const double* __restrict__ b,
                                                    double tol, int maxit, double* __restrict__ xout) {
    extern __shared__ __align__(16) float smem[];
    float* sR = smem;              // [n_agg] P^T r of every aggregate
    float* sX = smem + co.n_agg;   // [n_agg] coarse solution (the needed entries)
    float* sA = smem + 2 * co.n_agg;  // the block's rows of A_c^-1 (stage)
    if (co.stage) {
        const int j0 = co.need_ptr[blockIdx.x], j1 = co.need_ptr[blockIdx.x + 1];
        for (int q = threadIdx.x; q < (j1 - j0) * co.n_agg; q += blockDim.x) {
            const int j = q / co.n_agg, K = q - j * co.n_agg;
            sA[q] = co.ainv[(size_t)co.need[j0 + j] * co.n_agg + K];
        }
    }
    __shared__ float red[32 * 3 * AGG];
    const int n = lo.n, F = lo.F;
    const unsigned nblk = gridDim.x;
    const int c_lo = blockIdx.x * co.chunk, c_hi = min(n, c_lo + co.chunk);
    const int K0 = blockIdx.x * AGG;  // this block's first aggregate
    // the block's couplings, [F][chunk] each, by local cell c - c_lo
    const int ch = co.chunk;
    int* tNb = reinterpret_cast<int*>(smem + dsa_topo_offset(co.n_agg, co.stage ? co.rows : 0));
    int* tNagg = tNb + (size_t)F * ch;
    float* tW = reinterpret_cast<float*>(tNagg + (size_t)F * ch);
    int* tAgg = reinterpret_cast<int*>(tW + (size_t)F * ch);
    if (TOPO) {
        for (int q = threadIdx.x; q < F * ch; q += blockDim.x) {
            const int f = q / ch, c = c_lo + (q - f * ch);
            if (c >= c_hi) continue;
            tNb[q] = lo.nb[(size_t)f * n + c];
            tNagg[q] = lo.nagg[(size_t)f * n + c];
            tW[q] = lo.w[(size_t)f * n + c];
        }
        for (int c = c_lo + threadIdx.x; c < c_hi; c += blockDim.x) tAgg[c - c_lo] = lo.agg[c];
        __syncthreads();
    }
    auto nb_of = [&](int f, int c) { return TOPO ? tNb[f * ch + (c - c_lo)] : lo.nb[(size_t)f * n + c]; };
    auto nagg_of = [&](int f, int c) { return TOPO ? tNagg[f * ch + (c - c_lo)] : lo.nagg[(size_t)f * n + c]; };
    auto w_of = [&](int f, int c) { return TOPO ? tW[f * ch + (c - c_lo)] : lo.w[(size_t)f * n + c]; };
    auto agg_of = [&](int c) { return TOPO ? tAgg[c - c_lo] : lo.agg[c]; };
    // phase 0: ||D^-1/2 b|| and the aggregate sums of D^-1/2 b
    double nrm2 = 0.0, unused = 0.0;
    {
        double a0[AGG] = {};
        for (int c = c_lo + threadIdx.x; c < c_hi; c += blockDim.x) {
            const double v = lo.dsc[c] * b[c];
            nrm2 = fma(v, v, nrm2);
            const int a = (c - c_lo) / co.seg;
#pragma unroll
            for (int k = 0; k < AGG; ++k)
                if (k == a) a0[k] += v;
        }
        // aggregate sums in a fixed order: per warp, then warps in order
        __shared__ double r0s[32][AGG];
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
        for (int k = 0; k < AGG; ++k) {
            double v = a0[k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if (lane == 0) r0s[warp][k] = v;
        }
        __syncthreads();
        if (threadIdx.x < AGG) {
            double t = 0.0;
            for (int w = 0; w < nw; ++w) t += r0s[w][threadIdx.x];
            __stcg(co.sums0 + K0 + threadIdx.x, t);
        }
    }
    unsigned round = 0;  // barriers passed in this launch
    if (!grid_sum2(nrm2, unused, wk, nblk, round)) return;
    if (!(nrm2 > 0.0) || !isfinite(nrm2)) {  // nothing to correct
        for (int c = c_lo + threadIdx.x; c < c_hi; c += blockDim.x) xout[c] = 0.0;
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            wk.stat[0] = 0;
            wk.relres[0] = 0.0;
        }
        return;
    }
    const double scale = sqrt(nrm2), inv = 1.0 / scale;
    // r0 = D^-1/2 b / scale, u0 = M^-1 r0, w0 = A u0, s_{-1} = p_{-1} = 0
    for (int K = threadIdx.x; K < co.n_agg; K += blockDim.x) sR[K] = (float)(__ldcg(co.sums0 + K) * inv);
    __syncthreads();
    coarse_rows(co, sA, sR, sX);
    __syncthreads();
    float* pub = co.sums;  // parity 0
    double gamma = 0.0, delta = 0.0;
    float gp = 0.0f, dp = 0.0f;  // a thread's partial dot products (its one or two cells), FP32
    {
        float acc[AGG][3] = {};
        for (int c = c_lo + threadIdx.x; c < c_hi; c += blockDim.x) {
            const float rc = (float)(lo.dsc[c] * b[c] * inv);
            const float uc = rc + sX[agg_of(c)];
            float wc = uc;
            for (int f = 0; f < F; ++f) {
                const int o = nb_of(f, c);
                if (o < 0) continue;
                const float uo = (float)(lo.dsc[o] * b[o] * inv) + sX[nagg_of(f, c)];
                wc = __fmaf_rn(-w_of(f, c), uo, wc);
            }
            __stcg(wk.r + c, rc);
            __stcg(wk.aw + c, wc);
            __stcg(wk.s + (size_t)n + c, 0.0f);
            wk.u[c] = uc;
            wk.x[c] = 0.0f;
            wk.p[c] = 0.0f;
            gp = __fmaf_rn(rc, uc, gp);
            dp = __fmaf_rn(wc, uc, dp);
            const int a = (c - c_lo) / co.seg;
#pragma unroll
            for (int k = 0; k < AGG; ++k)
                if (k == a) { acc[k][0] += rc; acc[k][1] += wc; }
        }
        const float t = block_sum_aggs(acc, red);
        if (threadIdx.x < 3 * AGG) __stcg(pub + (size_t)3 * K0 + threadIdx.x, t);
        gamma = gp;
        delta = dp;
    }
    // the aggregate sums (r, A u, s) published before a barrier, loaded into
    // registers as soon as the barrier is passed (aggregates threadIdx.x +
    // q blockDim.x; any beyond KPT blockDim are loaded where they are used)
    constexpr int KPT = 4;
    float nr[KPT] = {}, nw[KPT] = {}, ns[KPT] = {};
    auto load_sums = [&](int Pn) {
        const float* got = co.sums + (size_t)3 * co.n_agg * Pn;
#pragma unroll
        for (int q = 0; q < KPT; ++q) {
            const int K = threadIdx.x + q * blockDim.x;
            if (K < co.n_agg) {
                nr[q] = __ldcg(got + 3 * K);
                nw[q] = __ldcg(got + 3 * K + 1);
                ns[q] = __ldcg(got + 3 * K + 2);
            }
        }
    };
    if (!grid_sum2(gamma, delta, wk, nblk, round, [&] { load_sums(0); }, [](double, double) {})) return;
    const double gamma0 = gamma;
    double alpha = delta > 0.0 ? gamma / delta : 0.0, beta = 0.0;
    int it = 0;
    bool stop = !(delta > 0.0) || gamma <= tol * tol * gamma0;
    // the iteration's scalars, formed once per block by thread 0 (FP64
    // divisions are slow on this part's FP64 pipe) and read by every thread:
    // alpha and beta, their FP32 forms, the stop flag
    __shared__ double s_alpha, s_beta;
    __shared__ float s_fa, s_fb;
    __shared__ int s_stop;
    float fa = (float)alpha, fb = (float)beta;
    while (!stop && it < maxit) {
        const int P = it & 1;
        const float fma_ = -fa;
        // P^T r_{i+1} of every aggregate from the published sums, then the coarse solve
#pragma unroll
        for (int q = 0; q < KPT; ++q) {
            const int K = threadIdx.x + q * blockDim.x;
            if (K < co.n_agg) sR[K] = __fmaf_rn(fma_, __fmaf_rn(fb, ns[q], nw[q]), nr[q]);
        }
        const float* got = co.sums + (size_t)3 * co.n_agg * P;
        for (int K = threadIdx.x + KPT * blockDim.x; K < co.n_agg; K += blockDim.x) {
            const float sr = __ldcg(got + 3 * K), sw = __ldcg(got + 3 * K + 1), ss = __ldcg(got + 3 * K + 2);
            sR[K] = __fmaf_rn(fma_, __fmaf_rn(fb, ss, sw), sr);
        }
        __syncthreads();
        coarse_rows(co, sA, sR, sX);
        __syncthreads();
        float gq = 0.0f, dq = 0.0f;
        float acc[AGG][3] = {};
        for (int c = c_lo + threadIdx.x; c < c_hi; c += blockDim.x) {
            const float so = __ldcg(wk.s + (size_t)(P ^ 1) * n + c);
            const float wi = __ldcg(wk.aw + (size_t)P * n + c);
            const float ri = __ldcg(wk.r + (size_t)P * n + c);
            const float si = __fmaf_rn(fb, so, wi);
            const float pc = __fmaf_rn(fb, wk.p[c], wk.u[c]);
            wk.p[c] = pc;
            wk.x[c] = __fmaf_rn(fa, pc, wk.x[c]);
            const float rn = __fmaf_rn(fma_, si, ri);
            const int ac = agg_of(c);
            const float un = rn + sX[ac];
            float wn = un;
            for (int f = 0; f < F; ++f) {
                const int o = nb_of(f, c);
                if (o < 0) continue;
                const float uo = next_residual(wk, P, o, fma_, fb, n) + sX[nagg_of(f, c)];
                wn = __fmaf_rn(-w_of(f, c), uo, wn);
            }
            __stcg(wk.s + (size_t)P * n + c, si);
            __stcg(wk.r + (size_t)(P ^ 1) * n + c, rn);
            __stcg(wk.aw + (size_t)(P ^ 1) * n + c, wn);
            wk.u[c] = un;
            gq = __fmaf_rn(rn, un, gq);
            dq = __fmaf_rn(wn, un, dq);
            const int a = ac - K0;
#pragma unroll
            for (int k = 0; k < AGG; ++k)
                if (k == a) { acc[k][0] += rn; acc[k][1] += wn; acc[k][2] += si; }
        }
        const float t = block_sum_aggs(acc, red);
        if (threadIdx.x < 3 * AGG)
            __stcg(co.sums + (size_t)3 * co.n_agg * (P ^ 1) + (size_t)3 * K0 + threadIdx.x, t);
        // thread 0 forms the next scalars from the sums inside the barrier's
        // last step (every thread holds the same gamma and alpha)
        auto scalars = [&](double g, double dd) {
            const double bnew = g / gamma;
            const double den = dd - bnew * g / alpha;
            const bool st = g <= tol * tol * gamma0 || !(den > 0.0) || !isfinite(den);
            s_stop = st;
            if (!st) {
                s_beta = bnew;
                s_alpha = g / den;
                s_fa = (float)s_alpha;
                s_fb = (float)bnew;
            }
        };
        double gn = gq, dn = dq;  // summed over the block and the grid in FP64
        if (!grid_sum2(gn, dn, wk, nblk, round, [&] { load_sums(P ^ 1); }, scalars)) return;
        ++it;
        gamma = gn;
        if (s_stop) {
            stop = true;
        } else {
            beta = s_beta;
            alpha = s_alpha;
            fa = s_fa;
            fb = s_fb;
        }
    }
    for (int c = c_lo + threadIdx.x; c < c_hi; c += blockDim.x) xout[c] = (double)wk.x[c] * lo.dsc[c] * scale;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        wk.stat[0] = it;
        wk.stat[2] += it;
        wk.relres[0] = sqrt(fabs(gamma / gamma0));
    }
}

// One step of the in-place Gauss-Jordan inversion of a symmetric positive
// definite m x m matrix (no pivoting: its pivots stay positive): B = the
// matrix after eliminating column k of A.  After m steps (A and B swapped
// between steps) the matrix is the inverse.  A pivot that is not positive
// sets *bad (the matrix is not positive definite).
__global__ void k_gj_step(const double* __restrict__ A, double* __restrict__ B, int m, int k, int* bad) {
    __shared__ double s_rp;
    const int i = blockIdx.y;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (threadIdx.x == 0) {
        const double p = A[(size_t)k * m + k];
        if (!(p > 0.0) && i == 0 && blockIdx.x == 0) atomicExch(bad, 1);
        s_rp = 1.0 / p;
    }
    __syncthreads();
    if (j >= m) return;
    const double rp = s_rp;
    const double aik = A[(size_t)i * m + k], akj = A[(size_t)k * m + j];
    double v;
    if (i == k) v = j == k ? rp : akj * rp;
    else if (j == k) v = -aik * rp;
    else v = fma(-aik, akj * rp, A[(size_t)i * m + j]);
    B[(size_t)i * m + j] = v;
}

// All m steps of the same inversion in one cooperative launch (every block
// resident): step k reads src and writes dst (rows by block, columns by
// thread), then a grid barrier -- a counter that only grows during the
// launch, zero before it -- and the buffers swap; after the last step the
// inverse is in A when m is even, else in B.  Values another block wrote are
// read through L2 (__ldcg).  A wait that runs out (kBarrierPolls polls) sets
// *bad = 2 and the block returns; a pivot that is not positive sets *bad = 1.
__global__ void __launch_bounds__(1024) k_gj_all(double* A, double* B, int m, unsigned* bar, int* bad) {
    __shared__ double s_rp;
    __shared__ int s_abort;
    const unsigned nblk = gridDim.x;
    double* src = A;
    double* dst = B;
    for (int k = 0; k < m; ++k) {
        if (threadIdx.x == 0) {
            const double p = __ldcg(src + (size_t)k * m + k);
            if (!(p > 0.0) && blockIdx.x == 0) atomicExch(bad, 1);
            s_rp = 1.0 / p;
        }
        __syncthreads();
        const double rp = s_rp;
        for (int i = blockIdx.x; i < m; i += nblk) {
            const double aik = __ldcg(src + (size_t)i * m + k);
            for (int j = threadIdx.x; j < m; j += blockDim.x) {
                const double akj = __ldcg(src + (size_t)k * m + j);
                double v;
                if (i == k) v = j == k ? rp : akj * rp;
                else if (j == k) v = -aik * rp;
                else v = fma(-aik, akj * rp, __ldcg(src + (size_t)i * m + j));
                __stcg(dst + (size_t)i * m + j, v);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            s_abort = 0;
            red_release_add(bar, 1u);
            const unsigned target = (unsigned)(k + 1) * nblk;
            long long polls = 0;
            while (ld_acquire(bar) < target) {
                if ((++polls & 63) == 0 && (polls > kBarrierPolls || *(volatile int*)bad == 2)) {
                    atomicExch(bad, 2);
                    s_abort = 1;
                    break;
                }
                __nanosleep(20);
            }
        }
        __syncthreads();
        if (s_abort) return;
        double* t = src;
        src = dst;
        dst = t;
    }
}

// The same inversion kGjBlock pivots at a time: ceil(m / kGjBlock) grid
// barriers instead of m.  A step with pivot set K (rows and columns K0 ..
// K0 + kb - 1, P = A[K,K]) is the kb scalar steps of k_gj_all at once:
//   B[K,K] = P^-1,  B[K,j] = P^-1 A[K,j],  B[i,K] = -A[i,K] P^-1,
//   B[i,j] = A[i,j] - (A[i,K] P^-1) A[K,j]   (i, j outside K);
// every block forms P^-1 in shared memory by the scalar steps, then updates
// its rows (rows by block, columns by thread) from the pivot rows A[K,:],
// which it holds in shared memory.  Rounding differs from the scalar steps'
// (a kb-term sum per entry instead of kb updates).  Dynamic shared memory:
// kGjBlock * (m + kGjBlock + 1) doubles.  Barriers, buffers and *bad as in
// k_gj_all; the inverse is in A when the number of steps is even, else in B.
constexpr int kGjBlock = 16;
__global__ void __launch_bounds__(1024) k_gj_block_all(double* A, double* B, int m, unsigned* bar, int* bad) {
    extern __shared__ double gsm[];
    double* sR = gsm;                                   // [kGjBlock][m] pivot rows A[K,:]
    double* sP = gsm + (size_t)kGjBlock * m;           // [kGjBlock][kGjBlock] P, then P^-1
    double* sT = sP + kGjBlock * kGjBlock;             // [kGjBlock] A[i,K] P^-1 of the current row
    __shared__ int s_abort;
    const unsigned nblk = gridDim.x;
    const int tid = threadIdx.x;
    double* src = A;
    double* dst = B;
    int step = 0;
    for (int K0 = 0; K0 < m; K0 += kGjBlock, ++step) {
        const int kb = min(kGjBlock, m - K0);
        for (int q = tid; q < kb * m; q += blockDim.x) {
            const int r = q / m, j = q - r * m;
            sR[q] = __ldcg(src + (size_t)(K0 + r) * m + j);
        }
        __syncthreads();
        // P^-1 by kb scalar steps (each thread one entry; read, barrier, write)
        const int pr = tid / kb, pc = tid - pr * kb;
        const bool pin = tid < kb * kb;
        if (pin) sP[pr * kGjBlock + pc] = sR[(size_t)pr * m + K0 + pc];
        __syncthreads();
        for (int k = 0; k < kb; ++k) {
            const double p = sP[k * kGjBlock + k];
            if (tid == 0 && !(p > 0.0) && blockIdx.x == 0) atomicExch(bad, 1);
            double v = 0.0;
            if (pin) {
                const double rp = 1.0 / p;
                const double aik = sP[pr * kGjBlock + k], akj = sP[k * kGjBlock + pc];
                if (pr == k) v = pc == k ? rp : akj * rp;
                else if (pc == k) v = -aik * rp;
                else v = fma(-aik, akj * rp, sP[pr * kGjBlock + pc]);
            }
            __syncthreads();
            if (pin) sP[pr * kGjBlock + pc] = v;
            __syncthreads();
        }
        for (int i = blockIdx.x; i < m; i += nblk) {
            const bool piv = i >= K0 && i < K0 + kb;
            if (!piv && tid < kb) {  // t = A[i,K] P^-1
                double t = 0.0;
                for (int l = 0; l < kb; ++l) t = fma(__ldcg(src + (size_t)i * m + K0 + l), sP[l * kGjBlock + tid], t);
                sT[tid] = t;
            }
            __syncthreads();
            for (int j = tid; j < m; j += blockDim.x) {
                const bool jk = j >= K0 && j < K0 + kb;
                double v;
                if (piv) {
                    const int r = i - K0;
                    if (jk) {
                        v = sP[r * kGjBlock + (j - K0)];
                    } else {
                        v = 0.0;
                        for (int l = 0; l < kb; ++l) v = fma(sP[r * kGjBlock + l], sR[(size_t)l * m + j], v);
                    }
                } else if (jk) {
                    v = -sT[j - K0];
                } else {
                    double acc = 0.0;
                    for (int l = 0; l < kb; ++l) acc = fma(sT[l], sR[(size_t)l * m + j], acc);
                    v = __ldcg(src + (size_t)i * m + j) - acc;
                }
                __stcg(dst + (size_t)i * m + j, v);
            }
            __syncthreads();
        }
        if (tid == 0) {
            s_abort = 0;
            red_release_add(bar, 1u);
            const unsigned target = (unsigned)(step + 1) * nblk;
            long long polls = 0;
            while (ld_acquire(bar) < target) {
                if ((++polls & 63) == 0 && (polls > kBarrierPolls || *(volatile int*)bad == 2)) {
                    atomicExch(bad, 2);
                    s_abort = 1;
                    break;
                }
                __nanosleep(20);
            }
        }
        __syncthreads();
        if (s_abort) return;
        double* t = src;
        src = dst;
        dst = t;
    }
}

__global__ void k_to_float(const double* __restrict__ a, float* __restrict__ out, size_t n) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) out[q] = (float)a[q];
}

// Right-hand side V_c (T_c - T_src,c) of the low-order solve, in its numbering:
// position k holds cell order[k].
__global__ void k_dsa_rhs(const double* __restrict__ T, const double* __restrict__ Tsrc,
                          const double* __restrict__ volume, const int* __restrict__ order, int n,
                          double* __restrict__ b) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int c = order[k];
    b[k] = volume[c] * (T[c] - Tsrc[c]);
}

// T += x, and the equilibrium energy density follows: ebar[b][c] = C_b / Omega_tot (T - T_ref).
// x is in the solve's numbering (pos[c] = position of cell c); xc[c] receives it by cell.
__global__ void k_dsa_apply(const double* __restrict__ x, const int* __restrict__ pos, const double* __restrict__ Cb,
                            double solid_angle, double T_ref, int n, int n_band, size_t Np, double* __restrict__ T,
                            double* __restrict__ ebar, double* __restrict__ xc) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const double dx = x[pos[c]];
    xc[c] = dx;
    const double t = T[c] + dx;
    T[c] = t;
    for (int b = 0; b < n_band; ++b) ebar[(size_t)b * Np + c] = Cb[b] / solid_angle * (t - T_ref);
}

// The intensities of the cells with boundary faces, which the next outer
// iteration reflects at diffuse and specular walls, take the same correction
// isotropically: e[b][d][c] += C_b / Omega_tot x_c.  One thread per (boundary
// cell, direction), grid.y = band.
__global__ void k_dsa_shift_boundary(const double* __restrict__ x, const int* __restrict__ bcell, int nbcell,
                                     const double* __restrict__ Cb, double solid_angle, int n_dir, size_t Np,
                                     double* __restrict__ e) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int b = blockIdx.y;
    if (t >= nbcell * n_dir) return;
    const int i = t % nbcell, d = t / nbcell;
    const int c = bcell[i];
    e[((size_t)b * n_dir + d) * Np + c] += Cb[b] / solid_angle * x[c];
}

__global__ void k_fill(double* __restrict__ v, double value, int n) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < n) v[c] = value;
}

}  // namespace dsa
}  // namespace bte
