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
// The diffusion solve is one persistent cooperative kernel: conjugate
// gradients in the Chronopoulos-Gear form on the symmetrically Jacobi-scaled
// operator (unit diagonal), FP32 vectors, FP64 dot products, with one grid
// barrier per iteration, which also completes the iteration's two dot
// products.  One barrier suffices because r, w = A r and s are kept in two
// parity copies: after a barrier every block recomputes the new residual of
// its cells' neighbours from the previous iteration's r, w and s with the same
// fused operations as the neighbours' owners, so the values agree to the bit
// and the product A r_new needs no second barrier.
#pragma once
#include <cuda_runtime.h>

#include "bte_kernels.cuh"

namespace bte {
namespace dsa {

constexpr int THREADS = 512;
// polls of the barrier flag before a block gives up (~a second)
constexpr long long kBarrierPolls = 1ll << 22;

// The low-order operator, symmetrically scaled: unit diagonal, off-diagonal
// -w[f][c] coupling c to nb[f][c]; dsc[c] = 1 / sqrt(diagonal) (0 for a cell
// with no coupling at all).
struct Lo {
    int n, F;
    const int* nb;     // [F][n]
    const float* w;    // [F][n]
    const double* dsc; // [n]
};

// Work and control of one solve (all device memory, 16-byte aligned).
struct CgWork {
    float* r;          // [2][n] residual, two parity copies
    float* aw;         // [2][n] A r
    float* s;          // [2][n] A p
    float* x;          // [n]
    float* p;          // [n]
    double* part;      // [nblk][2] per-block partial dot products, then [2] the grid's sums
    unsigned* bar;     // [2] barrier arrival count and generation (zero before the launch)
    int* stat;         // [0] iterations of the last solve, [1] error flag (barrier timeout),
                       // [2] iterations summed over solves
    double* relres;    // [1] final sqrt(r.r / r0.r0)
};

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
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
// block is resident).  Each block sums its threads' values (fixed order) and
// publishes the pair; the block that arrives last adds the blocks' pairs in
// block order (lane l takes blocks l, l+32, ..., then a fixed butterfly), so
// the sums never depend on which block was last or on timing, writes them
// once and releases the others, which read just the two sums.  The wait is
// bounded: after kBarrierPolls polls a block records an error and the call
// reports failure, so a kernel never spins forever.
__device__ __forceinline__ bool grid_sum2(double& a, double& b, const CgWork& wk, unsigned nblk) {
    __shared__ int s_last, s_ok;
    __shared__ double s_a, s_b;
    block_sum2(a, b);
    double* sums = wk.part + 2 * (size_t)nblk;
    if (threadIdx.x == 0) {
        wk.part[2 * blockIdx.x] = a;
        wk.part[2 * blockIdx.x + 1] = b;
        const unsigned gen = ld_acquire(wk.bar + 1);
        __threadfence();
        const bool last = atomicAdd(wk.bar, 1u) == nblk - 1;
        s_last = last;
        s_ok = 1;
        if (!last) {
            long long k = 0;
            while (ld_acquire(wk.bar + 1) == gen) {
                if (++k > kBarrierPolls || *(volatile int*)(wk.stat + 1)) {
                    atomicExch(wk.stat + 1, 1);
                    s_ok = 0;
                    break;
                }
                __nanosleep(20);
            }
            __threadfence();
            s_a = __ldcg(sums);
            s_b = __ldcg(sums + 1);
        }
    }
    __syncthreads();
    if (s_last && threadIdx.x < 32) {
        __threadfence();
        double x = 0.0, y = 0.0;
#pragma unroll 4
        for (unsigned i = threadIdx.x; i < nblk; i += 32) {
            x += __ldcg(wk.part + 2 * i);
            y += __ldcg(wk.part + 2 * i + 1);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            x += __shfl_xor_sync(0xffffffffu, x, o);
            y += __shfl_xor_sync(0xffffffffu, y, o);
        }
        if (threadIdx.x == 0) {
            __stcg(sums, x);
            __stcg(sums + 1, y);
            s_a = x;
            s_b = y;
            __threadfence();
            atomicExch(wk.bar, 0u);
            __threadfence();
            atomicAdd(wk.bar + 1, 1u);
        }
    }
    __syncthreads();
    a = s_a;
    b = s_b;
    const bool ok = s_ok != 0;
    __syncthreads();
    return ok;
}

// r_{i+1} of cell c from the previous iteration's parity copies: the one
// formula every block uses for it.
__device__ __forceinline__ float next_residual(const CgWork& wk, int P, int c, float malpha, float beta, int n) {
    const float so = __ldcg(wk.s + (size_t)(P ^ 1) * n + c);
    const float wi = __ldcg(wk.aw + (size_t)P * n + c);
    const float ri = __ldcg(wk.r + (size_t)P * n + c);
    return __fmaf_rn(malpha, __fmaf_rn(beta, so, wi), ri);
}

// Solve A x = b (A = the low-order operator before scaling) for b[n] (FP64)
// into xout[n] (FP64), relative tolerance tol on ||r|| of the scaled system,
// at most maxit iterations.  Launched cooperatively with every block resident.
__global__ void __launch_bounds__(THREADS) k_dsa_cg(Lo lo, CgWork wk, const double* __restrict__ b, double tol,
                                                   int maxit, double* __restrict__ xout) {
    const int n = lo.n, F = lo.F;
    const unsigned nblk = gridDim.x;
    const int stride = gridDim.x * blockDim.x;
    const int c0 = blockIdx.x * blockDim.x + threadIdx.x;
    // phase 0: ||D^-1/2 b||
    double nrm2 = 0.0, unused = 0.0;
    for (int c = c0; c < n; c += stride) {
        const double v = lo.dsc[c] * b[c];
        nrm2 = fma(v, v, nrm2);
    }
    if (!grid_sum2(nrm2, unused, wk, nblk)) return;
    if (!(nrm2 > 0.0) || !isfinite(nrm2)) {  // nothing to correct
        for (int c = c0; c < n; c += stride) xout[c] = 0.0;
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            wk.stat[0] = 0;
            wk.relres[0] = 0.0;
        }
        return;
    }
    const double scale = sqrt(nrm2), inv = 1.0 / scale;
    // r0 = D^-1/2 b / scale, w0 = A r0, s_{-1} = 0
    double gamma = 0.0, delta = 0.0;
    for (int c = c0; c < n; c += stride) {
        const float rc = (float)(lo.dsc[c] * b[c] * inv);
        float acc = rc;
        for (int f = 0; f < F; ++f) {
            const int o = lo.nb[(size_t)f * n + c];
            if (o < 0) continue;
            const float ro = (float)(lo.dsc[o] * b[o] * inv);
            acc = __fmaf_rn(-lo.w[(size_t)f * n + c], ro, acc);
        }
        __stcg(wk.r + c, rc);
        __stcg(wk.aw + c, acc);
        __stcg(wk.s + (size_t)n + c, 0.0f);
        wk.x[c] = 0.0f;
        wk.p[c] = 0.0f;
        gamma = fma((double)rc, (double)rc, gamma);
        delta = fma((double)acc, (double)rc, delta);
    }
    if (!grid_sum2(gamma, delta, wk, nblk)) return;
    const double gamma0 = gamma;
    double alpha = delta > 0.0 ? gamma / delta : 0.0, beta = 0.0;
    int it = 0;
    bool stop = !(delta > 0.0) || gamma <= tol * tol * gamma0;
    while (!stop && it < maxit) {
        const int P = it & 1;
        const float fa = (float)alpha, fma_ = -(float)alpha, fb = (float)beta;
        double gn = 0.0, dn = 0.0;
        for (int c = c0; c < n; c += stride) {
            const float so = __ldcg(wk.s + (size_t)(P ^ 1) * n + c);
            const float wi = __ldcg(wk.aw + (size_t)P * n + c);
            const float ri = __ldcg(wk.r + (size_t)P * n + c);
            const float si = __fmaf_rn(fb, so, wi);
            const float pc = __fmaf_rn(fb, wk.p[c], ri);
            wk.p[c] = pc;
            wk.x[c] = __fmaf_rn(fa, pc, wk.x[c]);
            const float rn = __fmaf_rn(fma_, si, ri);
            float acc = rn;
            for (int f = 0; f < F; ++f) {
                const int o = lo.nb[(size_t)f * n + c];
                if (o < 0) continue;
                acc = __fmaf_rn(-lo.w[(size_t)f * n + c], next_residual(wk, P, o, fma_, fb, n), acc);
            }
            __stcg(wk.s + (size_t)P * n + c, si);
            __stcg(wk.r + (size_t)(P ^ 1) * n + c, rn);
            __stcg(wk.aw + (size_t)(P ^ 1) * n + c, acc);
            gn = fma((double)rn, (double)rn, gn);
            dn = fma((double)acc, (double)rn, dn);
        }
        if (!grid_sum2(gn, dn, wk, nblk)) return;
        ++it;
        const double bnew = gn / gamma;
        const double den = dn - bnew * gn / alpha;
        gamma = gn;
        if (gn <= tol * tol * gamma0 || !(den > 0.0) || !isfinite(den)) {
            stop = true;
        } else {
            beta = bnew;
            alpha = gn / den;
        }
    }
    for (int c = c0; c < n; c += stride) xout[c] = (double)wk.x[c] * lo.dsc[c] * scale;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        wk.stat[0] = it;
        wk.stat[2] += it;
        wk.relres[0] = sqrt(gamma / gamma0);
    }
}

// Right-hand side V_c (T_c - T_src,c) of the low-order solve.
__global__ void k_dsa_rhs(const double* __restrict__ T, const double* __restrict__ Tsrc,
                          const double* __restrict__ volume, int n, double* __restrict__ b) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < n) b[c] = volume[c] * (T[c] - Tsrc[c]);
}

// T += x, and the equilibrium energy density follows: ebar[b][c] = C_b / Omega_tot (T - T_ref).
__global__ void k_dsa_apply(const double* __restrict__ x, const double* __restrict__ Cb, double solid_angle,
                            double T_ref, int n, int n_band, size_t Np, double* __restrict__ T,
                            double* __restrict__ ebar) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const double t = T[c] + x[c];
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
