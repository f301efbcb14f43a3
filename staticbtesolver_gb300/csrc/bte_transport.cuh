// bte_transport.cuh -- assembly, boundary conditions, reductions and heat flux.
#pragma once
#include <climits>

#include "bte_kernels.cuh"

namespace bte {

// Per-direction, band-independent geometry of the upwind operator (the parts of
// _get_Ke, src/StaticBTESolver.cpp:122-160, that do not depend on the band):
//   dg[d][c]    = sum over faces with s_d.n >= 0 of A_cf g_dcf
//   fc[d][f][c] = A_cf g_dcf on faces with s_d.n < 0 and a neighbour, else 0
//   vo[d][c]    = V_c Omega_d (1D: V_c)
// g = S_d.n (s_d.n on 1D meshes).  One launch per solve set-up.
__global__ void k_direction_geometry(const double* __restrict__ normal,  // [n][F][3]
                                     const double* __restrict__ area,    // [n][F]
                                     const int* __restrict__ nbr,        // [n][F]
                                     const double* __restrict__ volume,  // [n]
                                     const double* __restrict__ s, const double* __restrict__ S,
                                     const double* __restrict__ omega, int n, int F, int dim,
                                     size_t Np, double* dg, double* vo, double* fc) {
    const int d = blockIdx.y;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= Np) return;
    const size_t dc = (size_t)d * Np + c;
    if (c >= n) {  // padded cell: identity row
        dg[dc] = 0.0;
        vo[dc] = 1.0;
        for (int f = 0; f < F; ++f) fc[((size_t)d * F + f) * Np + c] = 0.0;
        return;
    }
    const double sx = s[3 * d], sy = s[3 * d + 1], sz = s[3 * d + 2];
    const double Sx = S[3 * d], Sy = S[3 * d + 1], Sz = S[3 * d + 2];
    double acc = 0.0;
    for (int f = 0; f < F; ++f) {
        const double* nn = normal + ((size_t)c * F + f) * 3;
        const double sn = sx * nn[0] + sy * nn[1] + sz * nn[2];
        const double g = dim > 1 ? Sx * nn[0] + Sy * nn[1] + Sz * nn[2] : sn;
        const double ag = area[(size_t)c * F + f] * g;
        double cf = 0.0;
        if (sn >= 0) acc += ag;
        else if (nbr[(size_t)c * F + f] >= 0) cf = ag;
        fc[((size_t)d * F + f) * Np + c] = cf;
    }
    dg[dc] = acc;
    vo[dc] = dim > 1 ? volume[c] * omega[d] : volume[c];
}

// Boundary description (host-built): faces whose neighbour code matches a
// boundary-condition row, sorted by (cell, face).  bptr[c]..bptr[c+1] are the
// entries of cell c.
struct Boundary {
    const int* bptr;      // [Np+1]
    const int* bf_cell;   // [nbf]
    const int* bf_kind;   // [nbf] 1, 2, 31, 32, 33
    const int* bf_bc;     // [nbf] boundary-condition row
    const int* bf_diff;   // [nbf] row in the diffuse list, or -1
    const double* cin;    // [n_dir][nbf] A g on inflow directions (s.n < 0), else 0
    const double* eiso;   // [n_band][n_bc] C_b / Omega_tot (T_bc - T_ref)
    const int* mirror;    // [3][n_dir] specular partner for 31, 32, 33
    const double* ediff;  // [n_band][nbf] diffuse wall energy (this outer iteration)
    int nbf, n_bc;
};

// Right-hand side of system (band b, direction d) at cell c (_get_Re,
// src/StaticBTESolver.cpp:162-269):
//   R[c] = - sum_{inflow boundary faces} e_wall k_b A g + ebar[b][c] V_c Omega_d
// e_wall: isothermal C_b/Omega_tot (T_bc - T_ref); diffuse: the outgoing
// energy of the previous iterate averaged over the wall; specular: the previous
// iterate at the mirrored direction.  Computed where it is consumed, so no
// right-hand-side array is written or read.
struct RhsSrc {
    Boundary bd;
    const double* ebar;    // [n_band][Np]
    const double* e_prev;  // [n_band][n_dir][Np]
    int n_dir;
    size_t Np;
    // the boundary part: - sum over the cell's inflow boundary faces of e_wall k A g (k = k_b)
    __device__ __forceinline__ double boundary(int b, int d, int c, double k) const {
        const double* ep_b = e_prev + (size_t)b * n_dir * Np;
        double r = 0.0;
        const int e0 = bd.bptr[c], e1 = bd.bptr[c + 1];
        for (int e = e0; e < e1; ++e) {
            const double cf = bd.cin[(size_t)d * bd.nbf + e];
            if (cf == 0.0) continue;
            double ew;
            switch (bd.bf_kind[e]) {
                case 1: ew = bd.eiso[(size_t)b * bd.n_bc + bd.bf_bc[e]]; break;
                case 2: ew = bd.ediff[(size_t)b * bd.nbf + e]; break;
                case 31: ew = ep_b[(size_t)bd.mirror[d] * Np + c]; break;
                case 32: ew = ep_b[(size_t)bd.mirror[n_dir + d] * Np + c]; break;
                default: ew = ep_b[(size_t)bd.mirror[2 * n_dir + d] * Np + c]; break;
            }
            r -= ew * (k * cf);
        }
        return r;
    }
    // vo = V_c Omega_d
    __device__ __forceinline__ double at(int b, int d, int c, double k, double vo) const {
        return boundary(b, d, c, k) + ebar[(size_t)b * Np + c] * vo;
    }
};

// Boundary part of the right-hand side per (system of the batch, boundary
// cell), for the sweep: bsum[y][i] = RhsSrc::boundary / D for cell bcell[i],
// with y -> direction y / nbb, band b0 + y % nbb as in FaceFluxOp.
__global__ void k_bound_rhs(RhsSrc src, const int* __restrict__ bcell, int nbcell, const double* __restrict__ kb,
                            const double* __restrict__ binvd, int nbb, int b0, double* bsum) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (i >= nbcell) return;
    const int d = y / nbb, b = b0 + y % nbb;
    // scaled by the cell's 1/D, as the sweep's other terms
    bsum[(size_t)y * nbcell + i] =
        src.boundary(b, d, bcell[i], kb[b]) * binvd[((size_t)b * src.n_dir + d) * nbcell + i];
}

// 1/D = 1 / (k_b dg[d][c] + vo[d][c]) of every boundary cell, per (band,
// direction): binvd[b][d][i] for cell bcell[i] (once per solve).
__global__ void k_bound_invd(const int* __restrict__ bcell, int nbcell, const double* __restrict__ kb,
                             const double* __restrict__ dg, const double* __restrict__ vo, int n_band, int n_dir,
                             size_t Np, double* binvd) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int d = blockIdx.y;
    if (i >= nbcell) return;
    const size_t dc = (size_t)d * Np + bcell[i];
    for (int b = 0; b < n_band; ++b)
        binvd[((size_t)b * n_dir + d) * nbcell + i] = 1.0 / fma(kb[b], dg[dc], vo[dc]);
}

// Right-hand sides of one batch for the Krylov forms: rhs[y][c].
__global__ void __launch_bounds__(THREADS) k_rhs(FaceFluxOp op, RhsSrc src, double* rhs, int n) {
    const int y = blockIdx.y;
    int b, d;
    op.bd(y, b, d);
    const double k = op.kb[b];
    const size_t o = (size_t)y * op.Np;
    BTE_CELL_LOOP(c) { rhs[o + c] = c < n ? src.at(b, d, c, k, op.vo[(size_t)d * op.Np + c]) : 0.0; }
}

// Diffuse wall energy per (band, diffuse face) from the previous iterate
// (src/StaticBTESolver.cpp:180-204): sum over outgoing directions of
// e w / sum w, w = (S.n) Omega in 3D, S.n in 2D; 1D: sum e (s.n) Omega / pi.
// One warp per (band, diffuse face): lane l sums directions l, l+32, ... and
// the lanes are combined by a fixed butterfly (the order does not depend on
// timing).
__global__ void k_diffuse_wall(const double* __restrict__ e_prev, const int* __restrict__ dlist,  // [ndiff] -> bf
                               const int* __restrict__ bf_cell, const double* __restrict__ wdiff,  // [ndiff][n_dir]
                               const double* __restrict__ wden,  // [ndiff]
                               int ndiff, int n_band, int n_dir, size_t Np, int nbf, double* ediff) {
    const int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;  // warp index: whole warps exit together
    const int lane = threadIdx.x & 31;
    if (t >= ndiff * n_band) return;
    const int b = t / ndiff, k = t % ndiff;
    const int e = dlist[k];
    const int c = bf_cell[e];
    const double* ep = e_prev + (size_t)b * n_dir * Np + c;
    const double* w = wdiff + (size_t)k * n_dir;
    double acc = 0.0;
    for (int d = lane; d < n_dir; d += 32)
        if (w[d] != 0.0) acc += ep[(size_t)d * Np] * w[d];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) ediff[(size_t)b * nbf + e] = acc / wden[k];
}

// The reductions that close an outer iteration (src/StaticBTESolver.cpp:96-104
// and :311-321), one pass over e_curr (and e_prev for MARGIN) with one block
// per (256 cells, band):
//   Tb[b][c] = sum_d e Omega_d / C_b + T_ref
//   margin partial[b][block] = sum_d (e_curr - e_prev)^2 over the block's cells
// (without MARGIN the sweep has already summed the margin partials).
template <bool MARGIN>
__global__ void __launch_bounds__(THREADS) k_reduce(const double* __restrict__ e_curr, const double* __restrict__ e_prev,
                                                    const double* __restrict__ omega, const double* __restrict__ Cb,
                                                    double T_ref, int n, int n_dir, size_t Np, double* Tb,
                                                    double* part) {
    __shared__ double sm[1][NWARP];
    const int c = blockIdx.x * THREADS + threadIdx.x;
    const int b = blockIdx.y;
    double m[1] = {0.0};
    if (c < n) {
        const double* ec = e_curr + (size_t)b * n_dir * Np + c;
        const double* ep = e_prev + (size_t)b * n_dir * Np + c;
        double e0 = 0.0;
#pragma unroll 8
        for (int d = 0; d < n_dir; ++d) {
            const double a = __ldcs(ec + (size_t)d * Np);
            e0 += a * omega[d];
            if (MARGIN) {
                const double df = a - __ldcs(ep + (size_t)d * Np);
                m[0] = fma(df, df, m[0]);
            }
        }
        Tb[(size_t)b * Np + c] = e0 / Cb[b] + T_ref;
    }
    if (MARGIN) {
        block_sum<1>(m, sm);
        if (threadIdx.x == 0) part[(size_t)b * gridDim.x + blockIdx.x] = m[0];
    }
}

// src/StaticBTESolver.cpp:106-120: T[c] = sum_b Lr_b Tb[b][c] / sum_b Lr_b and
// ebar[b][c] = C_b / Omega_tot (T[c] - T_ref).  A block covers 32 cells with
// 8 band slices (thread (x, y): cell x, bands y, y + 8, ...), so every load and
// store is coalesced along the cells and the grid has n / 32 blocks; the 8
// slice sums are added in slice order.
constexpr int RC_CELLS = 32, RC_SLICES = 8;
__global__ void __launch_bounds__(RC_CELLS * RC_SLICES)
    k_recover(const double* __restrict__ Tb, const double* __restrict__ Cb, const double* __restrict__ Lr,
              double Lr_sum, double T_ref, double solid_angle, int n, int n_band, size_t Np, double* T,
              double* ebar) {
    __shared__ double part[RC_SLICES][RC_CELLS];
    __shared__ double tc[RC_CELLS];
    const int x = threadIdx.x % RC_CELLS, y = threadIdx.x / RC_CELLS;
    const int c = blockIdx.x * RC_CELLS + x;
    double acc = 0.0;
    if (c < n)
        for (int b = y; b < n_band; b += RC_SLICES) acc += Lr[b] * Tb[(size_t)b * Np + c];
    part[y][x] = acc;
    __syncthreads();
    if (y == 0) {
        double t = 0.0;
        for (int k = 0; k < RC_SLICES; ++k) t += part[k][x];
        tc[x] = t / Lr_sum;
        if (c < n) T[c] = tc[x];
    }
    __syncthreads();
    if (c < n) {
        const double Tc = tc[x];
        for (int b = y; b < n_band; b += RC_SLICES) ebar[(size_t)b * Np + c] = Cb[b] / solid_angle * (Tc - T_ref);
    }
}

// margin = sum of partials / (n_band n_cell).  One block: thread t sums
// partials t, t+256, ... in order, then a fixed-order block reduction, so the
// result does not depend on timing.
__global__ void __launch_bounds__(THREADS) k_margin_final(const double* part, int nparts, double denom, double* out) {
    __shared__ double sm[1][NWARP];
    double v[1] = {0.0};
    for (int i = threadIdx.x; i < nparts; i += THREADS) v[0] += part[i];
    block_sum<1>(v, sm);
    if (threadIdx.x == 0) out[0] = v[0] / denom;
}

// Heat flux, step 1 (src/StaticBTESolver.cpp:331-354): per (band, boundary face),
// sum over all directions of e * hw[face][d], hw = (s.n) A Omega (DM 3 on a 3D
// mesh), (S.n) A (other 2D/3D), (s.n) Omega (1D).
__global__ void k_heat_face(const double* __restrict__ e, const int* __restrict__ bf_cell,
                            const double* __restrict__ hw, int nbf, int n_band, int n_dir, size_t Np,
                            double* part) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nbf * n_band) return;
    const int b = t / nbf, k = t % nbf;
    const double* ep = e + (size_t)b * n_dir * Np + bf_cell[k];
    const double* w = hw + (size_t)k * n_dir;
    double acc = 0.0;
    for (int d = 0; d < n_dir; ++d) acc += ep[(size_t)d * Np] * w[d];
    part[(size_t)b * nbf + k] = acc;
}

// Heat flux, step 2 (:357-364): per (boundary condition, band), sum the faces
// in (cell, face) order, divide by the wall length (not in 1D), times v_g;
// q[i] = sum over bands.  One block.
__global__ void k_heat_final(const double* __restrict__ part, const int* __restrict__ bf_bc,
                             const double* __restrict__ bf_area, const double* __restrict__ vg, int nbf,
                             int n_band, int n_bc, int dim, double* q_band, double* q) {
    for (int t = threadIdx.x; t < n_bc * n_band; t += blockDim.x) {
        const int i = t / n_band, b = t % n_band;
        double heat = 0.0, length = 0.0;
        for (int k = 0; k < nbf; ++k) {
            if (bf_bc[k] != i) continue;
            heat += part[(size_t)b * nbf + k];
            length += bf_area[k];
        }
        q_band[(size_t)i * n_band + b] = dim != 1 ? heat / length * vg[b] : heat * vg[b];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n_bc; i += blockDim.x) {
        double s = 0.0;
        for (int b = 0; b < n_band; ++b) s += q_band[(size_t)i * n_band + b];
        q[i] = s;
    }
}

}  // namespace bte

namespace bte {

// ---------------------------------------------------------------------------
// Upwind sweep: for direction d the system couples a cell only to its inflow
// neighbours, so in topological ("level") order of the upwind graph it is
// lower triangular and one forward substitution solves it exactly:
//   x[c] = (R[c] - k_b sum_{inflow f} fc[d][f][c] x[nb]) / (k_b dg[d][c] + vo[d][c]).
// Cells of one level depend only on earlier levels.  Edges that close a cycle
// of the upwind graph (none on Delaunay triangulations) are "lagged": their
// upstream cell sits on a later level, so the substitution reads its previous
// value (a Gauss-Seidel sweep) and the host repeats sweeps until the
// residual test passes.
//
// Sweep-ordered arrays, direction-major, position j in level order:
//   sw_cell[d][j], sw_dg[d][j], sw_vo[d][j], sw_fc[d][k][j], and sw_nb[d][k][j]
//   = the upstream cell's POSITION in this direction's order (-1 none,
//   -2-position for a lagged edge) for the k-th inflow face of the cell (slots
//   k = 0 .. F-1, inflow faces first in face order, the rest -1); levels
//   lvl[lvl_off[d] .. lvl_off[d+1]] are start positions (the last entry is n).
struct SweepPlan {
    const int* cell;
    const int* bidx;  // [n_dir][n] row of the cell in the boundary-cell list, -1 interior
    const double* dg;
    const double* vo;
    const int* nb;
    const double* fc;
    const int* lvl;
    const int* lvl_off;
    int n, F;
    int n2;  // row length of the per-system arrays (voi, kinv): n rounded up to even
};

// The diagonal folded into the sweep's coefficients, per system in level
// order: with D = k_b dg[d][j] + vo[d][j],
//   voi[b][d][j] = vo / D,   kinv[b][d][j] = k_b / D,
// so x = (R - k_b off) / D becomes x = ebar voi + bs/D - kinv off: two FP64
// operations per cell fewer in the sweep (GB300 issues FP64 at ~2 lanes per SM
// per clock).  The diagonal does not change across outer iterations: once per solve.
__global__ void k_sweep_invd(SweepPlan sp, const double* __restrict__ kb, int n_band, int n_dir, double* voi,
                             double* kinv) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int d = blockIdx.y;
    if (j >= sp.n) return;
    const size_t pj = (size_t)d * sp.n + j;
    const double vo = sp.vo[pj], dg = sp.dg[pj];
    for (int b = 0; b < n_band; ++b) {
        const double invD = 1.0 / fma(kb[b], dg, vo);
        const size_t q = ((size_t)b * n_dir + d) * sp.n2 + j;
        voi[q] = vo * invD;
        kinv[q] = kb[b] * invD;
    }
}

// Operands of one sweep item that do not depend on the level being solved
// (FM = faces per cell: 2, 3 or 4).
template <int FM>
struct SweepItem {
    int c, bi;
    int u[FM];
    double cf[FM];
    double kinv, voi, eb, bs, old;
};

// The cell-addressed operands come from SweepSrc (ebar, the boundary part of
// the right-hand side, and with MARGIN the previous iterate).
struct SweepSrc {
    const double* ebar;   // [n_band][Np]
    const double* bsum;   // [nbb * n_dir][nbcell] (k_bound_rhs)
    const double* x_old;  // e_prev
    int nbcell;
};

// Row pointers of one thread's (band, direction) system, computed once per
// block so the per-item work is 32-bit indexing only.
struct SweepRows {
    const int* cell;   // [n] level order of direction d
    const int* bidx;   // [n]
    const int* nb;     // [F][n]
    const double* fc;  // [F][n]
    const double* voi; // [n] this band
    const double* kinv;
    const double* eb;  // ebar of this band, by cell
    const double* bs;  // boundary part of this system, by boundary row
    const double* xold;
    int n, F;
};

// Stage A: everything addressed by the position j alone.
template <int FM>
__device__ __forceinline__ void sweep_load_a(const SweepRows& r, int j, SweepItem<FM>& it) {
    it.c = r.cell[j];
#pragma unroll
    for (int f = 0; f < FM; ++f) {
        it.u[f] = r.nb[f * r.n + j];
        it.cf[f] = r.fc[f * r.n + j];
    }
    it.kinv = r.kinv[j];
    it.voi = r.voi[j];
    it.bi = r.bidx[j];
}

// Stage B: what is addressed by the cell, issued a level after stage A so the
// cell index has arrived and the loads do not stall the sweep.
template <bool MARGIN, int FM>
__device__ __forceinline__ void sweep_load_b(const SweepRows& r, SweepItem<FM>& it) {
    it.eb = r.eb[it.c];
    it.bs = it.bi >= 0 ? r.bs[it.bi] : 0.0;
    if (MARGIN) it.old = r.xold[it.c];
}

// Fixed-order sum over a block of any whole-warp size (<= 1024 threads); the
// result is valid in thread 0.
__device__ __forceinline__ double block_sum_any(double v, double* smem /* [32] */) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0) smem[warp] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < nw; ++w) s += smem[w];
    return s;
}

// One block sweeps direction blockIdx.y for bands b0 + blockIdx.x * G .. + G - 1.
// x and x_old are e_curr / e_prev ([band][n_dir][Np]).  Thread t serves band
// t mod gp (gp = the power of two >= the block's band count, which divides
// the block size) at positions t / gp, t / gp + blockDim / gp, ... of each
// level, so each thread's band -- and its row pointers -- are fixed.  Each
// thread's first item of the next two levels is loaded ahead (everything but
// the upstream values), and the block keeps its last W solved positions per
// band in a shared-memory ring, so after a level barrier the upstream values
// come from shared memory.  A position p is still in the ring during the
// level [j0, j1) whenever p >= j1 - W: no position written in this level maps
// to its slot.  W is a power of two.  Older and lagged upstream values are
// read from global memory.
// At most 128 threads, 5 blocks per SM (<= 96 registers, no spills): 640
// blocks of the 40-band, 32-direction workload fit in one wave.
// MARGIN (acyclic plans: one sweep is the exact solve): the block also sums
// (x - x_old)^2 over its items, in a fixed order, into
// mpart[d * n_band + b0 + blockIdx.x * G], the outer iteration's margin partial.
// FM = the plan's face slots (inflow faces first).
template <bool MARGIN, int FM>
__global__ void __launch_bounds__(128, 5) k_sweep(SweepPlan sp, const double* __restrict__ voi,
                                                  const double* __restrict__ kinv, SweepSrc src, double* x,
                                                  int first_sweep, int G, int W, int nbb, int b0, int n_band,
                                                  int n_dir, size_t Np, double* __restrict__ mpart) {
    extern __shared__ double ring[];  // [G][W]
    __shared__ double red[32];
    const int d = blockIdx.y;
    const int g0 = blockIdx.x * G;
    const int gn = min(G, nbb - g0);
    if (gn <= 0) return;
    int gp = 1;
    while (gp < gn) gp <<= 1;
    const int sh = __ffs(gp) - 1;
    const int bl = threadIdx.x & (gp - 1);
    const bool serves = bl < gn;  // threads of a padded band slot only load
    const int b = b0 + g0 + (serves ? bl : 0);
    const int n = sp.n;
    const size_t sys = (size_t)b * n_dir + d;
    SweepRows rows;
    rows.cell = sp.cell + (size_t)d * n;
    rows.bidx = sp.bidx + (size_t)d * n;
    rows.nb = sp.nb + (size_t)d * sp.F * n;
    rows.fc = sp.fc + (size_t)d * sp.F * n;
    rows.voi = voi + sys * sp.n2;
    rows.kinv = kinv + sys * sp.n2;
    rows.eb = src.ebar + (size_t)b * Np;
    rows.bs = src.bsum + ((size_t)d * nbb + (b - b0)) * src.nbcell;
    rows.xold = src.x_old + sys * Np;
    rows.n = n;
    rows.F = sp.F;
    double* xb = x + sys * Np;
    double* rg = ring + (size_t)bl * W;
    const int* cell_d = rows.cell;
    const int per_round = blockDim.x >> sh;  // positions per round of the block
    const int tpos = threadIdx.x >> sh;      // this thread's first position in a level
    const int L0 = sp.lvl_off[d], L1 = sp.lvl_off[d + 1] - 1;  // levels L0 .. L1-1
    SweepItem<FM> p1, p2;  // this thread's first item of levels l and l+1
    bool h1 = false, h2 = false;
    double msum = 0.0;
    // level bounds carried from level to level: lA, lB, lC = starts of levels
    // l, l+1, l+2 (the last start is n), so a level begins without a load
    const int* lvl = sp.lvl;
    int lA = lvl[L0], lB = lvl[L0 + 1], lC = L0 + 2 <= L1 ? lvl[L0 + 2] : lB;
    auto pre = [&](int j_begin, int j_end, SweepItem<FM>& dst) -> bool {
        const int j = j_begin + tpos;
        if (j >= j_end) return false;
        sweep_load_a(rows, j, dst);
        return true;
    };
    h1 = pre(lA, lB, p1);
    if (h1) sweep_load_b<MARGIN, FM>(rows, p1);
    h2 = L0 + 1 < L1 && pre(lB, lC, p2);
    for (int l = L0; l < L1; ++l) {
        const int j0 = lA, j1 = lB;
        const int lD = l + 3 <= L1 ? lvl[l + 3] : lC;  // for the prefetch of level l+2, issued now
        const int keep = j1 - W;  // oldest position still readable from the ring
        for (int j = j0 + tpos; j < j1; j += per_round) {
            SweepItem<FM> cur;
            if (j == j0 + tpos && h1) cur = p1;
            else {
                sweep_load_a(rows, j, cur);
                sweep_load_b<MARGIN, FM>(rows, cur);
            }
            if (!serves) continue;
            double off = 0.0;
#pragma unroll
            for (int f = 0; f < FM; ++f) {
                const int u = cur.u[f];
                if (u == -1) continue;
                double xu;
                if (u >= 0) xu = u >= keep ? rg[u & (W - 1)] : xb[cell_d[u]];
                else {  // lagged (u = -2 - position): previous sweep's value (or the previous outer iterate)
                    const int cu = cell_d[-u - 2];
                    xu = first_sweep ? rows.xold[cu] : xb[cu];
                }
                off = fma(cur.cf[f], xu, off);
            }
            const double v = fma(-cur.kinv, off, fma(cur.eb, cur.voi, cur.bs));
            xb[cur.c] = v;
            rg[j & (W - 1)] = v;
            if (MARGIN) {
                const double df = v - cur.old;
                msum = fma(df, df, msum);
            }
        }
        p1 = p2;
        h1 = h2;
        if (h1) sweep_load_b<MARGIN, FM>(rows, p1);
        h2 = l + 2 < L1 && pre(lC, lD, p2);
        lA = lB;
        lB = lC;
        lC = lD;
        __syncthreads();
    }
    if (MARGIN) {
        const double s = block_sum_any(msum, red);
        if (threadIdx.x == 0) mpart[(size_t)d * n_band + b0 + g0] = s;
    }
}

// ---------------------------------------------------------------------------
// Staged sweep: the substitution of k_sweep with every operand of a level
// already in shared memory or in registers when the level starts.
//
// k_sweep's items wait on two dependent loads each level (the cell index, then
// the cell's ebar and boundary value): load latency along the level chain,
// not HBM or the FP64 pipe, sets its time.  Here everything a stage reads by
// position is a contiguous slice of a position-indexed array: the plan
// records (cell, boundary row, upstream positions, face coefficients) and per
// band k/D and V Omega/D.  One thread copies those slices for stage s + 3 into
// one of three shared-memory buffers with 1-D bulk copies (cp.async.bulk,
// completion on an mbarrier) while the block solves stage s.  The gathers by
// cell (ebar, the boundary value) of stage s + 1's items are issued while
// stage s is solved, from the cells in its records, and their right-hand
// sides src = ebar voi + bs/D (the fma k_sweep forms) are kept in registers.
// A stage is a level, or a slice of at most `cap` positions of a wider one
// (positions of one level never depend on each other, so splitting a level
// keeps the substitution exact).  The arithmetic is k_sweep's term for term,
// so x is the same to the bit.

// Record of one position in a direction's level order: ints (cell, its
// boundary row or -1, upstream positions of the FM face slots, padding to 16
// bytes), then the FM face coefficients (FP64, padding to 16 bytes).
template <int FM>
struct SweepRecLayout {
    static constexpr int ints = 4 * ((FM + 5) / 4);    // 2 + FM rounded up to 4
    static constexpr int dbls = 2 * ((FM + 1) / 2);    // FM rounded up to 2
    static constexpr int bytes = 4 * ints + 8 * dbls;  // 32 (FM 2), 64 (FM 3, 4)
};

// rec[d][j] from the level-ordered plan arrays (k_sweep_layout's output).
template <int FM>
__global__ void k_sweep_records(const int* __restrict__ cell, const int* __restrict__ bidx,
                                const int* __restrict__ nb, const double* __restrict__ fc, int n, int F, int n_dir,
                                unsigned char* __restrict__ rec) {
    using L = SweepRecLayout<FM>;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int d = blockIdx.y;
    if (j >= n) return;
    unsigned char* r = rec + ((size_t)d * n + j) * L::bytes;
    int* ri = reinterpret_cast<int*>(r);
    double* rd = reinterpret_cast<double*>(r + 4 * L::ints);
    ri[0] = cell[(size_t)d * n + j];
    ri[1] = bidx[(size_t)d * n + j];
    for (int f = 0; f < FM; ++f) {
        const bool in = f < F;
        ri[2 + f] = in ? nb[((size_t)d * F + f) * n + j] : -1;
        rd[f] = in ? fc[((size_t)d * F + f) * n + j] : 0.0;
    }
    for (int k = 2 + FM; k < L::ints; ++k) ri[k] = -1;
    for (int k = FM; k < L::dbls; ++k) rd[k] = 0.0;
}

// Shared-memory barrier and bulk-copy primitives (PTX ISA: mbarrier,
// cp.async.bulk; one CTA, no cluster: the CTA's own shared memory is its
// shared::cluster window).
__device__ __forceinline__ unsigned smem_addr(const void* p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
// One bounded wait for the phase of the given parity: the thread is suspended
// for at most ~1 us (the suspend-time hint) before the call returns false.
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity), "r"(1000u)
        : "memory");
    return ok != 0;
}
// Global -> shared, `bytes` a multiple of 16, both addresses 16-byte aligned.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}
// Orders this thread's earlier generic-proxy accesses to shared memory before
// later async-proxy ones (a bulk copy into a buffer the block has just read).
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Bounded waits on a stage's mbarrier before the block gives up (the copies
// of a stage complete within microseconds; ~1 s at most, then an error).
constexpr long long kStagePolls = 1ll << 20;

// Plan of the staged sweep: records, stage bounds and the level order's cells.
struct StagedPlan {
    const unsigned char* rec;  // [n_dir][n] records (SweepRecLayout<FM>)
    const int* stages;         // per direction: start positions of its stages, then n
    const int* stage_off;      // [n_dir + 1] first entry of direction d in stages
    const int* cell;           // [n_dir][n] level order (lagged and old upstream values)
    int n, n2, cap;            // cells, row length of k/D and src, positions per stage (even)
};

// Bytes of one stage buffer: cap records, then per band of the block k/D and
// V Omega/D slices of cap + 2 doubles (a slice starts at an even position).
template <int FM>
__host__ __device__ constexpr size_t staged_buffer_bytes(int cap, int G) {
    return (size_t)cap * SweepRecLayout<FM>::bytes + sizeof(double) * 2 * (size_t)G * (cap + 2);
}
// Dynamic shared memory of k_sweep_staged: a 64-byte header (three mbarriers,
// the bounds of the stage each buffer holds), the ring of G x W solved
// values, three stage buffers.
template <int FM>
__host__ __device__ constexpr size_t staged_smem_bytes(int cap, int G, int W) {
    return 64 + sizeof(double) * (size_t)G * W + 3 * staged_buffer_bytes<FM>(cap, G);
}

// One block sweeps direction blockIdx.y for the batch's bands blockIdx.x * G
// .. + G - 1 (thread t serves band t mod gp, positions t / gp, t / gp +
// blockDim / gp, ... of each stage, as in k_sweep; cap = 2 blockDim / gp, so a
// thread has at most two items per stage).  x = e_curr, x_old = e_prev
// ([band][n_dir][Np]); kinv and voi [band][n_dir][n2] (all bands); src: ebar
// and the boundary parts.  The ring keeps the last W solved positions per
// band: a position p is still there during the stage [j0, j1) whenever
// p >= j1 - W.  A stage's copies that have not landed after kStagePolls polls
// set *err; the block then waits (bounded) for its copies in flight and
// returns (x is then not valid; the host reports the error).
template <int FM>
__global__ void __launch_bounds__(256) k_sweep_staged(StagedPlan sp, const double* __restrict__ kinv,
                                                      const double* __restrict__ voi, SweepSrc src,
                                                      const double* __restrict__ x_old, double* x, int first_sweep,
                                                      int G, int W, int nbb, int b0, int n_dir, size_t Np, int* err) {
    using L = SweepRecLayout<FM>;
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned long long* bar = reinterpret_cast<unsigned long long*>(smem);  // [3]
    int* hdr = reinterpret_cast<int*>(smem + 32);                           // [3][2] stage bounds per buffer
    double* ring = reinterpret_cast<double*>(smem + 64);                    // [G][W]
    unsigned char* bufs = smem + 64 + sizeof(double) * (size_t)G * W;
    const int cap = sp.cap;
    const size_t rec_bytes = (size_t)cap * L::bytes;
    const int vlen = cap + 2;
    const size_t buf_bytes = staged_buffer_bytes<FM>(cap, G);
    const int d = blockIdx.y;
    const int g0 = blockIdx.x * G;
    const int gn = min(G, nbb - g0);
    if (gn <= 0) return;
    int gp = 1;
    while (gp < gn) gp <<= 1;
    const int sh = __ffs(gp) - 1;
    const int bl = threadIdx.x & (gp - 1);
    const bool serves = bl < gn;
    const int bb = g0 + (serves ? bl : 0);  // band within the batch
    const int n = sp.n, n2 = sp.n2;
    double* xb = x + ((size_t)(b0 + bb) * n_dir + d) * Np;
    const double* xo = x_old + ((size_t)(b0 + bb) * n_dir + d) * Np;
    const double* eb = src.ebar + (size_t)(b0 + bb) * Np;
    const double* bsb = src.bsum + ((size_t)d * nbb + bb) * src.nbcell;
    double* rg = ring + (size_t)bl * W;
    const int* cell_d = sp.cell + (size_t)d * n;
    const unsigned char* rec_d = sp.rec + (size_t)d * n * L::bytes;
    const int* stg = sp.stages + sp.stage_off[d];
    const int ns = sp.stage_off[d + 1] - sp.stage_off[d] - 1;  // stages; stg[0 .. ns]
    const int per_round = blockDim.x >> sh;
    const int tpos = threadIdx.x >> sh;
    // thread 0 copies stage s (bounds j0, j1) into buffer s % 3 and records
    // the bounds in the buffer's header, where the block reads them
    auto issue = [&](int s, int j0, int j1) {
        const int q = s % 3;
        unsigned char* B = bufs + (size_t)q * buf_bytes;
        hdr[2 * q] = j0;
        hdr[2 * q + 1] = j1;
        const int ja = j0 & ~1, jb = (j1 + 1) & ~1;
        const unsigned rb = (unsigned)(j1 - j0) * (unsigned)L::bytes;
        const unsigned vb = (unsigned)(jb - ja) * 8u;
        mbar_arrive_expect_tx(&bar[q], rb + 2u * (unsigned)gn * vb);
        bulk_load(B, rec_d + (size_t)j0 * L::bytes, rb, &bar[q]);
        double* kv = reinterpret_cast<double*>(B + rec_bytes);
        for (int g = 0; g < gn; ++g) {
            const size_t sys = (size_t)(b0 + g0 + g) * n_dir + d;
            bulk_load(kv + (size_t)g * vlen, kinv + sys * n2 + ja, vb, &bar[q]);
            bulk_load(kv + (size_t)(G + g) * vlen, voi + sys * n2 + ja, vb, &bar[q]);
        }
    };
    // a stage's buffer, once its copies have landed (bounded polls)
    auto wait_stage = [&](int s) -> bool {
        long long k = 0;
        while (!mbar_try_wait(&bar[s % 3], (unsigned)(s / 3) & 1u))
            if (++k > kStagePolls) return false;
        return true;
    };
    // the cell-indexed loads of this thread's (at most two) items of stage s
    // (issued a stage ahead), then their right-hand sides
    double geb[2] = {0.0, 0.0}, gbs[2] = {0.0, 0.0}, rhs[2] = {0.0, 0.0};
    auto gather = [&](int s) {
        const int q = s % 3;
        const unsigned char* B = bufs + (size_t)q * buf_bytes;
        const int j0 = hdr[2 * q], j1 = hdr[2 * q + 1];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const int j = j0 + tpos + k * per_round;
            if (j >= j1) continue;
            const int2 cb = *reinterpret_cast<const int2*>(B + (size_t)(j - j0) * L::bytes);
            geb[k] = eb[cb.x];
            gbs[k] = cb.y >= 0 ? bsb[cb.y] : 0.0;
        }
    };
    auto form_rhs = [&](int s) {
        const int q = s % 3;
        const unsigned char* B = bufs + (size_t)q * buf_bytes;
        const int j0 = hdr[2 * q], j1 = hdr[2 * q + 1], ja = j0 & ~1;
        const double* vv = reinterpret_cast<const double*>(B + rec_bytes) + (size_t)(G + bl) * vlen;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const int j = j0 + tpos + k * per_round;
            if (j < j1) rhs[k] = fma(geb[k], vv[j - ja], gbs[k]);
        }
    };
    if (threadIdx.x == 0) {
        for (int q = 0; q < 3; ++q) mbar_init(&bar[q], 1);
        mbar_init_fence();
    }
    __syncthreads();
    int issued = 0;  // thread 0: stages whose copies were issued
    int next_start = 0;  // thread 0: start of the next stage to issue
    if (threadIdx.x == 0) {
        int j = stg[0];
        for (; issued < 3 && issued < ns; ++issued) {
            const int e = stg[issued + 1];
            issue(issued, j, e);
            j = e;
        }
        next_start = j;
    }
    __syncthreads();  // the headers of the first stages
    bool failed = false;
    if (ns > 0) {
        failed = !wait_stage(0);
        if (!failed && serves) {
            gather(0);
            form_rhs(0);
        }
    }
    failed = __syncthreads_or(failed);
    int s = 0;
    for (; s < ns && !failed; ++s) {
        const int q = s % 3;
        // thread 0: the end of stage s + 3, loaded now and used after this stage
        const int next_end = threadIdx.x == 0 ? stg[min(s + 4, ns)] : 0;
        // stage s + 1: its buffer, and the gathers of its items
        const bool ahead = s + 1 < ns;
        if (ahead && !wait_stage(s + 1)) failed = true;
        if (ahead && !failed && serves) gather(s + 1);
        if (!failed && serves) {
            const unsigned char* B = bufs + (size_t)q * buf_bytes;
            const double* kv = reinterpret_cast<const double*>(B + rec_bytes) + (size_t)bl * vlen;
            const int j0 = hdr[2 * q], j1 = hdr[2 * q + 1];
            const int ja = j0 & ~1;
            const int keep = j1 - W;  // oldest position still readable from the ring
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                const int j = j0 + tpos + k * per_round;
                if (j >= j1) continue;
                const unsigned char* r = B + (size_t)(j - j0) * L::bytes;
                int iv[L::ints];
                double dv[L::dbls];
#pragma unroll
                for (int m = 0; m < L::ints / 4; ++m) {
                    const int4 t = reinterpret_cast<const int4*>(r)[m];
                    iv[4 * m] = t.x;
                    iv[4 * m + 1] = t.y;
                    iv[4 * m + 2] = t.z;
                    iv[4 * m + 3] = t.w;
                }
#pragma unroll
                for (int m = 0; m < L::dbls / 2; ++m) {
                    const double2 t = reinterpret_cast<const double2*>(r + 4 * L::ints)[m];
                    dv[2 * m] = t.x;
                    dv[2 * m + 1] = t.y;
                }
                double off = 0.0;
#pragma unroll
                for (int f = 0; f < FM; ++f) {
                    const int u = iv[2 + f];
                    if (u == -1) continue;
                    double xu;
                    if (u >= 0) xu = u >= keep ? rg[u & (W - 1)] : xb[cell_d[u]];
                    else {  // lagged (u = -2 - position): previous sweep's value (or the previous outer iterate)
                        const int cu = cell_d[-u - 2];
                        xu = first_sweep ? xo[cu] : xb[cu];
                    }
                    off = fma(dv[f], xu, off);
                }
                const double v = fma(-kv[j - ja], off, rhs[k]);
                xb[iv[0]] = v;
                rg[j & (W - 1)] = v;
            }
        }
        if (ahead && !failed && serves) form_rhs(s + 1);
        if (__syncthreads_or(failed)) {
            failed = true;
            break;
        }
        if (threadIdx.x == 0 && s + 3 < ns) {
            fence_proxy_async_smem();  // the block's reads of buffer q come before the copy into it
            issue(s + 3, next_start, next_end);
            next_start = next_end;
            ++issued;
        }
    }
    if (failed && threadIdx.x == 0) {
        atomicExch(err, 1);
        // copies still in flight land in this block's shared memory: wait
        // for them (bounded) before the block exits
        for (int r = s; r < issued; ++r) {
            long long k = 0;
            while (!mbar_try_wait(&bar[r % 3], (unsigned)(r / 3) & 1u) && ++k <= kStagePolls) {
            }
        }
    }
}

// Residual test of the sweep solution: partials of ||R - A x||^2 and ||R||^2
// per (row, chunk), positions j in sweep order.
__global__ void __launch_bounds__(THREADS) k_sweep_residual(FaceFluxOp op, RhsSrc src, const int* __restrict__ perm,
                                                            double* part, int nchunk, int n) {
    __shared__ double sm[2][NWARP];
    const int y = blockIdx.y;
    int b, d;
    op.bd(y, b, d);
    const double k = op.kb[b];
    const double* xs = op.x_of(y);
    double acc[2] = {0, 0};
    BTE_CELL_LOOP(j) {
        if (j < n) {
            const int c = perm[(size_t)d * n + j];
            const double R = src.at(b, d, c, k, op.vo[(size_t)d * op.Np + c]);
            const double r = R - op.template apply<double>(y, c, xs);
            acc[0] = fma(r, r, acc[0]);
            acc[1] = fma(R, R, acc[1]);
        }
    }
    block_sum<2>(acc, sm);
    if (threadIdx.x == 0) {
        part[((size_t)y * nchunk + blockIdx.x) * 2] = acc[0];
        part[((size_t)y * nchunk + blockIdx.x) * 2 + 1] = acc[1];
    }
}

// Count rows whose residual still fails ||R - A x|| <= tol ||R||.
__global__ void k_sweep_check(const double* part, int S, int nchunk, double tol, int* n_bad) {
    const int y = blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= S) return;
    double rr = 0, bb = 0;
    for (int i = 0; i < nchunk; ++i) {
        rr += part[((size_t)y * nchunk + i) * 2];
        bb += part[((size_t)y * nchunk + i) * 2 + 1];
    }
    if (!(rr <= tol * tol * bb)) atomicAdd(n_bad, 1);
}

// Inflow-face bit mask per (direction, cell) from the device's own
// coefficients, so the host builds the level order from exactly the couplings
// the kernels use.
__global__ void k_inflow_mask(const double* __restrict__ fc, int F, int n, size_t Np, int n_dir, uint8_t* mask) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int d = blockIdx.y;
    if (c >= n) return;
    uint8_t m = 0;
    for (int f = 0; f < F; ++f)
        if (fc[((size_t)d * F + f) * Np + c] != 0.0) m |= (uint8_t)(1u << f);
    mask[(size_t)d * n + c] = m;
}

// Downstream edges of every direction's upwind graph, for k_level_order.
// mask[d][c] bit f: face f of c is an inflow face; an edge u -> c exists once
// per such face g of c with nbr[c][g] == u.  down[d][u][f] = (k << 28) | c
// when c = nbr[u][f] is named by no earlier face of u and k >= 1 edges run
// u -> c, else -1.  Needs n < 2^28 and F <= 4.
__global__ void k_downstream(const uint8_t* __restrict__ mask, const int* __restrict__ nbr, int n, int F,
                             int* __restrict__ down) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;  // u * F + f
    const int d = blockIdx.y;
    if (q >= (size_t)n * F) return;
    const int u = (int)(q / F), f = (int)(q - (size_t)u * F);
    const int c = nbr[q];
    int out = -1;
    if (c >= 0 && c < n) {
        bool dup = false;
        for (int f2 = 0; f2 < f; ++f2) dup |= nbr[(size_t)u * F + f2] == c;
        if (!dup) {
            const unsigned mc = mask[(size_t)d * n + c];
            int k = 0;
            for (int g = 0; g < F; ++g) k += ((mc >> g) & 1u) && nbr[(size_t)c * F + g] == u;
            if (k > 0) out = (k << 28) | c;
        }
    }
    down[(size_t)d * n * F + q] = out;
}

// Level order of every direction's upwind graph on the device, one block per
// direction: Kahn's algorithm in waves (a wave is the cells whose inflow
// neighbours all lie in earlier waves), each wave sorted by cell index -- the
// order bte::level_order (sweep_order.h) builds on the host, for acyclic
// graphs.  The edges come from k_downstream.
//
// k_level_order_smem keeps the whole state in shared memory: the remaining
// in-degrees, one byte per cell (a cell has at most F <= 4 inflow faces, so a
// byte never borrows from its neighbour), two bitmaps of cells, the current
// wave and the next, and the wave's list (cap cells).  Thread t owns a
// contiguous range of bitmap words, so reading the wave's bits thread by
// thread, in bit order, lists it by cell index: after one block scan of the
// threads' counts each thread writes its cells' positions and list entries,
// then one thread per wave cell releases its downstream cells into the other
// bitmap.  Four block barriers per wave; a wave wider than cap sets status 2.
// Dynamic shared memory: 4 (ceil(n / 4) + 2 ceil(n / 32) + cap) bytes.
// Outputs: perm[d][pos], lvl[d][0 .. nlev] (level starts, then n), the
// largest inflow count over all directions in *fmax; status 1: a cycle (cells
// left when no cell is free) or 2 (a wave wider than cap), the direction is
// left to the host.
__global__ void __launch_bounds__(1024) k_level_order_smem(const uint8_t* __restrict__ mask,
                                                           const int* __restrict__ down, int n, int F, int cap,
                                                           int* __restrict__ perm, int* __restrict__ lvl,
                                                           int* __restrict__ nlev, int* __restrict__ status,
                                                           int* __restrict__ fmax) {
    extern __shared__ unsigned sw[];
    const int nd = (n + 3) / 4, nw = (n + 31) / 32;
    unsigned* deg = sw;         // [nd], 4 cells per word
    unsigned* bmA = sw + nd;    // [nw]
    unsigned* bmB = bmA + nw;   // [nw]
    int* wave = reinterpret_cast<int*>(bmB + nw);  // [cap] the wave's cells in order
    __shared__ int wsum[32];
    const int d = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nwarps = (int)(blockDim.x >> 5);
    const uint8_t* md = mask + (size_t)d * n;
    const int* dd = down + (size_t)d * n * F;
    int* pd = perm + (size_t)d * n;
    int* ld = lvl + (size_t)d * (n + 1);
    int fm = 0;
    for (int w = tid; w < nd; w += blockDim.x) {
        unsigned word = 0;
        for (int q = 0; q < 4 && 4 * w + q < n; ++q) {
            const int k = __popc((unsigned)md[4 * w + q]);
            word |= (unsigned)k << (8 * q);
            fm = max(fm, k);
        }
        deg[w] = word;
    }
    for (int w = tid; w < nw; w += blockDim.x) {
        unsigned bits = 0;
        for (int b = 0; b < 32 && 32 * w + b < n; ++b)
            if (md[32 * w + b] == 0) bits |= 1u << b;
        bmA[w] = bits;
        bmB[w] = 0u;
    }
    if (fm > 0) atomicMax(fmax, fm);
    __syncthreads();
    const int per = (nw + (int)blockDim.x - 1) / (int)blockDim.x;
    const int w0 = min(nw, tid * per), w1 = min(nw, w0 + per);
    unsigned* cur = bmA;
    unsigned* nxt = bmB;
    int pos = 0, level = 0;
    bool over = false;
    for (;;) {
        // block exclusive scan of the threads' wave-cell counts, in thread order
        int cnt = 0;
        for (int w = w0; w < w1; ++w) cnt += __popc(cur[w]);
        int x = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wsum[warp] = x;
        __syncthreads();
        if (warp == 0) {
            int v = lane < nwarps ? wsum[lane] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, v, o);
                if (lane >= o) v += y;
            }
            wsum[lane] = v;
        }
        __syncthreads();
        const int total = wsum[nwarps - 1];
        if (total == 0 || total > cap) {
            over = total > cap;
            break;
        }
        // the wave's cells, by cell index, into its positions and the list
        int o = x - cnt + (warp > 0 ? wsum[warp - 1] : 0);
        for (int w = w0; w < w1; ++w) {
            unsigned bits = cur[w];
            while (bits) {
                const int u = 32 * w + __ffs(bits) - 1;
                bits &= bits - 1;
                pd[pos + o] = u;
                wave[o++] = u;
            }
            cur[w] = 0u;
        }
        if (tid == 0) ld[level] = pos;
        __syncthreads();
        // release the downstream cells, one wave cell per thread
        for (int i = tid; i < total; i += blockDim.x) {
            const int u = wave[i];
            int e[4];
#pragma unroll
            for (int f = 0; f < 4; ++f) e[f] = f < F ? dd[(size_t)u * F + f] : -1;
#pragma unroll
            for (int f = 0; f < 4; ++f) {
                if (e[f] < 0) continue;
                const int c = e[f] & 0x0fffffff, k = e[f] >> 28;
                const unsigned sh = 8u * (unsigned)(c & 3);
                const unsigned old = atomicSub(&deg[c >> 2], (unsigned)k << sh);
                if (((old >> sh) & 0xffu) == (unsigned)k) atomicOr(&nxt[c >> 5], 1u << (c & 31));
            }
        }
        pos += total;
        ++level;
        unsigned* t = cur;
        cur = nxt;
        nxt = t;
        __syncthreads();
    }
    if (tid == 0) {
        const int stat = over ? 2 : (pos < n ? 1 : 0);
        status[d] = stat;
        nlev[d] = level;
        if (stat == 0) ld[level] = n;
    }
}

// k_level_order keeps the in-degrees in global memory, indeg [n_dir][n], for
// meshes whose state does not fit in shared memory: both frontiers live in
// dynamic shared memory, cap cells each (cap a power of two), each wave is
// sorted there (bitonic), and a wave wider than cap sets status 2 (the
// direction is left to the host).  Each thread loads the edges of its wave
// item before the wave is sorted, so the loads overlap the sort.  Outputs
// as k_level_order_smem's.
__global__ void __launch_bounds__(1024) k_level_order(const uint8_t* __restrict__ mask, const int* __restrict__ down,
                                                      int n, int F, int cap, int* __restrict__ indeg,
                                                      int* __restrict__ perm, int* __restrict__ lvl,
                                                      int* __restrict__ nlev, int* __restrict__ status,
                                                      int* __restrict__ fmax) {
    extern __shared__ int fr[];  // [2][cap]
    __shared__ int cnt[2];
    __shared__ int s_over;
    const int d = blockIdx.x;
    const uint8_t* md = mask + (size_t)d * n;
    int* ind = indeg + (size_t)d * n;
    const int* dd = down + (size_t)d * n * F;
    int* pd = perm + (size_t)d * n;
    int* ld = lvl + (size_t)d * (n + 1);
    if (threadIdx.x == 0) {
        cnt[0] = 0;
        cnt[1] = 0;
        s_over = 0;
    }
    __syncthreads();
    int fm = 0;
    auto seed = [&](int c, int k) {
        fm = max(fm, k);
        if (k == 0) {
            const int slot = atomicAdd(&cnt[0], 1);
            if (slot < cap) fr[slot] = c;
            else s_over = 1;
        }
    };
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
        const int k = __popc((unsigned)md[c]);
        ind[c] = k;
        seed(c, k);
    }
    if (fm > 0) atomicMax(fmax, fm);
    __syncthreads();
    int cur = 0, pos = 0, level = 0;
    for (;;) {
        const int m = cnt[cur];
        if (m == 0 || s_over) break;
        int* a = fr + (size_t)cur * cap;
        int* b = fr + (size_t)(cur ^ 1) * cap;
        // bitonic sort of the wave, padded to a power of two (<= cap) with INT_MAX
        int P = 1;
        while (P < m) P <<= 1;
        const bool regs = P <= (int)blockDim.x;
        const int i = threadIdx.x;
        int dn[4] = {-1, -1, -1, -1};  // the edges of this thread's (unsorted) item
        if (regs && i < m) {
            const int u = a[i];
#pragma unroll
            for (int f = 0; f < 4; ++f)
                if (f < F) dn[f] = dd[(size_t)u * F + f];
        }
        if (threadIdx.x == 0) cnt[cur ^ 1] = 0;  // read last before the previous wave's final barrier
        if (regs) {
            // one element per thread: compare-exchange partners closer than a
            // warp through shuffles, the others through shared memory
            int x = i < m ? a[i] : INT_MAX;
            for (int k = 2; k <= P; k <<= 1)
                for (int j = k >> 1; j > 0; j >>= 1) {
                    int y;
                    if (j >= 32) {
                        __syncthreads();
                        if (i < P) a[i] = x;
                        __syncthreads();
                        y = i < P ? a[i ^ j] : INT_MAX;
                    } else {
                        y = __shfl_xor_sync(0xffffffffu, x, j);
                    }
                    const bool lower = (i & j) == 0, up = (i & k) == 0;
                    // keep the smaller of the pair in the lower slot of an ascending run
                    if (i < P) x = (lower == up) ? min(x, y) : max(x, y);
                }
            __syncthreads();
            if (i < P) a[i] = x;
            __syncthreads();
        } else {
            for (int t = m + threadIdx.x; t < P; t += blockDim.x) a[t] = INT_MAX;
            __syncthreads();
            for (int k = 2; k <= P; k <<= 1)
                for (int j = k >> 1; j > 0; j >>= 1) {
                    for (int t = threadIdx.x; t < P; t += blockDim.x) {
                        const int l = t ^ j;
                        if (l > t) {
                            const int x = a[t], y = a[l];
                            if ((x > y) == ((t & k) == 0)) {
                                a[t] = y;
                                a[l] = x;
                            }
                        }
                    }
                    __syncthreads();
                }
        }
        for (int t = threadIdx.x; t < m; t += blockDim.x) pd[pos + t] = a[t];
        if (threadIdx.x == 0) ld[level] = pos;
        // release the wave's downstream cells into the other frontier
        auto relax = [&](int e) {
            if (e < 0) return;
            const int c = e & 0x0fffffff, k = e >> 28;
            if (atomicSub(&ind[c], k) == k) {
                const int slot = atomicAdd(&cnt[cur ^ 1], 1);
                if (slot < cap) b[slot] = c;
                else s_over = 1;
            }
        };
        if (regs) {
#pragma unroll
            for (int f = 0; f < 4; ++f) relax(dn[f]);
        } else {
            for (int t = threadIdx.x; t < m; t += blockDim.x)
                for (int f = 0; f < F; ++f) relax(dd[(size_t)a[t] * F + f]);
        }
        pos += m;
        ++level;
        cur ^= 1;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const int stat = s_over ? 2 : (pos < n ? 1 : 0);
        status[d] = stat;
        nlev[d] = level;
        if (stat == 0) ld[level] = n;
    }
}

// pos[d][perm[d][j]] = j: the position of each cell in direction d's order.
__global__ void k_inverse_perm(const int* __restrict__ perm, int n, int* __restrict__ pos) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int d = blockIdx.y;
    if (j < n) pos[(size_t)d * n + perm[(size_t)d * n + j]] = j;
}

// Gather the per-direction geometry into level order.
__global__ void k_sweep_layout(const int* __restrict__ perm, const int* __restrict__ pos,  // pos [n_dir][n]: cell -> position
                               const int* __restrict__ lagged,  // [n_dir][F][n] 0/1, or null: none
                               const double* __restrict__ dg, const double* __restrict__ vo,
                               const double* __restrict__ fc, const int* __restrict__ nbr,  // nbr [n][F]
                               const int* __restrict__ bidx,                                // [n] boundary-cell row or -1
                               int F, int n, size_t Np, int n_dir, int* cell, int* sbidx, double* sdg, double* svo,
                               int* snb, double* sfc) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int d = blockIdx.y;
    if (j >= n) return;
    const size_t pj = (size_t)d * n + j;
    const int c = perm[pj];
    cell[pj] = c;
    sbidx[pj] = bidx[c];
    sdg[pj] = dg[(size_t)d * Np + c];
    svo[pj] = vo[(size_t)d * Np + c];
    // inflow faces first, in face order (the sweep adds their terms in the
    // same order, so the compaction does not change a bit of x); the slots
    // after them hold -1 / 0 and the sweep is instantiated for the largest
    // inflow count (2D triangles: 2 of 3 faces, 3D tetrahedra: 3 of 4)
    int k = 0;
    for (int f = 0; f < F; ++f) {
        const double v = fc[((size_t)d * F + f) * Np + c];
        if (v == 0.0) continue;
        const size_t q = ((size_t)d * F + k) * n + j;
        const int pu = pos[(size_t)d * n + nbr[(size_t)c * F + f]];
        sfc[q] = v;
        snb[q] = lagged && lagged[((size_t)d * F + f) * n + c] ? -2 - pu : pu;
        ++k;
    }
    for (; k < F; ++k) {
        const size_t q = ((size_t)d * F + k) * n + j;
        sfc[q] = 0.0;
        snb[q] = -1;
    }
}

}  // namespace bte

namespace bte {

// ---------------------------------------------------------------------------
// Mixed form: FP32 BiCGSTAB corrections inside FP64 iterative refinement.

// FP32 copy of the per-direction geometry scaled by kappa[d].
__global__ void k_geometry32(const double* __restrict__ dg, const double* __restrict__ vo,
                             const double* __restrict__ fc, const double* __restrict__ kappa, int n, int F,
                             size_t Np, float* dg32, float* vo32, float* fc32) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int d = blockIdx.y;
    if (c >= Np) return;
    const size_t dc = (size_t)d * Np + c;
    const double k = kappa[d];
    dg32[dc] = (float)(dg[dc] * k);
    vo32[dc] = c < n ? (float)(vo[dc] * k) : 1.0f;
    for (int f = 0; f < F; ++f) {
        const size_t q = ((size_t)d * F + f) * Np + c;
        fc32[q] = (float)(fc[q] * k);
    }
}

// Warm start: x (e_curr) = previous outer iterate (e_prev) for every system of the batch.
__global__ void __launch_bounds__(THREADS) k_mixed_start(FaceFluxOp op, const double* __restrict__ e_prev) {
    const int y = blockIdx.y;
    int b, d;
    op.bd(y, b, d);
    const size_t off = ((size_t)b * op.n_dir + d) * op.Np;
    BTE_CELL_LOOP(c) { op.x_out[off + c] = e_prev[off + c]; }
}

// FP64 residual r = b - A x of every system; r32 = kappa_d r for the FP32
// correction solve; partials of ||r||^2 and ||b||^2 per (system, chunk).
__global__ void __launch_bounds__(THREADS) k_mixed_residual(FaceFluxOp op, const double* __restrict__ rhs,
                                                            const double* __restrict__ kappa, float* r32,
                                                            double* part, int nchunk, int n) {
    __shared__ double sm[2][NWARP];
    const int y = blockIdx.y;
    int b, d;
    op.bd(y, b, d);
    const size_t o = (size_t)y * op.Np;
    const double* xs = op.x_of(y);
    const double k = kappa[d];
    double acc[2] = {0, 0};
    BTE_CELL_LOOP(c) {
        double r = 0.0;
        if (c < n) {
            r = rhs[o + c] - op.template apply<double>(y, c, xs);
            acc[0] = fma(r, r, acc[0]);
            acc[1] = fma(rhs[o + c], rhs[o + c], acc[1]);
        }
        r32[o + c] = (float)(k * r);
    }
    block_sum<2>(acc, sm);
    if (threadIdx.x == 0) {
        part[((size_t)y * nchunk + blockIdx.x) * 2] = acc[0];
        part[((size_t)y * nchunk + blockIdx.x) * 2 + 1] = acc[1];
    }
}

// skip[y] = 1 when ||b - A x|| <= tol ||b|| (the reference's criterion for x0 = 0).
__global__ void k_mixed_check(const double* part, int S, int nchunk, double tol, int* skip, int* n_active) {
    const int y = blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= S) return;
    double rr = 0, bb = 0;
    for (int i = 0; i < nchunk; ++i) {
        rr += part[((size_t)y * nchunk + i) * 2];
        bb += part[((size_t)y * nchunk + i) * 2 + 1];
    }
    const int ok = rr <= tol * tol * bb;
    skip[y] = ok;
    if (!ok) atomicAdd(n_active, 1);
}

// x += dx for the systems that were corrected.
__global__ void __launch_bounds__(THREADS) k_mixed_update(FaceFluxOp op, const float* __restrict__ dx,
                                                          const int* __restrict__ skip) {
    const int y = blockIdx.y;
    if (skip[y]) return;
    double* x = op.x_of(y);
    const size_t o = (size_t)y * op.Np;
    BTE_CELL_LOOP(c) { x[c] += (double)dx[o + c]; }
}

}  // namespace bte
