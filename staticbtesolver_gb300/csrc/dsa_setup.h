// Host side of the diffusion-synthetic acceleration (DSA) of the outer
// iteration: the face coefficients of its low-order diffusion operator.
// Plain C++ (no CUDA), so it is also compiled into host tests.
//
// The source iteration's change r = T_new - T_old of one outer iteration is,
// cell by cell, the divergence of the upwind scheme's band energy fluxes
// weighted by Lr (src/StaticBTESolver.cpp:96-120 with _get_Ke :122-160).
// For a temperature field that varies slowly over a mean free path the
// discrete flux through a face f between cells c and c' is, to first order,
//   F_f = (A_f / Omega_tot) sum_b Lr_b Lambda_b (Gabs_f + beta Lambda_b q_f / delta_f) (T_c - T_c')
// with Lambda_b = v_b tau_b, Gabs_f = 1/2 sum_d |g_df| (the upwind scheme's
// own numerical diffusion, g_df = S_d.n_f in 2D/3D), q_f = sum_d g_df (s_d.n_f)
// (the physical second moment) and delta_f the distance between the cells'
// centroids along n_f.  The DSA step solves sum_f W_f (x_c - x_c') = V_c r_c
// for the remaining error x and adds it to T.  Faces on isothermal walls (and
// boundary faces that no boundary-condition row names, whose wall energy the
// reference leaves at 0) hold x = 0 on the wall; diffuse and specular walls
// are adiabatic and carry no term.  The operator is symmetric by
// construction: each interior face is evaluated once and stored on both sides.
#pragma once

#include <algorithm>
#include <cmath>
#include <numeric>
#include <thread>
#include <vector>

namespace bte {

struct DsaCoefficients {
    std::vector<double> W;   // [F][n] face coefficient (0: no coupling)
    std::vector<int> nb;     // [F][n] neighbour of the coupling, -1 for a wall or none
    std::vector<double> diag;  // [n] sum of the cell's face coefficients
    int n_dirichlet = 0;     // wall faces held at x = 0
};

// dirichlet[c*F+f] != 0: boundary face (c, f) is held at fixed temperature.
// beta scales the physical second-moment term (0: numerical diffusion only).
inline void dsa_coefficients(int dim, int n, int F, const int* nbr, const double* area, const double* normal,
                             const double* volume, int n_dir, const double* s, const double* S, double solid_angle,
                             int n_band, const double* vg, const double* tau, const double* Lr,
                             const std::vector<char>& dirichlet, double beta, DsaCoefficients& out) {
    double lr_sum = 0.0;
    for (int b = 0; b < n_band; ++b) lr_sum += Lr[b];
    double a1 = 0.0, a2 = 0.0;  // sum_b Lr_b Lambda_b, sum_b Lr_b Lambda_b^2 (Lr normalised)
    for (int b = 0; b < n_band; ++b) {
        const double lam = vg[b] * tau[b], w = Lr[b] / lr_sum;
        a1 += w * lam;
        a2 += w * lam * lam;
    }
    const double* G = dim > 1 ? S : s;  // g = S.n (s.n on 1D meshes)
    out.W.assign((size_t)F * n, 0.0);
    out.nb.assign((size_t)F * n, -1);
    out.diag.assign(n, 0.0);
    out.n_dirichlet = 0;
    const double hfac = (double)dim / (dim + 1);  // centroid-to-face distance = hfac V / A (simplices)
    auto coefficient = [&](int c, int f, double delta) {
        const double* nn = normal + ((size_t)c * F + f) * 3;
        double gabs = 0.0, q = 0.0;
        for (int d = 0; d < n_dir; ++d) {
            const double g = G[3 * d] * nn[0] + G[3 * d + 1] * nn[1] + G[3 * d + 2] * nn[2];
            const double sn = s[3 * d] * nn[0] + s[3 * d + 1] * nn[1] + s[3 * d + 2] * nn[2];
            gabs += std::fabs(g);
            q += g * sn;
        }
        gabs *= 0.5;
        return area[(size_t)c * F + f] / solid_angle * (gabs * a1 + beta * a2 * q / delta);
    };
    // Each stored face's coefficient (the expensive part: a sum over the
    // directions) and its two slots, cells split over host threads.  A face
    // between c and o > c is stored by c: its own slot (c, f) and the mirror
    // slot (o, back), back the first face of o that names c; no other face
    // writes either slot (a second face of c naming o, on a degenerate mesh,
    // rewrites the same mirror on the same thread), so the threads never
    // share one.  The diagonal is then each cell's slots summed in face order.
    const int nth = std::max(1, std::min(16, (int)std::thread::hardware_concurrency()));
    const int T = std::max(1, std::min(nth, n / 8192));
    std::vector<int> fixed_count(T, 0);
    auto run = [&](int t) {
        for (int c = t; c < n; c += T)
            for (int f = 0; f < F; ++f) {
                const size_t cf = (size_t)c * F + f;
                const int o = nbr[cf];
                const double A = area[cf];
                if (!(A > 0.0)) continue;
                if (o < 0 || o >= n) {
                    if (o < 0 && dirichlet[cf]) {
                        out.W[(size_t)f * n + c] = coefficient(c, f, hfac * volume[c] / A);
                        ++fixed_count[t];
                    }
                    continue;
                }
                if (o <= c) continue;  // evaluated once, from the lower-numbered cell
                int back = -1;
                for (int g = 0; g < F; ++g)
                    if (nbr[(size_t)o * F + g] == c) { back = g; break; }
                if (back < 0) continue;  // a one-sided link (no face of o names c): left out
                const double w = coefficient(c, f, hfac * (volume[c] + volume[o]) / A);
                out.W[(size_t)f * n + c] = w;
                out.nb[(size_t)f * n + c] = o;
                out.W[(size_t)back * n + o] = w;
                out.nb[(size_t)back * n + o] = c;
            }
    };
    auto diag = [&](int t) {
        for (int c = t; c < n; c += T) {
            double sum = 0.0;
            for (int f = 0; f < F; ++f) sum += out.W[(size_t)f * n + c];
            out.diag[c] = sum;
        }
    };
    if (T == 1) {
        run(0);
        diag(0);
    } else {
        std::vector<std::thread> pool;
        for (int t = 0; t < T; ++t) pool.emplace_back(run, t);
        for (auto& th : pool) th.join();
        pool.clear();
        for (int t = 0; t < T; ++t) pool.emplace_back(diag, t);
        for (auto& th : pool) th.join();
    }
    for (int k : fixed_count) out.n_dirichlet += k;
}

// ---------------------------------------------------------------------------
// Two-level preconditioner of the low-order solve.
//
// The low-order operator's conjugate gradients need O(cells across the
// domain) iterations with a diagonal preconditioner: too slow for the smooth
// errors it exists to remove.  The preconditioner adds a coarse correction on
// aggregates of neighbouring cells, M^-1 = I + P A_c^-1 P^T (on the
// Jacobi-scaled operator, P piecewise constant on the aggregates,
// A_c = P^T A P), which resolves every mode longer than an aggregate.  The
// kernel gives each block one contiguous range of cells and splits it into
// `per_block` contiguous aggregates, so the cells are first put in an order in
// which contiguous ranges are compact: a Hilbert curve through the centroids
// (hilbert_order) when they are known, else recursive bisection of the face
// adjacency graph by breadth-first distance (locality_order).

// order[k] = the cell at position k.  Each range of more than `leaf` cells is
// ordered by breadth-first distance from the farthest cell (found by a first
// search from the range's first cell), ties by cell index, and split at the
// median, then each half again; cells the search did not reach (another
// component of the range) go last.  (Searching from a half's end cell without
// the first search saves that search but made the aggregates less compact:
// ~20 % more conjugate-gradient iterations on a 100k-cell square.)  The ranges of one depth are disjoint, so
// they are ordered in parallel (host threads); the result does not depend on
// the thread count.
inline void locality_order(int n, int F, const int* nbr /* [n][F], < 0 none */, int leaf, std::vector<int>& order) {
    order.resize(n);
    std::iota(order.begin(), order.end(), 0);
    // mark[c] = id of the range being ordered that holds c (unique per depth and range)
    std::vector<long long> mark(n, -1);
    std::vector<int> dist(n, -1), scratch(n);
    struct Work {
        std::vector<int> queue, count;
    };
    struct Range {
        int b, e;
    };
    auto split = [&](const Range& r, long long id, Work& w) {
        const int b = r.b, e = r.e;
        auto bfs = [&](int src) {  // distances within the range; returns the last cell reached
            w.queue.clear();
            w.queue.push_back(src);
            dist[src] = 0;
            int last = src;
            for (size_t h = 0; h < w.queue.size(); ++h) {
                const int c = w.queue[h];
                last = c;
                for (int f = 0; f < F; ++f) {
                    const int o = nbr[(size_t)c * F + f];
                    if (o < 0 || o >= n || mark[o] != id || dist[o] >= 0) continue;
                    dist[o] = dist[c] + 1;
                    w.queue.push_back(o);
                }
            }
            return last;
        };
        for (int k = b; k < e; ++k) { mark[order[k]] = id; dist[order[k]] = -1; }
        const int far = bfs(order[b]);
        for (int k = b; k < e; ++k) dist[order[k]] = -1;
        bfs(far);
        // (distance, index) order: an index sort, then a stable counting sort by distance
        std::sort(order.begin() + b, order.begin() + e);
        int dmax = 0;
        for (int k = b; k < e; ++k) dmax = std::max(dmax, dist[order[k]]);
        w.count.assign((size_t)dmax + 3, 0);
        for (int k = b; k < e; ++k) ++w.count[(dist[order[k]] < 0 ? dmax + 1 : dist[order[k]]) + 1];
        for (int v = 1; v < dmax + 3; ++v) w.count[v] += w.count[v - 1];
        for (int k = b; k < e; ++k) {
            const int c = order[k];
            scratch[b + w.count[dist[c] < 0 ? dmax + 1 : dist[c]]++] = c;
        }
        std::copy(scratch.begin() + b, scratch.begin() + e, order.begin() + b);
    };
    const int nth = std::max(1, std::min(16, (int)std::thread::hardware_concurrency()));
    std::vector<Work> work(nth);
    std::vector<Range> ranges{{0, n}}, next;
    for (long long depth = 0; !ranges.empty(); ++depth) {
        std::vector<Range> todo;
        long long cells = 0;
        for (const Range& r : ranges)
            if (r.e - r.b > std::max(leaf, 1)) {
                todo.push_back(r);
                cells += r.e - r.b;
            }
        // threads only where there is enough work to pay for starting them
        const int T = (int)std::min<long long>({(long long)nth, (long long)todo.size(), cells / 16384 + 1});
        auto run = [&](int t) {
            for (size_t i = t; i < todo.size(); i += T) split(todo[i], depth * (long long)n + todo[i].b, work[t]);
        };
        if (T <= 1) {
            if (!todo.empty()) run(0);
        } else {
            std::vector<std::thread> pool;
            for (int t = 0; t < T; ++t) pool.emplace_back(run, t);
            for (auto& th : pool) th.join();
        }
        next.clear();
        for (const Range& r : todo) {
            const int mid = r.b + (r.e - r.b) / 2;
            next.push_back({r.b, mid});
            next.push_back({mid, r.e});
        }
        ranges.swap(next);
    }
}

// Position of a point on a Hilbert curve through a 2^b x 2^b (x 2^b) grid:
// the published transpose algorithm of J. Skilling, "Programming the Hilbert
// curve", AIP Conf. Proc. 707 (2004) 381 -- undo the excess work of the
// Gray-code walk from the top bit down, Gray-encode, then read the key's bits
// from the transposed coordinates, most significant first.  x[0..dim-1] < 2^b,
// dim * b <= 64.  Consecutive keys are neighbouring grid cells.
inline unsigned long long hilbert_key(unsigned x[3], int dim, int b) {
    const unsigned top = 1u << (b - 1);
    for (unsigned q = top; q > 1; q >>= 1) {
        const unsigned low = q - 1;
        for (int i = 0; i < dim; ++i) {
            if (x[i] & q) {
                x[0] ^= low;
            } else {
                const unsigned t = (x[0] ^ x[i]) & low;
                x[0] ^= t;
                x[i] ^= t;
            }
        }
    }
    for (int i = 1; i < dim; ++i) x[i] ^= x[i - 1];
    unsigned t = 0;
    for (unsigned q = top; q > 1; q >>= 1)
        if (x[dim - 1] & q) t ^= q - 1;
    for (int i = 0; i < dim; ++i) x[i] ^= t;
    unsigned long long key = 0;
    for (int q = b - 1; q >= 0; --q)
        for (int i = 0; i < dim; ++i) key = (key << 1) | ((x[i] >> q) & 1u);
    return key;
}

// Locality order from the cells' centroids ([n][3]; dim 1, 2 or 3 used): the
// cells sorted by their position on a Hilbert curve through the bounding box
// (one scale for every axis, 2^21 steps along the longest side), ties by cell
// index.  A range of the curve is a compact, mostly connected piece of the
// domain.  On a 100k-triangle square its 608 aggregates need 120 conjugate-
// gradient iterations where recursive bisection's need 167-206 (to a 1e-3
// relative residual), and it cuts a third fewer faces between the blocks.
// Keys are formed on host threads; the sort is a stable radix sort, so the
// order does not depend on the thread count.
inline void hilbert_order(int dim, int n, const double* centroid, std::vector<int>& order) {
    order.resize(n);
    if (n <= 0) return;
    dim = std::max(1, std::min(dim, 3));
    const int b = dim == 1 ? 32 : 21;
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int i = 0; i < dim; ++i) lo[i] = hi[i] = centroid[i];
    for (int c = 0; c < n; ++c)
        for (int i = 0; i < dim; ++i) {
            lo[i] = std::min(lo[i], centroid[3 * (size_t)c + i]);
            hi[i] = std::max(hi[i], centroid[3 * (size_t)c + i]);
        }
    double ext = 0.0;
    for (int i = 0; i < dim; ++i) ext = std::max(ext, hi[i] - lo[i]);
    const double steps = std::ldexp(1.0, b);
    const double scale = ext > 0.0 ? steps / ext : 0.0;
    const double cap = steps - 1.0;
    std::vector<unsigned long long> key(n);
    auto keys = [&](int c0, int c1) {
        for (int c = c0; c < c1; ++c) {
            unsigned x[3] = {0, 0, 0};
            for (int i = 0; i < dim; ++i) {
                const double v = (centroid[3 * (size_t)c + i] - lo[i]) * scale;
                x[i] = (unsigned)std::min(std::max(v, 0.0), cap);
            }
            key[c] = dim == 1 ? (unsigned long long)x[0] : hilbert_key(x, dim, b);
        }
    };
    const int nt = (int)std::max(1u, std::min(8u, std::thread::hardware_concurrency()));
    if (nt > 1 && n >= 65536) {
        std::vector<std::thread> th;
        for (int t = 0; t < nt; ++t)
            th.emplace_back(keys, (int)((long long)n * t / nt), (int)((long long)n * (t + 1) / nt));
        for (auto& t : th) t.join();
    } else {
        keys(0, n);
    }
    // least significant digit first, 16 bits per pass, over the key bits in use
    const int bits = dim * b;
    std::vector<int> tmp(n);
    std::iota(order.begin(), order.end(), 0);
    std::vector<int> cnt(1 << 16);
    for (int sh = 0; sh < bits; sh += 16) {
        std::fill(cnt.begin(), cnt.end(), 0);
        for (int k = 0; k < n; ++k) ++cnt[(key[order[k]] >> sh) & 0xffff];
        int run = 0;
        for (int& v : cnt) {
            const int c = v;
            v = run;
            run += c;
        }
        for (int k = 0; k < n; ++k) tmp[cnt[(key[order[k]] >> sh) & 0xffff]++] = order[k];
        order.swap(tmp);
    }
}

// Aggregates of the permuted cell range [0, n): block k owns [k chunk, (k+1) chunk)
// and its aggregate a the cells with local index in [a seg, (a+1) seg).
struct DsaCoarse {
    int nblk = 0, per_block = 0, chunk = 0, seg = 0, n_agg = 0;
    std::vector<double> ac;    // [n_agg][n_agg] coarse operator (identity rows for empty aggregates); its
                               // inverse is formed on the device (k_gj_step)
    std::vector<int> agg;      // [n] agg_of(c), filled without divisions
    std::vector<int> need_ptr; // [nblk+1] aggregates a block's cells and their neighbours belong to
    std::vector<int> need;
    int agg_of(int c) const { const int k = c / chunk; return k * per_block + (c - k * chunk) / seg; }
};

// Coarse operator A_c = P^T A P of the scaled low-order operator (unit
// diagonal, off-diagonal -w[f][c] to nb[f][c], in the permuted numbering).
// Symmetric positive definite when a wall holds a fixed temperature.
inline void dsa_coarse(int n, int F, const int* nb /* [F][n] */, const double* w /* [F][n] */, int nblk,
                       int per_block, DsaCoarse& out) {
    out.nblk = nblk;
    out.per_block = per_block;
    out.chunk = (n + nblk - 1) / nblk;
    out.seg = (out.chunk + per_block - 1) / per_block;
    const int m = out.n_agg = nblk * per_block;
    std::vector<int>& agg = out.agg;
    agg.assign(n, 0);
    for (int k = 0; k < nblk; ++k)
        for (int a = 0; a < per_block; ++a) {
            const int lo = k * out.chunk + a * out.seg;
            const int hi = std::min(std::min(n, (k + 1) * out.chunk), lo + out.seg);
            for (int c = lo; c < hi; ++c) agg[c] = k * per_block + a;
        }
    // Block k's cells add only to the rows of block k's aggregates, in cell
    // order, so the blocks' rows (and their need lists) are formed on host
    // threads independently; the result does not depend on the thread count.
    std::vector<double>& Ac = out.ac;
    Ac.resize((size_t)m * m);
    std::vector<std::vector<int>> lists(nblk);
    auto rows_of = [&](int k) {
        std::fill(Ac.begin() + (size_t)k * per_block * m, Ac.begin() + (size_t)(k + 1) * per_block * m, 0.0);
        const int lo = std::min(n, k * out.chunk), hi = std::min(n, lo + out.chunk);
        std::vector<int> size(per_block, 0);
        std::vector<char> seen(m, 0);
        std::vector<int>& list = lists[k];
        list.clear();
        for (int c = lo; c < hi; ++c) {
            const int J = agg[c];
            ++size[J - k * per_block];
            Ac[(size_t)J * m + J] += 1.0;
            if (!seen[J]) { seen[J] = 1; list.push_back(J); }
            for (int f = 0; f < F; ++f) {
                const int o = nb[(size_t)f * n + c];
                if (o < 0) continue;
                const int K = agg[o];
                Ac[(size_t)J * m + K] -= w[(size_t)f * n + c];
                if (!seen[K]) { seen[K] = 1; list.push_back(K); }
            }
        }
        for (int a = 0; a < per_block; ++a)
            if (size[a] == 0) Ac[(size_t)(k * per_block + a) * m + k * per_block + a] = 1.0;
        std::sort(list.begin(), list.end());
    };
    const int T = std::max(1, std::min({(int)std::thread::hardware_concurrency(), 8, nblk}));
    if (T == 1 || (size_t)n * F < 65536) {
        for (int k = 0; k < nblk; ++k) rows_of(k);
    } else {
        std::vector<std::thread> pool;
        for (int t = 0; t < T; ++t)
            pool.emplace_back([&, t] {
                for (int k = t; k < nblk; k += T) rows_of(k);
            });
        for (auto& th : pool) th.join();
    }
    out.need_ptr.assign(nblk + 1, 0);
    out.need.clear();
    for (int k = 0; k < nblk; ++k) {
        out.need.insert(out.need.end(), lists[k].begin(), lists[k].end());
        out.need_ptr[k + 1] = (int)out.need.size();
    }
}

}  // namespace bte
