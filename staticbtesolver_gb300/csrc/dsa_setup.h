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

#include <cmath>
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
    for (int c = 0; c < n; ++c)
        for (int f = 0; f < F; ++f) {
            const size_t cf = (size_t)c * F + f;
            const int o = nbr[cf];
            const double A = area[cf];
            if (!(A > 0.0)) continue;
            if (o < 0 || o >= n) {
                if (o < 0 && dirichlet[cf]) {
                    const double w = coefficient(c, f, hfac * volume[c] / A);
                    out.W[(size_t)f * n + c] = w;
                    out.diag[c] += w;
                    ++out.n_dirichlet;
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
            out.diag[c] += w;
            out.diag[o] += w;
        }
}

}  // namespace bte
