// oracle/krylov.h -- TEST INFRASTRUCTURE ONLY (the oracle).
//
// CPU restatements of the two inner linear solvers the reference uses for one
// (band, direction) upwind system A x = b:
//
//  * gmres_ilu0(): restarted GMRES(30) with left ILU(0) preconditioning, x0 = 0,
//    stop when the preconditioned residual norm drops below rtol * its initial
//    value (or below abstol), at most maxit iterations.  These are PETSc's
//    default KSP/PC settings for a sequential AIJ matrix, which is what
//    src/StaticBTESolver.cpp:291-300 ends up running (KSPSetType/PCSetType are
//    commented out at :294-297; KSPSetTolerances(1e-9, default, default, 1000)
//    at :298).  PETSc itself is not available; the algorithm is restated from
//    Saad, "Iterative Methods for Sparse Linear Systems", Alg. 6.11 (GMRES)
//    and Alg. 10.4 (ILU(0)).  Inner-iterate parity with PETSc is not claimed;
//    only the converged solution (to rtol) matters to the outer iteration.
//
//  * bicgstab_jacobi(): the reference GPU inner solver, src/bicgstab.hpp:138-300:
//    right-Jacobi BiCGSTAB, x0 = 0, p = r initially with beta = rho on the first
//    step, breakdown restart with r_hat = 6.8 b + 0.6 when |rho| or |r_hat.q|
//    is below 1e-200, stop on ||r|| / ||r0|| < tol, at most maxit iterations.
//
// Nothing in the product links this file.
#pragma once
#include <cmath>
#include <vector>
#include <cstddef>

namespace oracle {

struct Csr {
    int n = 0;
    std::vector<int> rowptr, col;
    std::vector<double> val;
};

// ILU(0) factors stored in the pattern of A (unit-lower L below the diagonal,
// U on and above it).  Requires sorted column indices and a stored diagonal,
// which the reference's _get_Ke guarantees (std::sort at
// src/StaticBTESolver.cpp:151, diagonal always emitted at :149).
struct Ilu0 {
    const Csr* a = nullptr;
    std::vector<double> lu;
    std::vector<int> diag;
    bool ok = true;

    void factor(const Csr& A) {
        a = &A;
        lu = A.val;
        diag.assign(A.n, -1);
        for (int i = 0; i < A.n; ++i)
            for (int k = A.rowptr[i]; k < A.rowptr[i + 1]; ++k)
                if (A.col[k] == i) diag[i] = k;
        std::vector<int> pos(A.n, -1);
        for (int i = 0; i < A.n; ++i) {
            if (diag[i] < 0) { ok = false; return; }
            for (int k = A.rowptr[i]; k < A.rowptr[i + 1]; ++k) pos[A.col[k]] = k;
            for (int k = A.rowptr[i]; k < A.rowptr[i + 1]; ++k) {
                int j = A.col[k];
                if (j >= i) break;
                double piv = lu[diag[j]];
                lu[k] /= piv;
                double lij = lu[k];
                for (int m = diag[j] + 1; m < A.rowptr[j + 1]; ++m) {
                    int p = pos[A.col[m]];
                    if (p >= 0) lu[p] -= lij * lu[m];
                }
            }
            for (int k = A.rowptr[i]; k < A.rowptr[i + 1]; ++k) pos[A.col[k]] = -1;
        }
    }

    // y = (LU)^{-1} x
    void apply(const double* x, double* y) const {
        const Csr& A = *a;
        for (int i = 0; i < A.n; ++i) {
            double s = x[i];
            for (int k = A.rowptr[i]; k < diag[i]; ++k) s -= lu[k] * y[A.col[k]];
            y[i] = s;
        }
        for (int i = A.n - 1; i >= 0; --i) {
            double s = y[i];
            for (int k = diag[i] + 1; k < A.rowptr[i + 1]; ++k) s -= lu[k] * y[A.col[k]];
            y[i] = s / lu[diag[i]];
        }
    }
};

inline void spmv(const Csr& A, const double* x, double* y) {
    for (int i = 0; i < A.n; ++i) {
        double s = 0;
        for (int k = A.rowptr[i]; k < A.rowptr[i + 1]; ++k) s += A.val[k] * x[A.col[k]];
        y[i] = s;
    }
}

inline double dot(int n, const double* a, const double* b) {
    double s = 0;
    for (int i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

struct KrylovResult {
    int iterations = 0;
    int converged = 0;
    double final_norm = 0;
};

// Left-preconditioned restarted GMRES(m) with ILU(0), x0 = 0.
inline KrylovResult gmres_ilu0(const Csr& A, const double* b, double* x, double rtol,
                               double abstol = 1e-50, double dtol = 1e5, int maxit = 1000,
                               int restart = 30) {
    KrylovResult res;
    const int n = A.n;
    Ilu0 M;
    M.factor(A);
    std::vector<double> w(n), r(n), tmp(n);
    std::vector<std::vector<double>> V(restart + 1, std::vector<double>(n));
    std::vector<double> H((restart + 1) * restart), cs(restart), sn(restart), g(restart + 1);
    for (int i = 0; i < n; ++i) x[i] = 0.0;
    // initial preconditioned residual: M^{-1} b
    M.apply(b, r.data());
    double rnorm0 = std::sqrt(dot(n, r.data(), r.data()));
    double rnorm = rnorm0;
    res.final_norm = rnorm;
    if (rnorm0 <= abstol) { res.converged = 1; return res; }
    const double target = std::fmax(rtol * rnorm0, abstol);
    int it = 0;
    while (it < maxit) {
        // r = M^{-1}(b - A x)
        spmv(A, x, tmp.data());
        for (int i = 0; i < n; ++i) tmp[i] = b[i] - tmp[i];
        M.apply(tmp.data(), r.data());
        double beta = std::sqrt(dot(n, r.data(), r.data()));
        if (beta <= target) { res.converged = 1; rnorm = beta; break; }
        for (int i = 0; i < n; ++i) V[0][i] = r[i] / beta;
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        int k = 0;
        bool done = false;
        for (; k < restart && it < maxit; ++k) {
            ++it;
            spmv(A, V[k].data(), tmp.data());
            M.apply(tmp.data(), w.data());
            for (int j = 0; j <= k; ++j) {  // modified Gram-Schmidt
                double h = dot(n, w.data(), V[j].data());
                H[j * restart + k] = h;
                for (int i = 0; i < n; ++i) w[i] -= h * V[j][i];
            }
            double hn = std::sqrt(dot(n, w.data(), w.data()));
            H[(k + 1) * restart + k] = hn;
            if (hn != 0.0)
                for (int i = 0; i < n; ++i) V[k + 1][i] = w[i] / hn;
            for (int j = 0; j < k; ++j) {  // apply previous Givens rotations
                double a0 = H[j * restart + k], a1 = H[(j + 1) * restart + k];
                H[j * restart + k] = cs[j] * a0 + sn[j] * a1;
                H[(j + 1) * restart + k] = -sn[j] * a0 + cs[j] * a1;
            }
            double a0 = H[k * restart + k], a1 = H[(k + 1) * restart + k];
            double d = std::hypot(a0, a1);
            cs[k] = d == 0.0 ? 1.0 : a0 / d;
            sn[k] = d == 0.0 ? 0.0 : a1 / d;
            H[k * restart + k] = d;
            H[(k + 1) * restart + k] = 0.0;
            g[k + 1] = -sn[k] * g[k];
            g[k] = cs[k] * g[k];
            rnorm = std::fabs(g[k + 1]);
            if (rnorm <= target || hn == 0.0) { done = true; ++k; break; }
            if (rnorm > dtol * rnorm0) { done = true; ++k; break; }
        }
        // solve the k x k upper-triangular system and update x
        std::vector<double> yv(k);
        for (int i = k - 1; i >= 0; --i) {
            double s = g[i];
            for (int j = i + 1; j < k; ++j) s -= H[i * restart + j] * yv[j];
            yv[i] = s / H[i * restart + i];
        }
        for (int j = 0; j < k; ++j)
            for (int i = 0; i < n; ++i) x[i] += yv[j] * V[j][i];
        if (done) { res.converged = rnorm <= target; break; }
    }
    res.iterations = it;
    res.final_norm = rnorm;
    return res;
}

// Right-Jacobi BiCGSTAB exactly as src/bicgstab.hpp:138-300 sequences it.
inline KrylovResult bicgstab_jacobi(const Csr& A, const double* b, double* x, double tol,
                                    int maxit = 1000) {
    KrylovResult res;
    const int n = A.n;
    std::vector<double> jac(n, 0.0);  // src/bicgstab.hpp:122-131
    for (int row = 0; row < n; ++row)
        for (int j = A.rowptr[row]; j < A.rowptr[row + 1]; ++j)
            if (A.col[j] == row) jac[row] = 1.0 / A.val[j];
    std::vector<double> r(b, b + n), p(b, b + n), rw(b, b + n), q(n, 0.0), ph(n), z(n), t(n);
    for (int i = 0; i < n; ++i) x[i] = 0.0;
    double nrmr0 = std::sqrt(dot(n, r.data(), r.data()));
    double nrmr = nrmr0;
    double rhop = 1, rho = 1, omega = 1, alpha = 1;
    auto restart_state = [&]() {  // src/bicgstab.hpp:170-179 and :224-234
        rho = 1; alpha = 1; omega = 1;
        for (int i = 0; i < n; ++i) {
            x[i] = 0; q[i] = 0; p[i] = 0; r[i] = b[i];
            rw[i] = b[i] * 6.8 + 0.6;
        }
    };
    int i = 1;
    for (; i <= maxit; ++i) {
        if (nrmr < 1e-50) break;
        rhop = rho;
        rho = dot(n, rw.data(), r.data());
        if (rho < 1e-200 && rho > -1e-200) { restart_state(); continue; }
        double beta = (rho / rhop) * (alpha / omega);
        for (int k = 0; k < n; ++k) p[k] = r[k] + beta * (p[k] - omega * q[k]);
        for (int k = 0; k < n; ++k) ph[k] = jac[k] * p[k];
        spmv(A, ph.data(), q.data());
        double temp = dot(n, rw.data(), q.data());
        if (temp < 1e-200 && temp > -1e-200) { restart_state(); continue; }
        alpha = rho / temp;
        for (int k = 0; k < n; ++k) r[k] -= alpha * q[k];
        for (int k = 0; k < n; ++k) z[k] = jac[k] * r[k];
        spmv(A, z.data(), t.data());
        double ts = dot(n, t.data(), r.data());
        double tt = dot(n, t.data(), t.data());
        omega = tt > 0.0 ? ts / tt : 0.0;  // s == 0: the reference would form 0/0 here
        for (int k = 0; k < n; ++k) x[k] += alpha * ph[k];  // two axpys, :283 and :285
        for (int k = 0; k < n; ++k) x[k] += omega * z[k];
        for (int k = 0; k < n; ++k) r[k] -= omega * t[k];
        nrmr = std::sqrt(dot(n, r.data(), r.data()));
        if (nrmr / nrmr0 < tol) { res.converged = 1; break; }
    }
    res.iterations = i > maxit ? maxit : i;
    res.final_norm = nrmr;
    return res;
}

}  // namespace oracle
