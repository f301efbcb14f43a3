// utility.cpp -- free functions of the StaticBTESolver API (include/StaticBTESolver/utility.h).
#include "../../include/StaticBTESolver/utility.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace staticbtesolver {

double dot_prod(const Point& a, const Point& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
double dot_prod(const std::shared_ptr<Point>& a, const std::shared_ptr<Point>& b) { return dot_prod(*a, *b); }

Point cross_prod(const Point& a, const Point& b) {
    return Point(a.y * b.z - b.y * a.z, b.x * a.z - a.x * b.z, a.x * b.y - b.x * a.y);
}
std::shared_ptr<Point> cross_prod(const std::shared_ptr<Point>& a, const std::shared_ptr<Point>& b) {
    return std::make_shared<Point>(cross_prod(*a, *b));
}

double getLength(const std::shared_ptr<Point>& a, const std::shared_ptr<Point>& b) { return (*a - *b).length(); }

// Triangle area as half the cross product of two edge vectors.
double getArea(const Point& p1, const Point& p2, const Point& p3) {
    return 0.5 * cross_prod(p3 - p1, p2 - p1).length();
}
double getArea(const std::shared_ptr<Point>& p1, const std::shared_ptr<Point>& p2, const std::shared_ptr<Point>& p3) {
    return 0.5 * cross_prod(*p3 - *p1, *p3 - *p2).length();
}

// Tetrahedron volume as |det[p1-p4, p2-p4, p3-p4]| / 6.
double getVolume(const Point& p1, const Point& p2, const Point& p3, const Point& p4) {
    const Point a = p1 - p4, b = p2 - p4, c = p3 - p4;
    return std::fabs(dot_prod(a, cross_prod(b, c))) / 6.0;
}
double getVolume(const std::shared_ptr<Point>& p1, const std::shared_ptr<Point>& p2,
                 const std::shared_ptr<Point>& p3, const std::shared_ptr<Point>& p4) {
    return getVolume(*p1, *p2, *p3, *p4);
}

// Gauss-Legendre: Newton's method on P_N from the asymptotic initial guesses,
// P_N and P_N' by the three-term recurrence; w = 2 / ((1 - x^2) P_N'(x)^2).
std::vector<double> GaussIntegrationPoints(double a, double b, int N) {
    std::vector<double> out;
    if (N <= 0) return out;
    std::vector<double> x(N), w(N);
    for (int i = 0; i < N; ++i) {
        double z = std::cos(M_PI * (i + 0.75) / (N + 0.5));
        double dp = 0;
        for (int it = 0; it < 100; ++it) {
            double p0 = 1.0, p1 = z;
            for (int k = 2; k <= N; ++k) {
                const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            double pn = N == 1 ? z : p1;
            double pm = N == 1 ? 1.0 : p0;
            dp = N * (z * pn - pm) / (z * z - 1.0);
            const double dz = pn / dp;
            z -= dz;
            if (std::fabs(dz) <= 1e-16) break;
        }
        x[i] = z;
        w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
    // nodes were produced in decreasing order; emit increasing
    for (int i = N - 1; i >= 0; --i) {
        out.push_back(0.5 * (a + b) + 0.5 * (b - a) * x[i]);
        out.push_back(0.5 * (b - a) * w[i]);
    }
    return out;
}

size_t get_host_memory() {
    FILE* f = std::fopen("/proc/self/status", "r");
    if (!f) return (size_t)-1;
    char line[256];
    long kb = -1;
    while (std::fgets(line, sizeof(line), f)) {
        if (std::strncmp(line, "VmRSS:", 6) == 0) {
            kb = std::strtol(line + 6, nullptr, 10);
            break;
        }
    }
    std::fclose(f);
    return (size_t)kb;
}

}  // namespace staticbtesolver
