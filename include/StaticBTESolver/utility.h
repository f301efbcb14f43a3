// utility.h -- geometric primitives and element records of the StaticBTESolver API.
//
// Same names, members and free functions as the reference's
// includes/StaticBTESolver/utility.h (namespace staticbtesolver: Point and its
// operators :24-98, dot_prod/cross_prod/getLength/getArea/getVolume :106-177,
// Segment :189, Triangle :203, Tetrahedron :218, BoundaryCondition :232,
// Band :251, ContinuousArray :270, GaussIntegrationPoints :333,
// get_host_memory :335), so code written against the reference compiles
// unchanged.  The solver itself does not use these types on its hot path.
#ifndef STATICBTESOLVER_GB300_UTILITY_H
#define STATICBTESOLVER_GB300_UTILITY_H

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstddef>
#include <iomanip>
#include <iostream>
#include <memory>
#include <string>
#include <vector>

namespace staticbtesolver {
#ifndef PI
#define PI M_PI
#endif

struct Point {
    double x, y, z;
    explicit Point(double xx = 0, double yy = 0, double zz = 0) : x{xx}, y{yy}, z{zz} {}
    Point(const Point&) = default;
    Point& operator=(const Point&) = default;
    Point operator+(const Point& o) const { return Point(x + o.x, y + o.y, z + o.z); }
    Point operator-(const Point& o) const { return Point(x - o.x, y - o.y, z - o.z); }
    Point operator/(const double k) const { return Point(x / k, y / k, z / k); }
    double operator*(const Point& o) const { return x * o.x + y * o.y + z * o.z; }  // dot product
    double length() const { return std::sqrt(x * x + y * y + z * z); }
    double distance(const Point& p) const { return (*this - p).length(); }
    friend std::ostream& operator<<(std::ostream& os, const Point& p) {
        os << std::fixed << std::setprecision(18) << "(" << p.x << ", " << p.y << " " << p.z << ")";
        return os;
    }
};

double dot_prod(const Point& p1, const Point& p2);
double dot_prod(const std::shared_ptr<Point>& p1, const std::shared_ptr<Point>& p2);
Point cross_prod(const Point& p1, const Point& p2);
std::shared_ptr<Point> cross_prod(const std::shared_ptr<Point>& p1, const std::shared_ptr<Point>& p2);
double getLength(const std::shared_ptr<Point>& p1, const std::shared_ptr<Point>& p2);
double getArea(const Point& p1, const Point& p2, const Point& p3);
double getArea(const std::shared_ptr<Point>& p1, const std::shared_ptr<Point>& p2, const std::shared_ptr<Point>& p3);
double getVolume(const Point& p1, const Point& p2, const Point& p3, const Point& p4);
double getVolume(const std::shared_ptr<Point>& p1, const std::shared_ptr<Point>& p2,
                 const std::shared_ptr<Point>& p3, const std::shared_ptr<Point>& p4);

template <typename A>
using vector2D = std::vector<std::vector<A>>;
template <typename A>
using vector3D = std::vector<vector2D<A>>;
template <typename A>
using vector4D = std::vector<vector3D<A>>;

struct Segment {
    int index[2]{};
    int entity_index;
    explicit Segment(int a = 0, int b = 0, int e = 0) : index{a, b}, entity_index(e) {}
};

struct Triangle {
    int index[3]{};
    int entity_index;
    explicit Triangle(int a = 0, int b = 0, int c = 0, int e = 0) : index{a, b, c}, entity_index(e) {}
};

struct Tetrahedron {
    int index[4]{};
    explicit Tetrahedron(int a = 0, int b = 0, int c = 0, int d = 0) : index{a, b, c, d} {}
};

struct BoundaryCondition {
    int index;  // -(boundary entity) - 1
    int type;   // 1 isothermal, 2 diffuse, 31/32/33 specular
    double temperature;
    explicit BoundaryCondition(int index = 0, int type = 0, int temp = 0)
        : index(index), type(type), temperature(temp) {}
    friend std::ostream& operator<<(std::ostream& os, const BoundaryCondition& bc) {
        os << "Index: " << bc.index << ", Condition: " << bc.type << ", Temperature: " << bc.temperature;
        return os;
    }
};

struct Band {
    double group_velocity;
    double relaxation_time;
    double Ctot;
    double Lr;
    explicit Band(double vg = 0, double rt = 0, double ct = 0, double Lr = 0)
        : group_velocity(vg), relaxation_time(rt), Ctot(ct), Lr(Lr) {}
    friend std::ostream& operator<<(std::ostream& os, const Band& b) {
        os << "Group velocity: " << b.group_velocity << ", relaxation time: " << b.relaxation_time
           << ", Ctot: " << b.Ctot << ", Lr: " << b.Lr;
        return os;
    }
};

// Row-major dim1 x dim2 array of doubles (the reference stores e[b] as N_dir x N_cell).
class ContinuousArray {
public:
    double* data{};
    int dim1{};
    int dim2{};
    ContinuousArray() = default;
    ContinuousArray(int d1, int d2) { init(d1, d2); }
    ContinuousArray(const ContinuousArray& o) : dim1(o.dim1), dim2(o.dim2) {
        data = new double[(size_t)dim1 * dim2];
        std::copy(o.data, o.data + (size_t)dim1 * dim2, data);
    }
    ContinuousArray& operator=(const ContinuousArray& o) {
        if (this != &o) {
            delete[] data;
            dim1 = o.dim1;
            dim2 = o.dim2;
            data = new double[(size_t)dim1 * dim2];
            std::copy(o.data, o.data + (size_t)dim1 * dim2, data);
        }
        return *this;
    }
    void init(int d1, int d2) {
        delete[] data;
        data = new double[(size_t)d1 * d2]();
        dim1 = d1;
        dim2 = d2;
    }
    double* get_ptr(int i, int j) const { return data + ((size_t)i * dim2 + j); }
    double get(int i, int j) const { return *get_ptr(i, j); }
    void clear() const { std::fill_n(data, (size_t)dim1 * dim2, 0.0); }
    void print() const {
        for (int i = 0; i < dim1; ++i) {
            for (int j = 0; j < dim2; ++j) std::cout << get(i, j) << "  ";
            std::cout << std::endl;
        }
    }
    ~ContinuousArray() { delete[] data; }
};

// Gauss-Legendre rule with N points on [a, b], returned interleaved as
// (node_0, weight_0, node_1, weight_1, ...), nodes in increasing order.
std::vector<double> GaussIntegrationPoints(double a, double b, int N);

// Resident set size of this process in kB (VmRSS), or -1.
size_t get_host_memory();
}  // namespace staticbtesolver

#endif
