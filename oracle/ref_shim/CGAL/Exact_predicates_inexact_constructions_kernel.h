// Stand-in for the few CGAL geometry types the reference's geometry code uses
// (include/geometry.hpp:114-126, src/geometry.cpp:13-107): points, spheres and
// iso-oriented cuboids with a strict "inside" test.  Test infrastructure only.
#pragma once
#include <algorithm>

namespace CGAL
{
struct Exact_predicates_inexact_constructions_kernel {};
struct Exact_spherical_kernel_3 {};

template <typename K>
struct Point_3
{
    double px{0}, py{0}, pz{0};
    Point_3() = default;
    Point_3(double x, double y, double z) : px(x), py(y), pz(z) {}
    double x() const { return px; }
    double y() const { return py; }
    double z() const { return pz; }
};

// Sphere from a centre and a SQUARED radius; bounded side = strictly inside.
template <typename K>
struct Sphere_3
{
    Point_3<K> c;
    double r2{0};
    Sphere_3() = default;
    Sphere_3(const Point_3<K> &center, double squared_radius) : c(center), r2(squared_radius) {}
    bool has_on_bounded_side(const Point_3<K> &p) const
    {
        double dx = p.x() - c.x(), dy = p.y() - c.y(), dz = p.z() - c.z();
        return dx * dx + dy * dy + dz * dz < r2;
    }
};

// Axis-aligned cuboid given two opposite corners (brought to min/max form);
// bounded side = strictly inside on every axis.
template <typename K>
struct Iso_cuboid_3
{
    double lo[3]{0, 0, 0}, hi[3]{0, 0, 0};
    Iso_cuboid_3() = default;
    Iso_cuboid_3(const Point_3<K> &p, const Point_3<K> &q)
    {
        lo[0] = std::min(p.x(), q.x()); hi[0] = std::max(p.x(), q.x());
        lo[1] = std::min(p.y(), q.y()); hi[1] = std::max(p.y(), q.y());
        lo[2] = std::min(p.z(), q.z()); hi[2] = std::max(p.z(), q.z());
    }
    bool has_on_bounded_side(const Point_3<K> &p) const
    {
        return p.x() > lo[0] && p.x() < hi[0] && p.y() > lo[1] && p.y() < hi[1] && p.z() > lo[2] && p.z() < hi[2];
    }
};

template <typename K>
struct Line_3 {};
} // namespace CGAL
