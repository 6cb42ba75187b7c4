// Geometry2D / Geometry3D (reference: src/geometry2d.cpp, src/geometry3d.cpp).
#include <cmath>
#include <stdexcept>
#include <string>
#include "eikonalxx/geometry2d.hpp"
#include "eikonalxx/geometry3d.hpp"

using namespace EikonalXX;

namespace
{
// One axis of a node-based grid.
struct Axis
{
    int n{-1};
    double d{-1};
    double origin{0};
    void setN(int v, char name)
    {
        if (v < 3)
            throw std::invalid_argument(std::string("Number of grid points in ") + name + " = " +
                                        std::to_string(v) + " must be at least 3");
        n = v;
    }
    int getN(char name) const
    {
        if (n <= 0) throw std::runtime_error(std::string("Number of grid points in ") + name + " not yet set");
        return n;
    }
    void setD(double v, char name)
    {
        if (!(v > 0))
            throw std::invalid_argument(std::string("Grid spacing in ") + name + " = " + std::to_string(v) +
                                        " must be positive");
        d = v;
    }
    double getD(char name) const
    {
        if (!(d > 0)) throw std::runtime_error(std::string("Grid spacing in ") + name + " not yet set");
        return d;
    }
    bool same(const Axis &o) const
    {
        if ((n > 0) != (o.n > 0) || (d > 0) != (o.d > 0)) return false;
        if (n > 0 && n != o.n) return false;
        if (d > 0 && std::abs(d - o.d) > 1.e-8) return false;
        return std::abs(origin - o.origin) <= 1.e-7;
    }
};
}

#define EIKX_AXIS_METHODS(CLS, A, a)                                                               \
    void CLS::setNumberOfGridPointsIn##A(int v) { pImpl->a.setN(v, #a[0]); }                       \
    int CLS::getNumberOfGridPointsIn##A() const { return pImpl->a.getN(#a[0]); }                   \
    int CLS::getNumberOfCellsIn##A() const { return getNumberOfGridPointsIn##A() - 1; }            \
    bool CLS::haveNumberOfGridPointsIn##A() const noexcept { return pImpl->a.n > 0; }              \
    void CLS::setGridSpacingIn##A(double v) { pImpl->a.setD(v, #a[0]); }                           \
    double CLS::getGridSpacingIn##A() const { return pImpl->a.getD(#a[0]); }                       \
    bool CLS::haveGridSpacingIn##A() const noexcept { return pImpl->a.d > 0; }                     \
    void CLS::setOriginIn##A(double v) noexcept { pImpl->a.origin = v; }                           \
    double CLS::getOriginIn##A() const noexcept { return pImpl->a.origin; }

#define EIKX_VALUE_TYPE(CLS)                                                                       \
    CLS::CLS() : pImpl(std::make_unique<CLS##Impl>()) {}                                           \
    CLS::CLS(const CLS &o) { *this = o; }                                                          \
    CLS::CLS(CLS &&o) noexcept { *this = std::move(o); }                                           \
    CLS &CLS::operator=(const CLS &o)                                                              \
    {                                                                                              \
        if (&o != this) pImpl = std::make_unique<CLS##Impl>(*o.pImpl);                             \
        return *this;                                                                              \
    }                                                                                              \
    CLS &CLS::operator=(CLS &&o) noexcept                                                          \
    {                                                                                              \
        if (&o != this) pImpl = std::move(o.pImpl);                                                \
        return *this;                                                                              \
    }                                                                                              \
    CLS::~CLS() = default;                                                                         \
    void CLS::clear() noexcept { pImpl = std::make_unique<CLS##Impl>(); }

class Geometry2D::Geometry2DImpl
{
public:
    Axis x, z;
};
EIKX_VALUE_TYPE(Geometry2D)
EIKX_AXIS_METHODS(Geometry2D, X, x)
EIKX_AXIS_METHODS(Geometry2D, Z, z)
int Geometry2D::getNumberOfGridPoints() const { return getNumberOfGridPointsInX() * getNumberOfGridPointsInZ(); }
int Geometry2D::getNumberOfCells() const { return getNumberOfCellsInX() * getNumberOfCellsInZ(); }
bool EikonalXX::operator==(const Geometry2D &l, const Geometry2D &r)
{
    auto axis = [](const Geometry2D &g, int k) {
        Axis a;
        a.n = k == 0 ? (g.haveNumberOfGridPointsInX() ? g.getNumberOfGridPointsInX() : -1)
                     : (g.haveNumberOfGridPointsInZ() ? g.getNumberOfGridPointsInZ() : -1);
        a.d = k == 0 ? (g.haveGridSpacingInX() ? g.getGridSpacingInX() : -1)
                     : (g.haveGridSpacingInZ() ? g.getGridSpacingInZ() : -1);
        a.origin = k == 0 ? g.getOriginInX() : g.getOriginInZ();
        return a;
    };
    return axis(l, 0).same(axis(r, 0)) && axis(l, 1).same(axis(r, 1));
}
bool EikonalXX::operator!=(const Geometry2D &l, const Geometry2D &r) { return !(l == r); }

class Geometry3D::Geometry3DImpl
{
public:
    Axis x, y, z;
};
EIKX_VALUE_TYPE(Geometry3D)
EIKX_AXIS_METHODS(Geometry3D, X, x)
EIKX_AXIS_METHODS(Geometry3D, Y, y)
EIKX_AXIS_METHODS(Geometry3D, Z, z)
int Geometry3D::getNumberOfGridPoints() const
{
    return getNumberOfGridPointsInX() * getNumberOfGridPointsInY() * getNumberOfGridPointsInZ();
}
int Geometry3D::getNumberOfCells() const
{
    return getNumberOfCellsInX() * getNumberOfCellsInY() * getNumberOfCellsInZ();
}
bool EikonalXX::operator==(const Geometry3D &l, const Geometry3D &r)
{
    auto axis = [](const Geometry3D &g, int k) {
        Axis a;
        if (k == 0) {
            a.n = g.haveNumberOfGridPointsInX() ? g.getNumberOfGridPointsInX() : -1;
            a.d = g.haveGridSpacingInX() ? g.getGridSpacingInX() : -1;
            a.origin = g.getOriginInX();
        } else if (k == 1) {
            a.n = g.haveNumberOfGridPointsInY() ? g.getNumberOfGridPointsInY() : -1;
            a.d = g.haveGridSpacingInY() ? g.getGridSpacingInY() : -1;
            a.origin = g.getOriginInY();
        } else {
            a.n = g.haveNumberOfGridPointsInZ() ? g.getNumberOfGridPointsInZ() : -1;
            a.d = g.haveGridSpacingInZ() ? g.getGridSpacingInZ() : -1;
            a.origin = g.getOriginInZ();
        }
        return a;
    };
    return axis(l, 0).same(axis(r, 0)) && axis(l, 1).same(axis(r, 1)) && axis(l, 2).same(axis(r, 2));
}
bool EikonalXX::operator!=(const Geometry3D &l, const Geometry3D &r) { return !(l == r); }
