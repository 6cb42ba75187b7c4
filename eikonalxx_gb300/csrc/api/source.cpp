// Source2D/3D and Station2D/3D (reference: src/source{2,3}d.cpp, src/station{2,3}d.cpp).
// Both are a location inside a grid; a station also carries a name.
#include <algorithm>
#include <stdexcept>
#include <string>
#include "eikonalxx/geometry2d.hpp"
#include "eikonalxx/geometry3d.hpp"
#include "eikonalxx/source2d.hpp"
#include "eikonalxx/source3d.hpp"
#include "eikonalxx/station2d.hpp"
#include "eikonalxx/station3d.hpp"

using namespace EikonalXX;

namespace
{
// A location along one axis of a grid.
struct Coord
{
    double value{0}, offset{0};
    int cell{0};
    bool have{false};
    void set(double v, char name, double x0, double d, int n)
    {
        const double x1 = x0 + static_cast<double>(n - 1) * d;
        if (v < x0 || v > x1)
            throw std::invalid_argument(std::string(1, name) + " = " + std::to_string(v) + " must be in range [" +
                                        std::to_string(x0) + "," + std::to_string(x1) + "]");
        value = v;
        offset = v - x0;
        cell = std::min(n - 2, static_cast<int>(offset / d));
        have = true;
    }
    void need(char name) const
    {
        if (!have) throw std::runtime_error(std::string(1, name) + " location not yet set");
    }
};

template <class G>
void checkGeometry(const G &g, bool threeD)
{
    if (!g.haveGridSpacingInX()) throw std::invalid_argument("Grid spacing in x must be set");
    if (!g.haveGridSpacingInZ()) throw std::invalid_argument("Grid spacing in z must be set");
    if (!g.haveNumberOfGridPointsInX()) throw std::invalid_argument("Number of grid points in x must be set");
    if (!g.haveNumberOfGridPointsInZ()) throw std::invalid_argument("Number of grid points in z must be set");
    (void)threeD;
}
void checkY(const Geometry3D &g)
{
    if (!g.haveGridSpacingInY()) throw std::invalid_argument("Grid spacing in y must be set");
    if (!g.haveNumberOfGridPointsInY()) throw std::invalid_argument("Number of grid points in y must be set");
}
}

#define EIKX_LOC_VALUE_TYPE(CLS)                                                                   \
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
    void CLS::clear() noexcept { pImpl = std::make_unique<CLS##Impl>(); }                         \
    bool CLS::haveGeometry() const noexcept { return pImpl->haveGeometry; }

#define EIKX_LOC_AXIS(CLS, A, a, GEOM)                                                             \
    void CLS::setLocationIn##A(double v)                                                           \
    {                                                                                              \
        if (!haveGeometry()) throw std::runtime_error("Geometry not yet set");                     \
        const auto &g = pImpl->geometry;                                                           \
        pImpl->a.set(v, #a[0], g.getOriginIn##A(), g.getGridSpacingIn##A(), g.getNumberOfGridPointsIn##A()); \
    }                                                                                              \
    double CLS::getLocationIn##A() const { pImpl->a.need(#a[0]); return pImpl->a.value; }          \
    double CLS::getOffsetIn##A() const { pImpl->a.need(#a[0]); return pImpl->a.offset; }          \
    int CLS::getCellIn##A() const { pImpl->a.need(#a[0]); return pImpl->a.cell; }                  \
    bool CLS::haveLocationIn##A() const noexcept { return pImpl->a.have; }

#define EIKX_LOC_2D(CLS)                                                                           \
    class CLS::CLS##Impl                                                                           \
    {                                                                                              \
    public:                                                                                        \
        Geometry2D geometry;                                                                       \
        Coord x, z;                                                                                \
        std::string name;                                                                          \
        bool haveGeometry{false};                                                                  \
    };                                                                                             \
    EIKX_LOC_VALUE_TYPE(CLS)                                                                       \
    EIKX_LOC_AXIS(CLS, X, x, Geometry2D)                                                           \
    EIKX_LOC_AXIS(CLS, Z, z, Geometry2D)                                                           \
    void CLS::setGeometry(const Geometry2D &g)                                                     \
    {                                                                                              \
        checkGeometry(g, false);                                                                   \
        pImpl->geometry = g;                                                                       \
        pImpl->x = Coord{};                                                                        \
        pImpl->z = Coord{};                                                                        \
        pImpl->haveGeometry = true;                                                                \
    }                                                                                              \
    Geometry2D CLS::getGeometry() const                                                            \
    {                                                                                              \
        if (!haveGeometry()) throw std::runtime_error("Geometry not yet set");                     \
        return pImpl->geometry;                                                                    \
    }                                                                                              \
    void CLS::setZToFreeSurface()                                                                  \
    {                                                                                              \
        if (!haveGeometry()) throw std::runtime_error("Geometry not yet set");                     \
        setLocationInZ(pImpl->geometry.getOriginInZ());                                            \
    }                                                                                              \
    int CLS::getCell() const                                                                       \
    {                                                                                              \
        pImpl->x.need('x');                                                                        \
        pImpl->z.need('z');                                                                        \
        return pImpl->z.cell * pImpl->geometry.getNumberOfCellsInX() + pImpl->x.cell;             \
    }

#define EIKX_LOC_3D(CLS)                                                                           \
    class CLS::CLS##Impl                                                                           \
    {                                                                                              \
    public:                                                                                        \
        Geometry3D geometry;                                                                       \
        Coord x, y, z;                                                                             \
        std::string name;                                                                          \
        bool haveGeometry{false};                                                                  \
    };                                                                                             \
    EIKX_LOC_VALUE_TYPE(CLS)                                                                       \
    EIKX_LOC_AXIS(CLS, X, x, Geometry3D)                                                           \
    EIKX_LOC_AXIS(CLS, Y, y, Geometry3D)                                                           \
    EIKX_LOC_AXIS(CLS, Z, z, Geometry3D)                                                           \
    void CLS::setGeometry(const Geometry3D &g)                                                     \
    {                                                                                              \
        checkGeometry(g, true);                                                                    \
        checkY(g);                                                                                 \
        pImpl->geometry = g;                                                                       \
        pImpl->x = Coord{};                                                                        \
        pImpl->y = Coord{};                                                                        \
        pImpl->z = Coord{};                                                                        \
        pImpl->haveGeometry = true;                                                                \
    }                                                                                              \
    Geometry3D CLS::getGeometry() const                                                            \
    {                                                                                              \
        if (!haveGeometry()) throw std::runtime_error("Geometry not yet set");                     \
        return pImpl->geometry;                                                                    \
    }                                                                                              \
    void CLS::setZToFreeSurface()                                                                  \
    {                                                                                              \
        if (!haveGeometry()) throw std::runtime_error("Geometry not yet set");                     \
        setLocationInZ(pImpl->geometry.getOriginInZ());                                            \
    }                                                                                              \
    int CLS::getCell() const                                                                       \
    {                                                                                              \
        pImpl->x.need('x');                                                                        \
        pImpl->y.need('y');                                                                        \
        pImpl->z.need('z');                                                                        \
        const auto &g = pImpl->geometry;                                                           \
        return (pImpl->z.cell * g.getNumberOfCellsInY() + pImpl->y.cell) * g.getNumberOfCellsInX() + \
               pImpl->x.cell;                                                                      \
    }

EIKX_LOC_2D(Source2D)
EIKX_LOC_2D(Station2D)
EIKX_LOC_3D(Source3D)
EIKX_LOC_3D(Station3D)

void Station2D::setName(const std::string &n) noexcept { pImpl->name = n; }
std::string Station2D::getName() const noexcept { return pImpl->name; }
void Station3D::setName(const std::string &n) noexcept { pImpl->name = n; }
std::string Station3D::getName() const noexcept { return pImpl->name; }

namespace
{
template <class L>
std::string describe2(const L &l, const char *what)
{
    if (!(l.haveLocationInX() && l.haveLocationInZ())) return std::string(what) + " location not set";
    return std::string(what) + " location: (x,z) = (" + std::to_string(l.getLocationInX()) + "," +
           std::to_string(l.getLocationInZ()) + ")";
}
template <class L>
std::string describe3(const L &l, const char *what)
{
    if (!(l.haveLocationInX() && l.haveLocationInY() && l.haveLocationInZ()))
        return std::string(what) + " location not set";
    return std::string(what) + " location: (x,y,z) = (" + std::to_string(l.getLocationInX()) + "," +
           std::to_string(l.getLocationInY()) + "," + std::to_string(l.getLocationInZ()) + ")";
}
}
std::ostream &EikonalXX::operator<<(std::ostream &os, const Source2D &s) { return os << describe2(s, "Source"); }
std::ostream &EikonalXX::operator<<(std::ostream &os, const Station2D &s) { return os << describe2(s, "Station"); }
std::ostream &EikonalXX::operator<<(std::ostream &os, const Source3D &s) { return os << describe3(s, "Source"); }
std::ostream &EikonalXX::operator<<(std::ostream &os, const Station3D &s) { return os << describe3(s, "Station"); }
