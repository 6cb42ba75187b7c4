// Ray classes of the C++ API (include/eikonalxx/ray/): points, segments, paths, the step
// rule, and the 2D gradient tracer, whose trace() runs on the GPU through eikx_trace_rays2d.
// Interfaces, messages and exception types follow the reference's src/ray/*.cpp.
#include <algorithm>
#include <cmath>
#include <iostream>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>
#include "eikonalxx/geometry2d.hpp"
#include "eikonalxx/io/vtkLines2d.hpp"
#include "eikonalxx/ray/gradientTracer2d.hpp"
#include "eikonalxx/ray/gradientTracerOptions.hpp"
#include "eikonalxx/ray/path2d.hpp"
#include "eikonalxx/ray/point2d.hpp"
#include "eikonalxx/ray/segment2d.hpp"
#include "eikonalxx/source2d.hpp"
#include "eikonalxx/station2d.hpp"
#include "gpu_context.hpp"

using namespace EikonalXX::Ray;

//------------------------------------------------------------------------- Point2D
class Point2D::Point2DImpl
{
public:
    double x = 0, z = 0;
    bool haveX = false, haveZ = false;
};
Point2D::Point2D() : pImpl(std::make_unique<Point2DImpl>()) {}
Point2D::Point2D(const double x, const double z) : Point2D()
{
    setPositionInX(x);
    setPositionInZ(z);
}
Point2D::Point2D(const Point2D &point) { *this = point; }
Point2D::Point2D(Point2D &&point) noexcept { *this = std::move(point); }
Point2D &Point2D::operator=(const Point2D &point)
{
    if (&point == this) return *this;
    pImpl = std::make_unique<Point2DImpl>(*point.pImpl);
    return *this;
}
Point2D &Point2D::operator=(Point2D &&point) noexcept
{
    if (&point == this) return *this;
    pImpl = std::move(point.pImpl);
    return *this;
}
Point2D::~Point2D() = default;
void Point2D::setPositionInX(const double x) noexcept { pImpl->x = x; pImpl->haveX = true; }
double Point2D::getPositionInX() const
{
    if (!havePositionInX()) throw std::runtime_error("x position not set");
    return pImpl->x;
}
bool Point2D::havePositionInX() const noexcept { return pImpl && pImpl->haveX; }
void Point2D::setPositionInZ(const double z) noexcept { pImpl->z = z; pImpl->haveZ = true; }
double Point2D::getPositionInZ() const
{
    if (!havePositionInZ()) throw std::runtime_error("z position not set");
    return pImpl->z;
}
bool Point2D::havePositionInZ() const noexcept { return pImpl && pImpl->haveZ; }
void Point2D::clear() noexcept { pImpl = std::make_unique<Point2DImpl>(); }

//----------------------------------------------------------------------- Segment2D
class Segment2D::Segment2DImpl
{
public:
    Point2D start, end;
    double length = 0;
    double slowness = 0;   // 0: not set
    int cell = -1;         // -1: not set
    bool havePoints = false;
};
Segment2D::Segment2D() : pImpl(std::make_unique<Segment2DImpl>()) {}
Segment2D::Segment2D(const Segment2D &segment) { *this = segment; }
Segment2D::Segment2D(Segment2D &&segment) noexcept { *this = std::move(segment); }
Segment2D &Segment2D::operator=(const Segment2D &segment)
{
    if (&segment == this) return *this;
    pImpl = std::make_unique<Segment2DImpl>(*segment.pImpl);
    return *this;
}
Segment2D &Segment2D::operator=(Segment2D &&segment) noexcept
{
    if (&segment == this) return *this;
    pImpl = std::move(segment.pImpl);
    return *this;
}
Segment2D::~Segment2D() = default;
void Segment2D::setStartAndEndPoint(const std::pair<Point2D, Point2D> &points)
{
    if (!points.first.havePositionInX()) throw std::invalid_argument("Start x position not set");
    if (!points.first.havePositionInZ()) throw std::invalid_argument("Start z position not set");
    if (!points.second.havePositionInX()) throw std::invalid_argument("End x position not set");
    if (!points.second.havePositionInZ()) throw std::invalid_argument("End z position not set");
    pImpl->start = points.first;
    pImpl->end = points.second;
    pImpl->length = std::hypot(points.second.getPositionInX() - points.first.getPositionInX(),
                               points.second.getPositionInZ() - points.first.getPositionInZ());
    pImpl->havePoints = true;
}
Point2D Segment2D::getStartPoint() const
{
    if (!haveStartAndEndPoint()) throw std::runtime_error("Start point not set");
    return pImpl->start;
}
Point2D Segment2D::getEndPoint() const
{
    if (!haveStartAndEndPoint()) throw std::runtime_error("End point not set");
    return pImpl->end;
}
bool Segment2D::haveStartAndEndPoint() const noexcept { return pImpl && pImpl->havePoints; }
void Segment2D::reverse()
{
    if (!haveStartAndEndPoint()) throw std::runtime_error("Start and end point not set");
    std::swap(pImpl->start, pImpl->end);
}
double Segment2D::getLength() const
{
    if (!haveStartAndEndPoint()) throw std::runtime_error("Start and end point not set");
    return pImpl->length;
}
void Segment2D::setVelocity(const double velocity)
{
    if (velocity <= 0) throw std::runtime_error("Velocity = " + std::to_string(velocity) + " must be positive");
    setSlowness(1. / velocity);
}
void Segment2D::setSlowness(const double slowness)
{
    if (slowness <= 0) throw std::runtime_error("Slowness = " + std::to_string(slowness) + " must be positive");
    pImpl->slowness = slowness;
}
double Segment2D::getVelocity() const
{
    if (!haveVelocity()) throw std::runtime_error("Velocity not set");
    return 1. / getSlowness();
}
double Segment2D::getSlowness() const { return pImpl->slowness; }
bool Segment2D::haveVelocity() const noexcept { return pImpl && pImpl->slowness > 0; }
double Segment2D::getTravelTime() const { return getSlowness() * getLength(); }
void Segment2D::setVelocityModelCellIndex(const int index)
{
    if (index < 0) throw std::invalid_argument("Cell index must be positive");
    pImpl->cell = index;
}
int Segment2D::getVelocityModelCellIndex() const
{
    if (!haveVelocityModelCellIndex()) throw std::runtime_error("Velocity model cell index not set");
    return pImpl->cell;
}
bool Segment2D::haveVelocityModelCellIndex() const noexcept { return pImpl && pImpl->cell >= 0; }
void Segment2D::clear() noexcept { pImpl = std::make_unique<Segment2DImpl>(); }
void EikonalXX::Ray::swap(Segment2D &lhs, Segment2D &rhs) noexcept { std::swap(lhs.pImpl, rhs.pImpl); }
std::ostream &EikonalXX::Ray::operator<<(std::ostream &os, const Segment2D &segment)
{
    if (segment.haveStartAndEndPoint()) {
        const Point2D a = segment.getStartPoint(), b = segment.getEndPoint();
        os << "Start point: (" << a.getPositionInX() << "," << a.getPositionInZ() << ")\n"
           << "End point: (" << b.getPositionInX() << "," << b.getPositionInZ() << ")\n"
           << "Length: " << segment.getLength() << "\n";
    }
    if (segment.haveVelocity()) os << "Velocity: " << segment.getVelocity() << "\n";
    if (segment.haveVelocityModelCellIndex()) os << "Cell index: " << segment.getVelocityModelCellIndex() << "\n";
    return os;
}

//-------------------------------------------------------------------------- Path2D
namespace
{
void checkSegment(const Segment2D &segment)
{
    if (!segment.haveStartAndEndPoint()) throw std::invalid_argument("Segment start/end point not set");
    if (!segment.haveVelocity()) throw std::invalid_argument("Segment velocity not set");
}
double gap(const Point2D &a, const Point2D &b)
{
    return std::hypot(b.getPositionInX() - a.getPositionInX(), b.getPositionInZ() - a.getPositionInZ());
}
constexpr double kJoinTolerance = std::numeric_limits<double>::epsilon() * 100;
}

class Path2D::Path2DImpl
{
public:
    void integrate()
    {
        travelTime = 0;
        length = 0;
        for (const auto &s : segments) {
            travelTime += s.getTravelTime();
            length += s.getLength();
        }
    }
    std::vector<Segment2D> segments, building;
    double travelTime = 0, length = 0;
    bool opened = false;
};
Path2D::Path2D() : pImpl(std::make_unique<Path2DImpl>()) {}
Path2D::Path2D(const Path2D &path) { *this = path; }
Path2D::Path2D(Path2D &&path) noexcept { *this = std::move(path); }
Path2D &Path2D::operator=(const Path2D &path)
{
    if (&path == this) return *this;
    pImpl = std::make_unique<Path2DImpl>(*path.pImpl);
    return *this;
}
Path2D &Path2D::operator=(Path2D &&path) noexcept
{
    if (&path == this) return *this;
    pImpl = std::move(path.pImpl);
    return *this;
}
Path2D::~Path2D() = default;
void Path2D::open()
{
    pImpl->building.clear();
    pImpl->building.reserve(std::max<size_t>(128, pImpl->segments.size()));
    pImpl->opened = true;
}
bool Path2D::isOpen() const noexcept { return pImpl->opened; }
void Path2D::append(const Segment2D &segment)
{
    Segment2D copy = segment;
    append(std::move(copy));
}
void Path2D::append(Segment2D &&segment)
{
    checkSegment(segment);
    if (!pImpl->building.empty() &&
        gap(pImpl->building.back().getEndPoint(), segment.getStartPoint()) > kJoinTolerance)
        throw std::invalid_argument("Segment does not start at last segments's end point");
    pImpl->building.push_back(std::move(segment));
}
void Path2D::close()
{
    if (!isOpen()) throw std::runtime_error("Path not open");
    pImpl->segments = std::move(pImpl->building);
    pImpl->building = std::vector<Segment2D>();
    pImpl->opened = false;
    pImpl->integrate();
}
void Path2D::set(const std::vector<Segment2D> &segments)
{
    std::vector<Segment2D> copy = segments;
    set(std::move(copy));
}
void Path2D::set(std::vector<Segment2D> &&segments)
{
    for (size_t i = 0; i < segments.size(); ++i) {
        checkSegment(segments[i]);
        if (i > 0 && gap(segments[i - 1].getEndPoint(), segments[i].getStartPoint()) > kJoinTolerance)
            throw std::invalid_argument("Segment " + std::to_string(i) + " does no start at last segments " +
                                        std::to_string(i - 1) + " end point");
    }
    pImpl->segments = std::move(segments);
    pImpl->building.clear();
    pImpl->opened = false;
    pImpl->integrate();
}
void Path2D::reverse()
{
    if (isOpen()) throw std::runtime_error("Construction is open");
    std::reverse(pImpl->segments.begin(), pImpl->segments.end());
    for (auto &s : pImpl->segments) s.reverse();
}
bool Path2D::empty() const noexcept { return pImpl->segments.empty(); }
size_t Path2D::size() const noexcept { return pImpl->segments.size(); }
double Path2D::getTravelTime() const { return pImpl->travelTime; }
double Path2D::getLength() const { return pImpl->length; }
double Path2D::getTakeOffAngle() const
{
    if (empty()) throw std::runtime_error("No segments in path");
    for (const auto &s : pImpl->segments)
        if (s.getLength() > 0) {
            const Point2D a = s.getStartPoint(), b = s.getEndPoint();
            return std::atan2(std::abs(b.getPositionInX() - a.getPositionInX()),
                              b.getPositionInZ() - a.getPositionInZ()) * (180 / M_PI);
        }
    std::cerr << "There may exist a zero-length segment at start" << std::endl;
    return 0;
}
void Path2D::clear() noexcept { pImpl = std::make_unique<Path2DImpl>(); }
Path2D::iterator Path2D::begin() { return pImpl->segments.begin(); }
Path2D::const_iterator Path2D::begin() const noexcept { return pImpl->segments.begin(); }
Path2D::const_iterator Path2D::cbegin() const noexcept { return pImpl->segments.cbegin(); }
Path2D::iterator Path2D::end() { return pImpl->segments.end(); }
Path2D::const_iterator Path2D::end() const noexcept { return pImpl->segments.cend(); }
Path2D::const_iterator Path2D::cend() const noexcept { return pImpl->segments.cend(); }
Segment2D &Path2D::at(const size_t index) { return pImpl->segments.at(index); }
const Segment2D &Path2D::at(const size_t index) const { return pImpl->segments.at(index); }

//----------------------------------------------------------- GradientTracerOptions
class GradientTracerOptions::GradientTracerOptionsImpl
{
public:
    std::vector<std::pair<int, double>> rsf{
        {1, 0.05}, {2, 0.10}, {3, 0.20}, {5, 0.30}, {std::numeric_limits<int>::max(), 0.45}};
};
GradientTracerOptions::GradientTracerOptions() : pImpl(std::make_unique<GradientTracerOptionsImpl>()) {}
GradientTracerOptions::GradientTracerOptions(const GradientTracerOptions &options) { *this = options; }
GradientTracerOptions::GradientTracerOptions(GradientTracerOptions &&options) noexcept { *this = std::move(options); }
GradientTracerOptions &GradientTracerOptions::operator=(const GradientTracerOptions &options)
{
    if (&options == this) return *this;
    pImpl = std::make_unique<GradientTracerOptionsImpl>(*options.pImpl);
    return *this;
}
GradientTracerOptions &GradientTracerOptions::operator=(GradientTracerOptions &&options) noexcept
{
    if (&options == this) return *this;
    pImpl = std::move(options.pImpl);
    return *this;
}
GradientTracerOptions::~GradientTracerOptions() = default;
void GradientTracerOptions::setRadiusScaleFactor(const std::vector<std::pair<int, double>> &rsf)
{
    if (rsf.empty()) throw std::invalid_argument("Input vector cannot be empty");
    for (const auto &item : rsf) {
        if (item.first < 0) throw std::invalid_argument("All radii must be non-negative");
        if (item.second <= std::numeric_limits<double>::epsilon())
            throw std::invalid_argument("All scale factors must be non-negative");
        if (item.second >= 1) throw std::invalid_argument("All scale factors must be less than 1");
    }
    auto sorted = rsf;
    std::stable_sort(sorted.begin(), sorted.end(), [](const auto &a, const auto &b) { return a.first < b.first; });
    for (size_t i = 0; i + 1 < sorted.size(); ++i)
        if (sorted[i].first == sorted[i + 1].first) throw std::invalid_argument("Duplicate radii");
    if (sorted.back().first < std::numeric_limits<int>::max())
        sorted.emplace_back(std::numeric_limits<int>::max(), sorted.back().second);
    pImpl->rsf = std::move(sorted);
}
std::vector<std::pair<int, double>> GradientTracerOptions::getRadiusScaleFactor() const noexcept { return pImpl->rsf; }
void GradientTracerOptions::clear() noexcept { pImpl = std::make_unique<GradientTracerOptionsImpl>(); }

//-------------------------------------------------------------- GradientTracer2D
namespace
{
// Geometry2D equality as the reference's geometryMatches (gradientTracer2d.cpp): sizes,
// spacing to millimetres, origin to centimetres.
bool geometryMatches(const EikonalXX::Geometry2D &a, const EikonalXX::Geometry2D &b)
{
    return a.getNumberOfGridPointsInX() == b.getNumberOfGridPointsInX() &&
           a.getNumberOfGridPointsInZ() == b.getNumberOfGridPointsInZ() &&
           std::abs(a.getGridSpacingInX() - b.getGridSpacingInX()) <= 1.e-3 &&
           std::abs(a.getGridSpacingInZ() - b.getGridSpacingInZ()) <= 1.e-3 &&
           std::abs(a.getOriginInX() - b.getOriginInX()) <= 1.e-2 &&
           std::abs(a.getOriginInZ() - b.getOriginInZ()) <= 1.e-2;
}
}

class GradientTracer2D::GradientTracer2DImpl
{
public:
    GradientTracer2DImpl() = default;
    GradientTracer2DImpl(const GradientTracer2DImpl &o)
        : geometry(o.geometry), options(o.options), stations(o.stations), paths(o.paths),
          initialized(o.initialized), haveRayPaths(o.haveRayPaths)
    {
    }
    EikonalXX::Geometry2D geometry;
    GradientTracerOptions options;
    std::vector<EikonalXX::Station2D> stations;
    std::vector<Path2D> paths;
    bool initialized = false, haveRayPaths = false;
    EikonalXX::Detail::GpuContext gpu;   // not copied: each tracer owns its context
};
GradientTracer2D::GradientTracer2D() : pImpl(std::make_unique<GradientTracer2DImpl>()) {}
GradientTracer2D::GradientTracer2D(const GradientTracer2D &tracer) { *this = tracer; }
GradientTracer2D::GradientTracer2D(GradientTracer2D &&tracer) noexcept { *this = std::move(tracer); }
GradientTracer2D &GradientTracer2D::operator=(const GradientTracer2D &tracer)
{
    if (&tracer == this) return *this;
    pImpl = std::make_unique<GradientTracer2DImpl>(*tracer.pImpl);
    return *this;
}
GradientTracer2D &GradientTracer2D::operator=(GradientTracer2D &&tracer) noexcept
{
    if (&tracer == this) return *this;
    pImpl = std::move(tracer.pImpl);
    return *this;
}
GradientTracer2D::~GradientTracer2D() = default;

void GradientTracer2D::initialize(const GradientTracerOptions &options, const EikonalXX::Geometry2D &geometry)
{
    if (!geometry.haveGridSpacingInX()) throw std::invalid_argument("x grid spacing not set");
    if (!geometry.haveGridSpacingInZ()) throw std::invalid_argument("z grid spacing not set");
    if (!geometry.haveNumberOfGridPointsInX()) throw std::invalid_argument("Grid points in x not set");
    if (!geometry.haveNumberOfGridPointsInZ()) throw std::invalid_argument("Grid points in z not set");
    pImpl->options = options;
    pImpl->geometry = geometry;
    pImpl->initialized = true;
    pImpl->paths.clear();
    pImpl->haveRayPaths = false;
}
bool GradientTracer2D::isInitialized() const noexcept { return pImpl->initialized; }

void GradientTracer2D::setStations(const std::vector<EikonalXX::Station2D> &stations)
{
    if (!isInitialized()) throw std::invalid_argument("Class not initialized");
    for (const auto &station : stations) {
        if (!station.haveGeometry()) throw std::invalid_argument("Station geometry not set");
        if (!station.haveLocationInX()) throw std::invalid_argument("Station x position not set");
        if (!station.haveLocationInZ()) throw std::invalid_argument("Station z position not set");
        if (!geometryMatches(pImpl->geometry, station.getGeometry()))
            throw std::invalid_argument("Inconsistent geometry");
    }
    pImpl->stations = stations;
    pImpl->paths.clear();
    pImpl->haveRayPaths = false;
}
bool GradientTracer2D::haveStations() const noexcept { return !pImpl->stations.empty(); }

template <typename T> void GradientTracer2D::trace(const EikonalXX::AbstractBaseClass::ISolver2D<T> &solver)
{
    if (!isInitialized()) throw std::runtime_error("Class not initialized");
    if (!solver.haveVelocityModel()) throw std::invalid_argument("Velocity model not set on solver");
    if (!solver.haveSource()) throw std::invalid_argument("Source not on solver");
    if (!solver.haveTravelTimeGradientField()) throw std::invalid_argument("Travel time gradient field not set");
    if (!haveStations()) throw std::runtime_error("No stations were set");
    pImpl->haveRayPaths = false;
    pImpl->paths.assign(pImpl->stations.size(), Path2D());
    const auto &geo = pImpl->geometry;
    const int nx = geo.getNumberOfGridPointsInX(), nz = geo.getNumberOfGridPointsInZ();
    const double dx = geo.getGridSpacingInX(), dz = geo.getGridSpacingInZ();
    const double x0 = geo.getOriginInX(), z0 = geo.getOriginInZ();
    // the cell slowness as the solver reports it (ISolver2D::getSlowness), natural order
    std::vector<double> slow(static_cast<size_t>(nx - 1) * (nz - 1));
    for (int iz = 0; iz < nz - 1; ++iz)
        for (int ix = 0; ix < nx - 1; ++ix)
            slow[static_cast<size_t>(iz) * (nx - 1) + ix] = static_cast<double>(solver.getSlowness(ix, iz));
    const auto source = solver.getSource();
    std::vector<double> st(2 * pImpl->stations.size());
    for (size_t i = 0; i < pImpl->stations.size(); ++i) {
        st[2 * i] = pImpl->stations[i].getLocationInX();
        st[2 * i + 1] = pImpl->stations[i].getLocationInZ();
    }
    eikx_ray_options opt;
    eikx_ray_options_default(&opt);
    const auto rsf = pImpl->options.getRadiusScaleFactor();
    if (rsf.size() > 16) throw std::invalid_argument("at most 16 radius / scale pairs");
    opt.n_radii = static_cast<int>(rsf.size());
    for (size_t k = 0; k < rsf.size(); ++k) {
        opt.radius[k] = rsf[k].first;
        opt.scale[k] = rsf[k].second;
    }
    const int capacity = 4 * (nx + nz) + 16;
    const int n = static_cast<int>(pImpl->stations.size());
    std::vector<eikx_ray_segment2d> seg(static_cast<size_t>(n) * capacity);
    std::vector<int> counts(n);
    Detail::check(eikx_trace_rays2d(pImpl->gpu.get(), nx, nz, dx, dz, x0, z0, solver.getTravelTimeGradientFieldPointer(),
                                    sizeof(T) == 8 ? EIKX_F64 : EIKX_F32, slow.data(), source.getLocationInX(),
                                    source.getLocationInZ(), st.data(), n, &opt, capacity, seg.data(), counts.data()));
    for (int i = 0; i < n; ++i) {
        if (counts[i] <= 0) {
            const std::string name = pImpl->stations[i].getName();
            std::cerr << "Ray for station: " << (name.empty() ? std::to_string(i) : name)
                      << " did not converge to source" << std::endl;
            continue;
        }
        Path2D path;
        path.open();
        for (int k = 0; k < counts[i]; ++k) {
            const eikx_ray_segment2d &s = seg[static_cast<size_t>(i) * capacity + k];
            Segment2D segment;
            segment.setStartAndEndPoint(std::pair{Point2D{s.x0, s.z0}, Point2D{s.x1, s.z1}});
            segment.setSlowness(s.slowness);
            if (s.cell >= 0) segment.setVelocityModelCellIndex(s.cell);
            path.append(std::move(segment));
        }
        path.close();
        pImpl->paths[i] = std::move(path);
    }
    pImpl->haveRayPaths = true;
}
bool GradientTracer2D::haveRayPaths() const noexcept { return pImpl->haveRayPaths; }
std::vector<Path2D> GradientTracer2D::getRayPaths() const
{
    if (!haveRayPaths()) throw std::runtime_error("Ray paths not computed");
    return pImpl->paths;
}
// src/ray/gradientTracer2d.cpp:617-655: each path as a polyline through its segments'
// start points and the last segment's end point.
void GradientTracer2D::writeVTK(const std::string &fileName, const std::string &title)
{
    if (!haveRayPaths()) throw std::runtime_error("Ray paths not computed");
    IO::VTKLines2D vtk;
    vtk.open(fileName, pImpl->geometry, title);
    if (!pImpl->paths.empty()) {
        std::vector<std::vector<std::pair<double, double>>> lines;
        lines.reserve(pImpl->paths.size());
        for (const auto &path : pImpl->paths) {
            std::vector<std::pair<double, double>> line;
            const size_t n = path.size();
            line.reserve(n + 1);
            for (size_t i = 0; i < n; ++i) {
                const auto &seg = path.at(i);
                line.emplace_back(seg.getStartPoint().getPositionInX(), seg.getStartPoint().getPositionInZ());
                if (i == n - 1) line.emplace_back(seg.getEndPoint().getPositionInX(), seg.getEndPoint().getPositionInZ());
            }
            lines.push_back(std::move(line));
        }
        vtk.write(lines);
    }
    vtk.close();
}

template void GradientTracer2D::trace(const EikonalXX::AbstractBaseClass::ISolver2D<double> &);
template void GradientTracer2D::trace(const EikonalXX::AbstractBaseClass::ISolver2D<float> &);
