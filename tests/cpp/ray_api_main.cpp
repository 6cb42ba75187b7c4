// Drives the C++ ray API (include/eikonalxx/ray/) as a user of the reference would.
// Usage: ray_api cpu   -- points, segments, paths and the step rule (no GPU);
//        ray_api gpu   -- the gradient tracer on the GPU: straight rays through an analytic
//                         homogeneous gradient (the reference's own case, testing/ray.cpp),
//                         and rays through the gradient of a GPU 2D solve.
// Prints "ray_api ok" and exits 0 when every check holds.
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>
#include "eikonalxx/geometry2d.hpp"
#include "eikonalxx/model2d.hpp"
#include "eikonalxx/ray/gradientTracer2d.hpp"
#include "eikonalxx/ray/gradientTracerOptions.hpp"
#include "eikonalxx/ray/path2d.hpp"
#include "eikonalxx/ray/point2d.hpp"
#include "eikonalxx/ray/segment2d.hpp"
#include "eikonalxx/solver2d.hpp"
#include "eikonalxx/solverOptions.hpp"
#include "eikonalxx/source2d.hpp"
#include "eikonalxx/station2d.hpp"

using namespace EikonalXX;
using namespace EikonalXX::Ray;

static int failures = 0;
#define CHECK(cond)                                                                       \
    do {                                                                                  \
        if (!(cond)) {                                                                    \
            std::cerr << __FILE__ << ":" << __LINE__ << " check failed: " #cond << "\n"; \
            ++failures;                                                                   \
        }                                                                                 \
    } while (0)
template <class E, class F> bool throws(F f)
{
    try {
        f();
    } catch (const E &) {
        return true;
    } catch (...) {
        return false;
    }
    return false;
}

static void cpuChecks()
{
    Point2D p;
    CHECK(!p.havePositionInX() && throws<std::runtime_error>([&] { (void)p.getPositionInX(); }));
    p.setPositionInX(3);
    p.setPositionInZ(4);
    CHECK(p.getPositionInX() == 3 && p.getPositionInZ() == 4);
    Point2D q = p;
    p.clear();
    CHECK(!p.havePositionInZ() && q.getPositionInZ() == 4);

    Segment2D s;
    CHECK(throws<std::invalid_argument>([&] { s.setStartAndEndPoint({Point2D{}, Point2D{1, 2}}); }));
    s.setStartAndEndPoint({Point2D{0, 0}, Point2D{3, 4}});
    CHECK(std::abs(s.getLength() - 5) < 1e-14);
    CHECK(!s.haveVelocity() && throws<std::runtime_error>([&] { (void)s.getVelocity(); }));
    CHECK(throws<std::runtime_error>([&] { s.setVelocity(-1); }));
    s.setVelocity(2000);
    CHECK(std::abs(s.getSlowness() - 1. / 2000) < 1e-18 && std::abs(s.getTravelTime() - 5. / 2000) < 1e-15);
    CHECK(!s.haveVelocityModelCellIndex() && throws<std::invalid_argument>([&] { s.setVelocityModelCellIndex(-2); }));
    s.setVelocityModelCellIndex(7);
    CHECK(s.getVelocityModelCellIndex() == 7);
    s.reverse();
    CHECK(s.getStartPoint().getPositionInX() == 3 && s.getEndPoint().getPositionInZ() == 0);

    // a path of three joined segments, with one that does not join
    Path2D path;
    path.open();
    CHECK(path.isOpen());
    const double xs[4] = {0, 1, 1, 3}, zs[4] = {0, 0, 2, 2}, v[3] = {1000, 2000, 4000};
    double tExp = 0, lExp = 0;
    for (int i = 0; i < 3; ++i) {
        Segment2D seg;
        seg.setStartAndEndPoint({Point2D{xs[i], zs[i]}, Point2D{xs[i + 1], zs[i + 1]}});
        seg.setVelocity(v[i]);
        lExp += seg.getLength();
        tExp += seg.getTravelTime();
        path.append(seg);
    }
    Segment2D bad;
    bad.setStartAndEndPoint({Point2D{9, 9}, Point2D{10, 10}});
    bad.setVelocity(1000);
    CHECK(throws<std::invalid_argument>([&] { path.append(bad); }));
    Segment2D noVelocity;
    noVelocity.setStartAndEndPoint({Point2D{3, 2}, Point2D{4, 2}});
    CHECK(throws<std::invalid_argument>([&] { path.append(noVelocity); }));
    path.close();
    CHECK(!path.isOpen() && path.size() == 3);
    CHECK(std::abs(path.getLength() - lExp) < 1e-14 && std::abs(path.getTravelTime() - tExp) < 1e-15);
    CHECK(std::abs(path.getTakeOffAngle() - 90) < 1e-12);   // first segment along +x
    path.reverse();
    CHECK(path.at(0).getStartPoint().getPositionInX() == 3 && std::abs(path.getTakeOffAngle() - 90) < 1e-12);
    double l = 0;
    for (const auto &seg : path) l += seg.getLength();
    CHECK(std::abs(l - lExp) < 1e-14);
    CHECK(throws<std::runtime_error>([&] { Path2D().close(); }));
    CHECK(throws<std::runtime_error>([&] { (void)Path2D().getTakeOffAngle(); }));

    GradientTracerOptions options;
    auto rsf = options.getRadiusScaleFactor();
    CHECK(rsf.size() == 5 && rsf.front().first == 1 && rsf.front().second == 0.05 &&
          rsf.back().first == std::numeric_limits<int>::max() && rsf.back().second == 0.45);
    options.setRadiusScaleFactor({{10, 0.3}, {0, 0.1}});
    rsf = options.getRadiusScaleFactor();
    CHECK(rsf.size() == 3 && rsf[0].first == 0 && rsf[1].first == 10 &&
          rsf[2].first == std::numeric_limits<int>::max() && rsf[2].second == 0.3);
    CHECK(throws<std::invalid_argument>([&] { options.setRadiusScaleFactor({}); }));
    CHECK(throws<std::invalid_argument>([&] { options.setRadiusScaleFactor({{-1, 0.1}}); }));
    CHECK(throws<std::invalid_argument>([&] { options.setRadiusScaleFactor({{1, 1.0}}); }));
    CHECK(throws<std::invalid_argument>([&] { options.setRadiusScaleFactor({{1, 0.1}, {1, 0.2}}); }));
    GradientTracerOptions copy(options);
    options.clear();
    CHECK(copy.getRadiusScaleFactor().size() == 3 && options.getRadiusScaleFactor().size() == 5);

    GradientTracer2D tracer;
    CHECK(!tracer.isInitialized() && throws<std::invalid_argument>([&] { tracer.setStations({}); }));
    CHECK(throws<std::runtime_error>([&] { (void)tracer.getRayPaths(); }));
}

// A homogeneous medium with its analytic travel times and gradient, as the reference's
// Analytic::Homogeneous2D provides them to its tracer test.
class Homogeneous : public AbstractBaseClass::ISolver2D<double>
{
public:
    Homogeneous(const Geometry2D &g, const Source2D &s, double v) : g_(g), s_(s), v_(v)
    {
        const int nx = g.getNumberOfGridPointsInX(), nz = g.getNumberOfGridPointsInZ();
        t_.resize(static_cast<size_t>(nx) * nz);
        grad_.resize(2 * t_.size());
        for (int iz = 0; iz < nz; ++iz)
            for (int ix = 0; ix < nx; ++ix) {
                const double x = ix * g.getGridSpacingInX() - s.getOffsetInX();
                const double z = iz * g.getGridSpacingInZ() - s.getOffsetInZ();
                const double r = std::hypot(x, z);
                const size_t i = static_cast<size_t>(iz) * nx + ix;
                t_[i] = r / v;
                grad_[2 * i] = r > 0 ? x / r / v : 0;
                grad_[2 * i + 1] = r > 0 ? z / r / v : 0;
            }
    }
    bool haveVelocityModel() const noexcept override { return true; }
    std::vector<double> getTravelTimeField() const override { return t_; }
    const double *getTravelTimeFieldPointer() const override { return t_.data(); }
    std::vector<double> getTravelTimeGradientField() const override { return grad_; }
    const double *getTravelTimeGradientFieldPointer() const override { return grad_.data(); }
    bool haveTravelTimeField() const noexcept override { return true; }
    bool haveTravelTimeGradientField() const noexcept override { return true; }
    Source2D getSource() const override { return s_; }
    bool haveSource() const noexcept override { return true; }
    double getSlowness(int, int) const override { return 1 / v_; }
private:
    Geometry2D g_;
    Source2D s_;
    double v_;
    std::vector<double> t_, grad_;
};

static void gpuChecks()
{
    const double v = 4000, dx = 100, dz = 101, x0 = 1, z0 = 2;
    const int nx = 201, nz = 101;
    Geometry2D geometry;
    geometry.setGridSpacingInX(dx);
    geometry.setGridSpacingInZ(dz);
    geometry.setNumberOfGridPointsInX(nx);
    geometry.setNumberOfGridPointsInZ(nz);
    geometry.setOriginInX(x0);
    geometry.setOriginInZ(z0);
    const double xs = x0 + nx / 2 * dx, zs = z0 + nz / 2 * dz;
    Source2D source;
    source.setGeometry(geometry);
    source.setLocationInX(xs);
    source.setLocationInZ(zs);
    std::vector<Station2D> stations;
    auto add = [&](double x, double z, bool surface) {
        Station2D st;
        st.setGeometry(geometry);
        st.setName("UU.T" + std::to_string(stations.size()));
        st.setLocationInX(x);
        if (surface) st.setZToFreeSurface(); else st.setLocationInZ(z);
        stations.push_back(st);
    };
    add(xs + 0.001, zs + 0.001, false);
    for (int i = 0; i < 11; ++i) add(x0 + i / 10.0 * (nx - 1) * dx, 0, true);
    for (int i = 0; i < 11; ++i) {
        add(x0, z0 + i / 10.0 * (nz - 1) * dz, false);
        add(x0 + (nx - 1) * dx, z0 + i / 10.0 * (nz - 1) * dz, false);
    }
    Homogeneous solver(geometry, source, v);
    GradientTracer2D tracer;
    tracer.initialize(GradientTracerOptions{}, geometry);
    tracer.setStations(stations);
    tracer.trace(solver);
    const auto rays = tracer.getRayPaths();
    CHECK(rays.size() == stations.size());
    // the paths as legacy-VTK polylines (src/ray/gradientTracer2d.cpp:617-655): one point per
    // segment start plus the last end point, z written as -z
    {
        const std::string vtk = std::string(std::getenv("RAY_VTK_DIR") ? std::getenv("RAY_VTK_DIR") : ".") +
                                "/rays.vtk";
        tracer.writeVTK(vtk, "ray paths");
        std::ifstream in(vtk);
        std::string l;
        std::getline(in, l); CHECK(l == "# vtk DataFile Version 3.0");
        std::getline(in, l); CHECK(l == "ray_paths");
        std::getline(in, l); CHECK(l == "ASCII");
        std::getline(in, l); CHECK(l == "DATASET POLYDATA");
        size_t nPoints = 0;
        for (const auto &r : rays) nPoints += r.empty() ? 0 : r.size() + 1;
        std::getline(in, l); CHECK(l == "POINTS " + std::to_string(nPoints) + " float");
        double px, py, pz;
        in >> px >> py >> pz;
        const auto p0 = rays[0].at(0).getStartPoint();
        CHECK(std::abs(px - p0.getPositionInX()) < 1e-9 && py == 0 && std::abs(pz + p0.getPositionInZ()) < 1e-9);
    }
    for (size_t i = 0; i < rays.size(); ++i) {
        const double d = std::hypot(stations[i].getLocationInX() - xs, stations[i].getLocationInZ() - zs);
        CHECK(!rays[i].empty());
        CHECK(std::abs(rays[i].getLength() - d) < 1.0);
        CHECK(std::abs(rays[i].getTravelTime() - d / v) < 1.e-3);
    }

    // rays through the gradient of a GPU solve in v(z) = 3000 + 0.5 z: travel times along
    // the rays agree with the solved times at the stations to a fraction of a percent
    const int mx = 201, mz = 101;
    const double h = 20;
    Geometry2D g2;
    g2.setGridSpacingInX(h);
    g2.setGridSpacingInZ(h);
    g2.setNumberOfGridPointsInX(mx);
    g2.setNumberOfGridPointsInZ(mz);
    std::vector<double> vel(static_cast<size_t>(mx) * mz);
    for (int iz = 0; iz < mz; ++iz)
        for (int ix = 0; ix < mx; ++ix) vel[static_cast<size_t>(iz) * mx + ix] = 3000 + 0.5 * iz * h;
    Model2D<double> model;
    model.initialize(g2);
    model.setNodalVelocities(vel.size(), vel.data(), EikonalXX::Ordering2D::Natural);
    SolverOptions sopt;
    sopt.setNumberOfSweeps(3);
    Solver2D<double> solver2;
    solver2.initialize(sopt, g2);
    solver2.setVelocityModel(model);
    Source2D src2;
    src2.setGeometry(g2);
    src2.setLocationInX(2010);
    src2.setLocationInZ(1210);
    solver2.setSource(src2);
    solver2.solve();
    solver2.computeTravelTimeGradientField();
    std::vector<Station2D> st2;
    for (int i = 0; i < 9; ++i) {
        Station2D st;
        st.setGeometry(g2);
        st.setLocationInX(100 + i * 450.0);
        st.setZToFreeSurface();
        st2.push_back(st);
    }
    GradientTracer2D tracer2;
    tracer2.initialize(GradientTracerOptions{}, g2);
    tracer2.setStations(st2);
    tracer2.trace(solver2);
    const auto rays2 = tracer2.getRayPaths();
    const auto tt = solver2.getTravelTimeField();
    for (size_t i = 0; i < rays2.size(); ++i) {
        const int ix = static_cast<int>(std::lround(st2[i].getOffsetInX() / h));
        const double tField = tt[static_cast<size_t>(ix)];
        CHECK(!rays2[i].empty());
        CHECK(std::abs(rays2[i].getTravelTime() - tField) < 0.01 * tField);
    }
}

int main(int argc, char **argv)
{
    const std::string mode = argc > 1 ? argv[1] : "cpu";
    try {
        if (mode == "cpu") cpuChecks(); else gpuChecks();
    } catch (const std::exception &e) {
        std::cerr << "exception: " << e.what() << "\n";
        return 2;
    }
    if (failures) {
        std::cerr << failures << " checks failed\n";
        return 1;
    }
    std::cout << "ray_api ok\n";
    return 0;
}
