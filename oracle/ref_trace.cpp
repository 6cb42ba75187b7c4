// Test infrastructure: drives the reference's own 2D gradient ray tracer
// (EikonalXX::Ray::GradientTracer2D, src/ray/gradientTracer2d.cpp, compiled from the
// reference checkout into oracle/_ref with the host shim) on a given gradient field, so
// that the oracle's restatement of trace() can be compared with it.  This file is a
// driver only: a solver object serving the arrays through the reference's ISolver2D
// interface, and a C entry point.
#include <cstddef>
#include <limits>
#include <utility>
#include <vector>
#include "eikonalxx/abstractBaseClass/solver2d.hpp"
#include "eikonalxx/geometry2d.hpp"
#include "eikonalxx/ray/gradientTracer2d.hpp"
#include "eikonalxx/ray/gradientTracerOptions.hpp"
#include "eikonalxx/ray/path2d.hpp"
#include "eikonalxx/ray/point2d.hpp"
#include "eikonalxx/ray/segment2d.hpp"
#include "eikonalxx/source2d.hpp"
#include "eikonalxx/station2d.hpp"

namespace {

template <class T>
class ArraySolver : public EikonalXX::AbstractBaseClass::ISolver2D<T> {
public:
    ArraySolver(const T *grad, size_t nGrad, const double *slow, int ncx, const EikonalXX::Source2D &src)
        : grad_(grad, grad + nGrad), slow_(slow), ncx_(ncx), src_(src) {}
    bool haveVelocityModel() const noexcept override { return true; }
    std::vector<T> getTravelTimeField() const override { return {}; }
    const T *getTravelTimeFieldPointer() const override { return nullptr; }
    std::vector<T> getTravelTimeGradientField() const override { return grad_; }
    const T *getTravelTimeGradientFieldPointer() const override { return grad_.data(); }
    bool haveTravelTimeField() const noexcept override { return false; }
    bool haveTravelTimeGradientField() const noexcept override { return true; }
    EikonalXX::Source2D getSource() const override { return src_; }
    bool haveSource() const noexcept override { return true; }
    T getSlowness(int ix, int iz) const override { return static_cast<T>(slow_[static_cast<size_t>(iz) * ncx_ + ix]); }

private:
    std::vector<T> grad_;
    const double *slow_;
    int ncx_;
    EikonalXX::Source2D src_;
};

template <class T>
int run(int nx, int nz, double dx, double dz, double x0, double z0, const T *grad, const double *slow, double sx,
        double sz, int n, const double *stations, int nRsf, const int *radii, const double *scales, int capacity,
        double *segments, int *counts) {
    EikonalXX::Geometry2D g;
    g.setNumberOfGridPointsInX(nx);
    g.setNumberOfGridPointsInZ(nz);
    g.setGridSpacingInX(dx);
    g.setGridSpacingInZ(dz);
    g.setOriginInX(x0);
    g.setOriginInZ(z0);
    EikonalXX::Source2D src;
    src.setGeometry(g);
    src.setLocationInX(sx);
    src.setLocationInZ(sz);
    std::vector<EikonalXX::Station2D> st(n);
    for (int i = 0; i < n; ++i) {
        st[i].setGeometry(g);
        st[i].setLocationInX(stations[2 * i]);
        st[i].setLocationInZ(stations[2 * i + 1]);
    }
    std::vector<std::pair<int, double>> rsf;
    for (int k = 0; k < nRsf; ++k) rsf.emplace_back(radii[k], scales[k]);
    EikonalXX::Ray::GradientTracerOptions options;
    options.setRadiusScaleFactor(rsf);
    EikonalXX::Ray::GradientTracer2D tracer;
    tracer.initialize(options, g);
    tracer.setStations(st);
    ArraySolver<T> solver(grad, 2 * static_cast<size_t>(nx) * nz, slow, nx - 1, src);
    tracer.trace(solver);
    const auto paths = tracer.getRayPaths();
    for (int i = 0; i < n; ++i) {
        const auto &p = paths[i];
        if (static_cast<int>(p.size()) > capacity) {
            counts[i] = -2;
            continue;
        }
        counts[i] = static_cast<int>(p.size());
        int k = 0;
        for (const auto &s : p) {
            double *o = segments + (static_cast<size_t>(i) * capacity + k++) * 6;
            const auto a = s.getStartPoint(), b = s.getEndPoint();
            o[0] = a.getPositionInX(); o[1] = a.getPositionInZ();
            o[2] = b.getPositionInX(); o[3] = b.getPositionInZ();
            o[4] = s.getSlowness();
            o[5] = s.haveVelocityModelCellIndex() ? s.getVelocityModelCellIndex() : -1;
        }
    }
    return 0;
}

}  // namespace

extern "C" int ref_trace_rays2d(int precision, int nx, int nz, double dx, double dz, double x0, double z0,
                                const void *grad, const double *slow, double sx, double sz, int n,
                                const double *stations, int nRsf, const int *radii, const double *scales,
                                int capacity, double *segments, int *counts) {
    try {
        return precision == 0
            ? run<float>(nx, nz, dx, dz, x0, z0, static_cast<const float *>(grad), slow, sx, sz, n, stations, nRsf,
                         radii, scales, capacity, segments, counts)
            : run<double>(nx, nz, dx, dz, x0, z0, static_cast<const double *>(grad), slow, sx, sz, n, stations,
                          nRsf, radii, scales, capacity, segments, counts);
    } catch (...) {
        return 1;
    }
}
