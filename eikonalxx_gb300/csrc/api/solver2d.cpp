// Solver2D<T> (reference: src/solver2d.cpp) over the C ABI; station times and the
// gradient field are computed on the GPU from the solved field.
#include <cmath>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>
#include "eikonalxx/geometry2d.hpp"
#include "eikonalxx/io/vtkRectilinearGrid2d.hpp"
#include "eikonalxx/model2d.hpp"
#include "eikonalxx/solver2d.hpp"
#include "eikonalxx/solverOptions.hpp"
#include "eikonalxx/source2d.hpp"
#include "eikonalxx/station2d.hpp"
#include "gpu_context.hpp"

using namespace EikonalXX;

template <class T>
class Solver2D<T>::Solver2DImpl
{
public:
    Detail::GpuContext gpu;
    Geometry2D geometry;
    SolverOptions options;
    Model2D<T> model;
    Source2D source;
    std::vector<Station2D> stations;
    std::vector<T> travelTimes, gradient, stationTimes;
    bool initialized{false}, haveModel{false}, haveSource{false}, haveField{false}, haveGradient{false};
    bool gridOnDevice{false}, modelOnDevice{false};

    // Travel times at the stations (src/solver2d.cpp:106-167): bilinear interpolation of
    // the solved field on the GPU, the straight-ray time in the source cell.
    void interpolate()
    {
        stationTimes.assign(stations.size(), 0);
        if (stations.empty()) return;
        std::vector<eikx_source2d> xz(stations.size());
        for (size_t i = 0; i < stations.size(); ++i) xz[i] = {stations[i].getLocationInX(), stations[i].getLocationInZ()};
        std::vector<double> t(stations.size());
        Detail::check(eikx_station_times2d(gpu.get(), 0, xz.data(), static_cast<int>(xz.size()), t.data()));
        for (size_t i = 0; i < t.size(); ++i) stationTimes[i] = static_cast<T>(t[i]);
    }
};

template <class T> Solver2D<T>::Solver2D() : pImpl(std::make_unique<Solver2DImpl>()) {}
template <class T> Solver2D<T>::~Solver2D() = default;

template <class T> void Solver2D<T>::clear() noexcept
{
    auto &p = *pImpl;
    p.geometry.clear();
    p.options.clear();
    p.model.clear();
    p.source.clear();
    p.stations.clear();
    p.travelTimes.clear();
    p.gradient.clear();
    p.stationTimes.clear();
    p.initialized = p.haveModel = p.haveSource = p.haveField = p.haveGradient = false;
    p.gridOnDevice = p.modelOnDevice = false;
}

template <class T> void Solver2D<T>::initialize(const SolverOptions &options, const Geometry2D &g)
{
    clear();
    if (!g.haveNumberOfGridPointsInX()) throw std::invalid_argument("Grid points in x not set on geometry");
    if (!g.haveNumberOfGridPointsInZ()) throw std::invalid_argument("Grid points in z not set on geometry");
    if (!g.haveGridSpacingInX()) throw std::invalid_argument("Grid spacing in x not set on geometry");
    if (!g.haveGridSpacingInZ()) throw std::invalid_argument("Grid spacing in z not set on geometry");
    pImpl->geometry = g;
    pImpl->options = options;
    pImpl->travelTimes.assign(static_cast<size_t>(g.getNumberOfGridPoints()), 0);
    pImpl->initialized = true;
}
template <class T> bool Solver2D<T>::isInitialized() const noexcept { return pImpl->initialized; }
template <class T> SolverOptions Solver2D<T>::getOptions() const
{
    if (!isInitialized()) throw std::runtime_error("Class not initialized");
    return pImpl->options;
}
template <class T> Geometry2D Solver2D<T>::getGeometry() const
{
    if (!isInitialized()) throw std::runtime_error("Class not initialized");
    return pImpl->geometry;
}
template <class T> void Solver2D<T>::setVelocityModel(const Model2D<T> &m)
{
    pImpl->haveModel = pImpl->haveField = pImpl->haveGradient = false;
    if (!isInitialized()) throw std::runtime_error("Class not initialized");
    if (!m.isInitialized()) throw std::invalid_argument("Velocity model not initialized");
    if (m.getGeometry() != pImpl->geometry)
        throw std::invalid_argument("Velocity model's geometry does not match the solver's geometry");
    pImpl->model = m;
    pImpl->modelOnDevice = false;
    pImpl->haveModel = true;
}
template <class T> Model2D<T> Solver2D<T>::getVelocityModel() const
{
    if (!haveVelocityModel()) throw std::runtime_error("Velocity model not set");
    return pImpl->model;
}
template <class T> bool Solver2D<T>::haveVelocityModel() const noexcept { return pImpl->haveModel; }
template <class T> T Solver2D<T>::getSlowness(const int ix, const int iz) const
{
    if (!haveVelocityModel()) throw std::runtime_error("Velocity model not set");
    return pImpl->model.getSlowness(ix, iz);
}
template <class T> void Solver2D<T>::setSource(const std::pair<double, double> &loc)
{
    pImpl->haveSource = pImpl->haveField = pImpl->haveGradient = false;
    if (!isInitialized()) throw std::runtime_error("Class not initialized");
    Source2D s;
    s.setGeometry(pImpl->geometry);
    s.setLocationInX(loc.first);
    s.setLocationInZ(loc.second);
    setSource(s);
}
template <class T> void Solver2D<T>::setSource(const Source2D &s)
{
    pImpl->haveSource = pImpl->haveField = pImpl->haveGradient = false;
    if (!isInitialized()) throw std::runtime_error("Class not initialized");
    if (!s.haveLocationInX()) throw std::invalid_argument("Source location in x not set");
    if (!s.haveLocationInZ()) throw std::invalid_argument("Source location in z not set");
    pImpl->source = s;
    pImpl->haveSource = true;
}
template <class T> Source2D Solver2D<T>::getSource() const
{
    if (!haveSource()) throw std::runtime_error("Source location not set");
    return pImpl->source;
}
template <class T> bool Solver2D<T>::haveSource() const noexcept { return pImpl->haveSource; }
template <class T> void Solver2D<T>::setStations(const std::vector<Station2D> &stations)
{
    const auto g = getGeometry();
    for (const auto &st : stations) {
        const auto sg = st.getGeometry();
        if (g.getNumberOfGridPointsInX() != sg.getNumberOfGridPointsInX()) throw std::invalid_argument("nx is inconsistent");
        if (g.getNumberOfGridPointsInZ() != sg.getNumberOfGridPointsInZ()) throw std::invalid_argument("nz is inconsistent");
        if (std::abs(g.getGridSpacingInX() - sg.getGridSpacingInX()) > 1.e-3) throw std::invalid_argument("dx is inconsistent");
        if (std::abs(g.getGridSpacingInZ() - sg.getGridSpacingInZ()) > 1.e-3) throw std::invalid_argument("dz is inconsistent");
        if (std::abs(g.getOriginInX() - sg.getOriginInX()) > 1.e-3) throw std::invalid_argument("x0 is inconsistent");
        if (std::abs(g.getOriginInZ() - sg.getOriginInZ()) > 1.e-3) throw std::invalid_argument("z0 is inconsistent");
        if (!st.haveLocationInX() || !st.haveLocationInZ()) throw std::invalid_argument("Station location not set");
    }
    pImpl->stations = stations;
    if (pImpl->haveField) pImpl->interpolate();
}
template <class T> std::vector<Station2D> Solver2D<T>::getStations() const { return pImpl->stations; }
template <class T> const std::vector<Station2D> &Solver2D<T>::getStationsReference() const { return pImpl->stations; }

template <class T> void Solver2D<T>::solve()
{
    auto &p = *pImpl;
    p.haveField = p.haveGradient = false;
    if (!isInitialized()) throw std::runtime_error("Class not initialized");
    if (!haveVelocityModel()) throw std::runtime_error("Velocity model not set");
    if (!haveSource()) throw std::runtime_error("Source location not set");
    eikx_ctx *ctx = p.gpu.get();
    const auto &g = p.geometry;
    if (!p.gridOnDevice) {
        Detail::check(eikx_set_grid2d(ctx, g.getNumberOfGridPointsInX(), g.getNumberOfGridPointsInZ(),
                                      g.getGridSpacingInX(), g.getGridSpacingInZ(), g.getOriginInX(),
                                      g.getOriginInZ()));
        p.gridOnDevice = true;
        p.modelOnDevice = false;
    }
    if (!p.modelOnDevice) {
        Detail::check(eikx_set_slowness2d(ctx, p.model.getSlownessPointer(), Detail::dtypeOf<T>(),
                                          EIKX_ORDER_NATURAL, EIKX_HOST));
        p.modelOnDevice = true;
    }
    const eikx_source2d src{p.source.getLocationInX(), p.source.getLocationInZ()};
    const eikx_options opt = Detail::toOptions(p.options);
    Detail::check(eikx_solve2d(ctx, &src, 1, &opt, Detail::dtypeOf<T>(), p.travelTimes.data(), EIKX_HOST));
    p.haveField = true;
    p.interpolate();
}

// The gradient of the solved field on the GPU (src/gradient.hpp:20-289): central
// differences inside, second-order one-sided differences at the edges, the analytic
// gradient at the source cell's corners; interleaved (dT/dx, dT/dz) per node.
template <class T> void Solver2D<T>::computeTravelTimeGradientField()
{
    if (!haveTravelTimeField()) throw std::runtime_error("Travel time field not yet computed");
    auto &p = *pImpl;
    p.gradient.resize(2 * p.travelTimes.size());
    Detail::check(eikx_gradient2d(p.gpu.get(), 0, p.gradient.data(), EIKX_HOST));
    p.haveGradient = true;
}

template <class T> std::vector<T> Solver2D<T>::getTravelTimeField() const { return pImpl->travelTimes; }
template <class T> const T *Solver2D<T>::getTravelTimeFieldPointer() const
{
    if (!haveTravelTimeField()) throw std::runtime_error("Travel time field not yet computed");
    return pImpl->travelTimes.data();
}
template <class T> bool Solver2D<T>::haveTravelTimeField() const noexcept { return pImpl->haveField; }
template <class T> std::vector<T> Solver2D<T>::getTravelTimesAtStations() const
{
    if (!haveTravelTimeField()) throw std::runtime_error("Travel time field not yet computed");
    return pImpl->stationTimes;
}
template <class T> bool Solver2D<T>::haveTravelTimeGradientField() const noexcept { return pImpl->haveGradient; }
template <class T> std::vector<T> Solver2D<T>::getTravelTimeGradientField() const
{
    if (!haveTravelTimeGradientField()) throw std::runtime_error("Travel time gradient field not computed");
    return pImpl->gradient;
}
template <class T> const T *Solver2D<T>::getTravelTimeGradientFieldPointer() const
{
    if (!haveTravelTimeGradientField()) throw std::runtime_error("Travel time gradient field not computed");
    return pImpl->gradient.data();
}
// src/solver2d.cpp:946-964: the travel times (and the gradient as vectors), binary.
template <class T> void Solver2D<T>::writeVTK(const std::string &fileName, const std::string &title,
                                              const bool writeGradient) const
{
    const T *t = getTravelTimeFieldPointer();                                  // throws
    const T *g = writeGradient ? getTravelTimeGradientFieldPointer() : nullptr;  // throws
    IO::VTKRectilinearGrid2D vtk;
    vtk.open(fileName, pImpl->geometry, title, true);
    vtk.writeNodalDataset(title, t, Ordering2D::Natural);
    if (writeGradient) vtk.writeNodalVectorDataset(title + "_gradient", g, Ordering2D::Natural);
    vtk.close();
}

template class EikonalXX::Solver2D<double>;
template class EikonalXX::Solver2D<float>;
