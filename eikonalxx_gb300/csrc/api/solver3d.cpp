// Solver3D<T> (reference: src/solver3d.cpp) over the C ABI.
#include <cmath>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>
#include "eikonalxx/geometry3d.hpp"
#include "eikonalxx/model3d.hpp"
#include "eikonalxx/solver3d.hpp"
#include "eikonalxx/solverOptions.hpp"
#include "eikonalxx/source3d.hpp"
#include "eikonalxx/station3d.hpp"
#include "gpu_context.hpp"

using namespace EikonalXX;

template <class T>
class Solver3D<T>::Solver3DImpl
{
public:
    Detail::GpuContext gpu;
    Geometry3D geometry;
    SolverOptions options;
    Model3D<T> model;
    Source3D source;
    std::vector<Station3D> stations;
    std::vector<T> travelTimes, gradient, stationTimes;
    bool initialized{false}, haveModel{false}, haveSource{false}, haveField{false}, haveGradient{false};
    bool gridOnDevice{false}, modelOnDevice{false};

    // travel times at the stations, interpolated on the GPU from the solved field
    void interpolate()
    {
        stationTimes.assign(stations.size(), 0);
        if (stations.empty()) return;
        std::vector<eikx_source3d> xyz(stations.size());
        for (size_t i = 0; i < stations.size(); ++i)
            xyz[i] = {stations[i].getLocationInX(), stations[i].getLocationInY(), stations[i].getLocationInZ()};
        std::vector<double> t(stations.size());
        Detail::check(eikx_station_times3d(gpu.get(), 0, xyz.data(), static_cast<int>(xyz.size()), t.data()));
        for (size_t i = 0; i < t.size(); ++i) stationTimes[i] = static_cast<T>(t[i]);
    }
};

template <class T> Solver3D<T>::Solver3D() : pImpl(std::make_unique<Solver3DImpl>()) {}
template <class T> Solver3D<T>::~Solver3D() = default;

template <class T> void Solver3D<T>::clear() noexcept
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

template <class T> void Solver3D<T>::initialize(const SolverOptions &options, const Geometry3D &g)
{
    clear();
    if (!g.haveNumberOfGridPointsInX()) throw std::invalid_argument("Grid points in x not set on geometry");
    if (!g.haveNumberOfGridPointsInY()) throw std::invalid_argument("Grid points in y not set on geometry");
    if (!g.haveNumberOfGridPointsInZ()) throw std::invalid_argument("Grid points in z not set on geometry");
    if (!g.haveGridSpacingInX()) throw std::invalid_argument("Grid spacing in x not set on geometry");
    if (!g.haveGridSpacingInY()) throw std::invalid_argument("Grid spacing in y not set on geometry");
    if (!g.haveGridSpacingInZ()) throw std::invalid_argument("Grid spacing in z not set on geometry");
    pImpl->geometry = g;
    pImpl->options = options;
    pImpl->travelTimes.assign(static_cast<size_t>(g.getNumberOfGridPoints()), 0);
    pImpl->initialized = true;
}
template <class T> bool Solver3D<T>::isInitialized() const noexcept { return pImpl->initialized; }
template <class T> SolverOptions Solver3D<T>::getOptions() const
{
    if (!isInitialized()) throw std::runtime_error("Class not initialized");
    return pImpl->options;
}
template <class T> Geometry3D Solver3D<T>::getGeometry() const
{
    if (!isInitialized()) throw std::runtime_error("Class not initialized");
    return pImpl->geometry;
}

template <class T> void Solver3D<T>::setVelocityModel(const Model3D<T> &m)
{
    pImpl->haveModel = pImpl->haveField = false;
    if (!isInitialized()) throw std::runtime_error("Class not initialized");
    if (!m.isInitialized()) throw std::invalid_argument("Velocity model not initialized");
    if (m.getGeometry() != pImpl->geometry)
        throw std::invalid_argument("Velocity model's geometry does not match the solver's geometry");
    pImpl->model = m;
    pImpl->modelOnDevice = false;
    pImpl->haveModel = true;
}
template <class T> Model3D<T> Solver3D<T>::getVelocityModel() const
{
    if (!haveVelocityModel()) throw std::runtime_error("Velocity model not set");
    return pImpl->model;
}
template <class T> bool Solver3D<T>::haveVelocityModel() const noexcept { return pImpl->haveModel; }
template <class T> T Solver3D<T>::getSlowness(const int ix, const int iy, const int iz) const
{
    if (!haveVelocityModel()) throw std::runtime_error("Velocity model not set");
    return pImpl->model.getSlowness(ix, iy, iz);
}

template <class T> void Solver3D<T>::setSource(const std::tuple<double, double, double> &loc)
{
    pImpl->haveSource = pImpl->haveField = false;
    if (!isInitialized()) throw std::runtime_error("Class not initialized");
    Source3D s;
    s.setGeometry(pImpl->geometry);
    s.setLocationInX(std::get<0>(loc));
    s.setLocationInY(std::get<1>(loc));
    s.setLocationInZ(std::get<2>(loc));
    setSource(s);
}
template <class T> void Solver3D<T>::setSource(const Source3D &s)
{
    pImpl->haveSource = pImpl->haveField = false;
    if (!isInitialized()) throw std::runtime_error("Class not initialized");
    if (!s.haveLocationInX()) throw std::invalid_argument("Source location in x not set");
    if (!s.haveLocationInY()) throw std::invalid_argument("Source location in y not set");
    if (!s.haveLocationInZ()) throw std::invalid_argument("Source location in z not set");
    pImpl->source = s;
    pImpl->haveSource = true;
}
template <class T> Source3D Solver3D<T>::getSource() const
{
    if (!haveSource()) throw std::runtime_error("Source location not set");
    return pImpl->source;
}
template <class T> bool Solver3D<T>::haveSource() const noexcept { return pImpl->haveSource; }

template <class T> void Solver3D<T>::setStations(const std::vector<Station3D> &stations)
{
    const auto g = getGeometry();
    for (const auto &st : stations) {
        const auto sg = st.getGeometry();
        if (g.getNumberOfGridPointsInX() != sg.getNumberOfGridPointsInX()) throw std::invalid_argument("nx is inconsistent");
        if (g.getNumberOfGridPointsInY() != sg.getNumberOfGridPointsInY()) throw std::invalid_argument("ny is inconsistent");
        if (g.getNumberOfGridPointsInZ() != sg.getNumberOfGridPointsInZ()) throw std::invalid_argument("nz is inconsistent");
        if (std::abs(g.getGridSpacingInX() - sg.getGridSpacingInX()) > 1.e-3) throw std::invalid_argument("dx is inconsistent");
        if (std::abs(g.getGridSpacingInY() - sg.getGridSpacingInY()) > 1.e-3) throw std::invalid_argument("dy is inconsistent");
        if (std::abs(g.getGridSpacingInZ() - sg.getGridSpacingInZ()) > 1.e-3) throw std::invalid_argument("dz is inconsistent");
        if (std::abs(g.getOriginInX() - sg.getOriginInX()) > 1.e-3) throw std::invalid_argument("x0 is inconsistent");
        if (std::abs(g.getOriginInY() - sg.getOriginInY()) > 1.e-3) throw std::invalid_argument("y0 is inconsistent");
        if (std::abs(g.getOriginInZ() - sg.getOriginInZ()) > 1.e-3) throw std::invalid_argument("z0 is inconsistent");
    }
    pImpl->stations = stations;
    if (pImpl->haveField) pImpl->interpolate();
}
template <class T> std::vector<Station3D> Solver3D<T>::getStations() const { return pImpl->stations; }
template <class T> const std::vector<Station3D> &Solver3D<T>::getStationsReference() const { return pImpl->stations; }

template <class T> void Solver3D<T>::solve()
{
    auto &p = *pImpl;
    p.haveField = p.haveGradient = false;
    if (!isInitialized()) throw std::runtime_error("Class not initialized");
    if (!haveVelocityModel()) throw std::runtime_error("Velocity model not set");
    if (!haveSource()) throw std::runtime_error("Source location not set");
    eikx_ctx *ctx = p.gpu.get();
    const auto &g = p.geometry;
    if (!p.gridOnDevice) {
        Detail::check(eikx_set_grid3d(ctx, g.getNumberOfGridPointsInX(), g.getNumberOfGridPointsInY(),
                                      g.getNumberOfGridPointsInZ(), g.getGridSpacingInX(), g.getGridSpacingInY(),
                                      g.getGridSpacingInZ(), g.getOriginInX(), g.getOriginInY(), g.getOriginInZ()));
        p.gridOnDevice = true;
        p.modelOnDevice = false;
    }
    if (!p.modelOnDevice) {
        Detail::check(eikx_set_slowness3d(ctx, p.model.getSlownessPointer(), Detail::dtypeOf<T>(),
                                          EIKX_ORDER_NATURAL, EIKX_HOST));
        p.modelOnDevice = true;
    }
    const eikx_source3d src{p.source.getLocationInX(), p.source.getLocationInY(), p.source.getLocationInZ()};
    const eikx_options opt = Detail::toOptions(p.options);
    Detail::check(eikx_solve3d(ctx, &src, 1, &opt, Detail::dtypeOf<T>(), p.travelTimes.data(), EIKX_HOST));
    p.haveField = true;
    p.interpolate();
}

template <class T> void Solver3D<T>::computeTravelTimeGradientField()
{
    if (!haveTravelTimeField()) throw std::runtime_error("Travel time field not yet computed");
    auto &p = *pImpl;
    p.gradient.resize(3 * p.travelTimes.size());
    Detail::check(eikx_gradient3d(p.gpu.get(), 0, p.gradient.data(), EIKX_HOST));
    p.haveGradient = true;
}

template <class T> std::vector<T> Solver3D<T>::getTravelTimesAtStations() const
{
    if (!haveTravelTimeField()) throw std::runtime_error("Travel time field not yet computed");
    return pImpl->stationTimes;
}

template <class T> std::vector<T> Solver3D<T>::getTravelTimeField() const { return pImpl->travelTimes; }
template <class T> const T *Solver3D<T>::getTravelTimeFieldPointer() const
{
    if (!haveTravelTimeField()) throw std::runtime_error("Travel time field not yet computed");
    return pImpl->travelTimes.data();
}
template <class T> bool Solver3D<T>::haveTravelTimeField() const noexcept { return pImpl->haveField; }
template <class T> bool Solver3D<T>::haveTravelTimeGradientField() const noexcept { return pImpl->haveGradient; }
template <class T> std::vector<T> Solver3D<T>::getTravelTimeGradientField() const
{
    if (!haveTravelTimeGradientField()) throw std::runtime_error("Travel time gradient field not computed");
    return pImpl->gradient;
}
template <class T> const T *Solver3D<T>::getTravelTimeGradientFieldPointer() const
{
    if (!haveTravelTimeGradientField()) throw std::runtime_error("Travel time gradient field not computed");
    return pImpl->gradient.data();
}

template class EikonalXX::Solver3D<double>;
template class EikonalXX::Solver3D<float>;
