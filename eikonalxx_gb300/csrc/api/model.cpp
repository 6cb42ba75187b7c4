// Model2D / Model3D (reference: src/model2d.cpp, src/model3d.cpp).  The model is a
// host-side container of cell slowness, as in the reference; the solvers upload it to
// the GPU once per setVelocityModel.
#include <algorithm>
#include <stdexcept>
#include <string>
#include <vector>
#include "eikonalxx/geometry2d.hpp"
#include "eikonalxx/io/vtkRectilinearGrid2d.hpp"
#include "eikonalxx/io/vtkRectilinearGrid3d.hpp"
#include "eikonalxx/geometry3d.hpp"
#include "eikonalxx/model2d.hpp"
#include "eikonalxx/model3d.hpp"

using namespace EikonalXX;

namespace
{
template <class U>
void checkPositive(size_t n, const U *v)
{
    if (v == nullptr) throw std::invalid_argument("velocities is NULL");
    for (size_t i = 0; i < n; ++i)
        if (!(v[i] > 0)) throw std::invalid_argument("Non-positive velocities detected");
}
}

//------------------------------------------------------------------------------ 3D
template <class T>
class Model3D<T>::Model3DImpl
{
public:
    Geometry3D geometry;
    std::vector<T> slowness;
    bool haveSlowness{false};
    bool initialized{false};
};

template <class T> Model3D<T>::Model3D() : pImpl(std::make_unique<Model3DImpl>()) {}
template <class T> Model3D<T>::Model3D(const Model3D &m) { *this = m; }
template <class T> Model3D<T>::Model3D(Model3D &&m) noexcept { *this = std::move(m); }
template <class T> Model3D<T> &Model3D<T>::operator=(const Model3D &m)
{
    if (&m != this) pImpl = std::make_unique<Model3DImpl>(*m.pImpl);
    return *this;
}
template <class T> Model3D<T> &Model3D<T>::operator=(Model3D &&m) noexcept
{
    if (&m != this) pImpl = std::move(m.pImpl);
    return *this;
}
template <class T> Model3D<T>::~Model3D() = default;
template <class T> void Model3D<T>::clear() noexcept { pImpl = std::make_unique<Model3DImpl>(); }

template <class T> void Model3D<T>::initialize(const Geometry3D &g)
{
    clear();
    if (!g.haveNumberOfGridPointsInX()) throw std::invalid_argument("Number of grid points in x not set");
    if (!g.haveNumberOfGridPointsInY()) throw std::invalid_argument("Number of grid points in y not set");
    if (!g.haveNumberOfGridPointsInZ()) throw std::invalid_argument("Number of grid points in z not set");
    if (!g.haveGridSpacingInX()) throw std::invalid_argument("Grid spacing in x not set");
    if (!g.haveGridSpacingInY()) throw std::invalid_argument("Grid spacing in y not set");
    if (!g.haveGridSpacingInZ()) throw std::invalid_argument("Grid spacing in z not set");
    pImpl->geometry = g;
    pImpl->initialized = true;
}
template <class T> bool Model3D<T>::isInitialized() const noexcept { return pImpl->initialized; }
template <class T> Geometry3D Model3D<T>::getGeometry() const
{
    if (!isInitialized()) throw std::runtime_error("Class not initialized");
    return pImpl->geometry;
}
template <class T> int Model3D<T>::getNumberOfGridPoints() const { return getGeometry().getNumberOfGridPoints(); }
template <class T> int Model3D<T>::getNumberOfCells() const { return getGeometry().getNumberOfCells(); }

// Cell slowness = 8 / (sum of the 8 corner velocities), pairs summed in the order of
// interpolate3d (src/model3d.cpp:79-137).
template <class T>
void Model3D<T>::setNodalVelocities(const int nGrid, const T v[], const Ordering3D ordering)
{
    pImpl->haveSlowness = false;
    const int n = getNumberOfGridPoints();
    if (nGrid != n)
        throw std::invalid_argument("Number of grid points = " + std::to_string(nGrid) + " must equal " +
                                    std::to_string(n));
    checkPositive(static_cast<size_t>(n), v);
    const auto &g = pImpl->geometry;
    const size_t ncx = g.getNumberOfCellsInX(), ncy = g.getNumberOfCellsInY(), ncz = g.getNumberOfCellsInZ();
    pImpl->slowness.assign(ncx * ncy * ncz, 0);
    const T eight = 8;
    for (size_t iz = 0; iz < ncz; ++iz)
        for (size_t iy = 0; iy < ncy; ++iy)
            for (size_t ix = 0; ix < ncx; ++ix) {
                size_t i1, d1, d3, d5;
                if (ordering == Ordering3D::Natural) {
                    d1 = 1; d3 = ncx + 1; d5 = (ncx + 1) * (ncy + 1);
                    i1 = iz * d5 + iy * d3 + ix;
                } else {
                    d1 = 1; d3 = ncz + 1; d5 = (ncz + 1) * (ncy + 1);
                    i1 = ix * d5 + iy * d3 + iz;
                }
                const T s1 = v[i1] + v[i1 + d1], s2 = v[i1 + d3] + v[i1 + d3 + d1];
                const T s3 = v[i1 + d5] + v[i1 + d5 + d1], s4 = v[i1 + d5 + d3] + v[i1 + d5 + d3 + d1];
                pImpl->slowness[(iz * ncy + iy) * ncx + ix] = eight / (s1 + s2 + s3 + s4);
            }
    pImpl->haveSlowness = true;
}

// Cell slowness = 1/v (src/model3d.cpp:318-375).
template <class T>
template <typename U>
void Model3D<T>::setCellularVelocities(const int nCellIn, const U v[], const Ordering3D ordering)
{
    pImpl->haveSlowness = false;
    const int nCell = getNumberOfCells();
    if (nCellIn != nCell)
        throw std::invalid_argument("Number of cells = " + std::to_string(nCellIn) + " must equal " +
                                    std::to_string(nCell));
    checkPositive(static_cast<size_t>(nCell), v);
    const auto &g = pImpl->geometry;
    const size_t ncx = g.getNumberOfCellsInX(), ncy = g.getNumberOfCellsInY(), ncz = g.getNumberOfCellsInZ();
    pImpl->slowness.assign(static_cast<size_t>(nCell), 0);
    if (ordering == Ordering3D::Natural) {
        for (size_t i = 0; i < static_cast<size_t>(nCell); ++i) pImpl->slowness[i] = static_cast<T>(U(1) / v[i]);
    } else {
        const T one = 1;
        for (size_t iz = 0; iz < ncz; ++iz)
            for (size_t iy = 0; iy < ncy; ++iy)
                for (size_t ix = 0; ix < ncx; ++ix)
                    pImpl->slowness[(iz * ncy + iy) * ncx + ix] =
                        static_cast<T>(one / v[(ix * ncy + iy) * ncz + iz]);
    }
    pImpl->haveSlowness = true;
}

template <class T> bool Model3D<T>::haveVelocities() const noexcept { return pImpl->haveSlowness; }
template <class T> const T *Model3D<T>::getSlownessPointer() const
{
    if (!haveVelocities()) throw std::runtime_error("Velocity model not yet set");
    return pImpl->slowness.data();
}
template <class T> std::vector<T> Model3D<T>::getSlowness() const
{
    (void)getSlownessPointer();
    return pImpl->slowness;
}
template <class T> std::vector<T> Model3D<T>::getVelocities() const
{
    (void)getSlownessPointer();
    std::vector<T> v(pImpl->slowness.size());
    const T one = 1;
    for (size_t i = 0; i < v.size(); ++i) v[i] = one / pImpl->slowness[i];
    return v;
}
template <class T> T Model3D<T>::getSlowness(const int ix, const int iy, const int iz) const
{
    if (!haveVelocities()) throw std::runtime_error("Velocity model not yet set");
    const auto &g = pImpl->geometry;
    const int ncx = g.getNumberOfCellsInX(), ncy = g.getNumberOfCellsInY(), ncz = g.getNumberOfCellsInZ();
    if (ix < 0 || ix >= ncx)
        throw std::invalid_argument("iCellX = " + std::to_string(ix) + " must be in range [0," + std::to_string(ncx) + ")");
    if (iy < 0 || iy >= ncy)
        throw std::invalid_argument("iCellY = " + std::to_string(iy) + " must be in range [0," + std::to_string(ncy) + ")");
    if (iz < 0 || iz >= ncz)
        throw std::invalid_argument("iCellZ = " + std::to_string(iz) + " must be in range [0," + std::to_string(ncz) + ")");
    return pImpl->slowness[(static_cast<size_t>(iz) * ncy + iy) * ncx + ix];
}
// src/model3d.cpp:470-480: the cell velocities, binary.
template <class T> void Model3D<T>::writeVTK(const std::string &fileName, const std::string &title) const
{
    const auto v = getVelocities();   // throws
    IO::VTKRectilinearGrid3D vtk;
    vtk.open(fileName, pImpl->geometry, title, true);
    vtk.writeCellularDataset(title, v.data(), Ordering3D::Natural);
    vtk.close();
}

//------------------------------------------------------------------------------ 2D
template <class T>
class Model2D<T>::Model2DImpl
{
public:
    Geometry2D geometry;
    std::vector<T> slowness;
    bool haveSlowness{false};
    bool initialized{false};
};

template <class T> Model2D<T>::Model2D() : pImpl(std::make_unique<Model2DImpl>()) {}
template <class T> Model2D<T>::Model2D(const Model2D &m) { *this = m; }
template <class T> Model2D<T>::Model2D(Model2D &&m) noexcept { *this = std::move(m); }
template <class T> Model2D<T> &Model2D<T>::operator=(const Model2D &m)
{
    if (&m != this) pImpl = std::make_unique<Model2DImpl>(*m.pImpl);
    return *this;
}
template <class T> Model2D<T> &Model2D<T>::operator=(Model2D &&m) noexcept
{
    if (&m != this) pImpl = std::move(m.pImpl);
    return *this;
}
template <class T> Model2D<T>::~Model2D() = default;
template <class T> void Model2D<T>::clear() noexcept { pImpl = std::make_unique<Model2DImpl>(); }
template <class T> void Model2D<T>::initialize(const Geometry2D &g)
{
    clear();
    if (!g.haveNumberOfGridPointsInX()) throw std::invalid_argument("Number of grid points in x not set");
    if (!g.haveNumberOfGridPointsInZ()) throw std::invalid_argument("Number of grid points in z not set");
    if (!g.haveGridSpacingInX()) throw std::invalid_argument("Grid spacing in x not set");
    if (!g.haveGridSpacingInZ()) throw std::invalid_argument("Grid spacing in z not set");
    pImpl->geometry = g;
    pImpl->initialized = true;
}
template <class T> bool Model2D<T>::isInitialized() const noexcept { return pImpl->initialized; }
template <class T> Geometry2D Model2D<T>::getGeometry() const
{
    if (!isInitialized()) throw std::runtime_error("Class not initialized");
    return pImpl->geometry;
}
template <class T> int Model2D<T>::getNumberOfGridPoints() const { return getGeometry().getNumberOfGridPoints(); }
template <class T> int Model2D<T>::getNumberOfCells() const { return getGeometry().getNumberOfCells(); }

// Cell slowness = 4 / (sum of the 4 corner velocities) (src/model2d.cpp:75-115).
template <class T>
void Model2D<T>::setNodalVelocities(const int nGrid, const T v[], const Ordering2D ordering)
{
    pImpl->haveSlowness = false;
    const int n = getNumberOfGridPoints();
    if (nGrid != n)
        throw std::invalid_argument("Number of grid points = " + std::to_string(nGrid) + " must equal " +
                                    std::to_string(n));
    checkPositive(static_cast<size_t>(n), v);
    const auto &g = pImpl->geometry;
    const size_t ncx = g.getNumberOfCellsInX(), ncz = g.getNumberOfCellsInZ();
    pImpl->slowness.assign(ncx * ncz, 0);
    const T four = 4;
    for (size_t iz = 0; iz < ncz; ++iz)
        for (size_t ix = 0; ix < ncx; ++ix) {
            size_t i1, d3;
            if (ordering == Ordering2D::Natural) { i1 = iz * (ncx + 1) + ix; d3 = ncx + 1; }
            else { i1 = ix * (ncz + 1) + iz; d3 = ncz + 1; }
            const T s1 = v[i1] + v[i1 + 1], s2 = v[i1 + d3] + v[i1 + d3 + 1];
            pImpl->slowness[iz * ncx + ix] = four / (s1 + s2);
        }
    pImpl->haveSlowness = true;
}

template <class T>
template <typename U>
void Model2D<T>::setCellularVelocities(const int nCellIn, const U v[], const Ordering2D ordering)
{
    pImpl->haveSlowness = false;
    const int nCell = getNumberOfCells();
    if (nCellIn != nCell)
        throw std::invalid_argument("Number of cells = " + std::to_string(nCellIn) + " must equal " +
                                    std::to_string(nCell));
    checkPositive(static_cast<size_t>(nCell), v);
    const auto &g = pImpl->geometry;
    const size_t ncx = g.getNumberOfCellsInX(), ncz = g.getNumberOfCellsInZ();
    pImpl->slowness.assign(static_cast<size_t>(nCell), 0);
    if (ordering == Ordering2D::Natural) {
        for (size_t i = 0; i < static_cast<size_t>(nCell); ++i) pImpl->slowness[i] = static_cast<T>(U(1) / v[i]);
    } else {
        const T one = 1;
        for (size_t iz = 0; iz < ncz; ++iz)
            for (size_t ix = 0; ix < ncx; ++ix)
                pImpl->slowness[iz * ncx + ix] = static_cast<T>(one / v[ix * ncz + iz]);
    }
    pImpl->haveSlowness = true;
}
template <class T> bool Model2D<T>::haveVelocities() const noexcept { return pImpl->haveSlowness; }
template <class T> const T *Model2D<T>::getSlownessPointer() const
{
    if (!haveVelocities()) throw std::runtime_error("Velocity model not yet set");
    return pImpl->slowness.data();
}
template <class T> std::vector<T> Model2D<T>::getSlowness() const
{
    (void)getSlownessPointer();
    return pImpl->slowness;
}
template <class T> std::vector<T> Model2D<T>::getVelocities() const
{
    (void)getSlownessPointer();
    std::vector<T> v(pImpl->slowness.size());
    const T one = 1;
    for (size_t i = 0; i < v.size(); ++i) v[i] = one / pImpl->slowness[i];
    return v;
}
template <class T> T Model2D<T>::getSlowness(const int ix, const int iz) const
{
    if (!haveVelocities()) throw std::runtime_error("Velocity model not yet set");
    const auto &g = pImpl->geometry;
    const int ncx = g.getNumberOfCellsInX(), ncz = g.getNumberOfCellsInZ();
    if (ix < 0 || ix >= ncx)
        throw std::invalid_argument("iCellX = " + std::to_string(ix) + " must be in range [0," + std::to_string(ncx) + ")");
    if (iz < 0 || iz >= ncz)
        throw std::invalid_argument("iCellZ = " + std::to_string(iz) + " must be in range [0," + std::to_string(ncz) + ")");
    return pImpl->slowness[static_cast<size_t>(iz) * ncx + ix];
}
// src/model2d.cpp:435-445: the cell velocities, binary.
template <class T> void Model2D<T>::writeVTK(const std::string &fileName, const std::string &title) const
{
    const auto v = getVelocities();   // throws
    IO::VTKRectilinearGrid2D vtk;
    vtk.open(fileName, pImpl->geometry, title, true);
    vtk.writeCellularDataset(title, v.data(), Ordering2D::Natural);
    vtk.close();
}

template class EikonalXX::Model3D<double>;
template class EikonalXX::Model3D<float>;
template void EikonalXX::Model3D<double>::setCellularVelocities(int, const double[], Ordering3D);
template void EikonalXX::Model3D<double>::setCellularVelocities(int, const float[], Ordering3D);
template void EikonalXX::Model3D<float>::setCellularVelocities(int, const double[], Ordering3D);
template void EikonalXX::Model3D<float>::setCellularVelocities(int, const float[], Ordering3D);
template class EikonalXX::Model2D<double>;
template class EikonalXX::Model2D<float>;
template void EikonalXX::Model2D<double>::setCellularVelocities(int, const double[], Ordering2D);
template void EikonalXX::Model2D<double>::setCellularVelocities(int, const float[], Ordering2D);
template void EikonalXX::Model2D<float>::setCellularVelocities(int, const double[], Ordering2D);
template void EikonalXX::Model2D<float>::setCellularVelocities(int, const float[], Ordering2D);
