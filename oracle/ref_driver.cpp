// ORACLE — test infrastructure only.
//
// Drives the reference's OWN hot-path code, compiled in place from the reference's
// sources by oracle/build_ref.py into oracle/_ref/libeikx_ref.so:
//   * Solver3DSweep<T,E>::updateFSM      include/private/solver3d.hpp:150-326
//   * Solver2DSweep<T,E>::updateFSM      include/private/solver2d.hpp:203-327
//   * Graph3D<E>::initialize             src/graph3d.cpp:120-221
// with a project-written host shim for SYCL/TBB (oracle/shim/).  Because the
// reference's Solver3D::solve stops after two sweeps (src/solver3d.cpp:460-463), the
// solve schedule below restates the one Solver2D::solve runs (src/solver2d.cpp:462-565)
// for all 8 (3D) or 4 (2D) sweep objects: corner initialisation as in
// src/solver3d.cpp:21-84 / src/solver2d.cpp:61-105 (computed with the reference's own
// computeAnalyticalTravelTime), one source-limited pass, then nSweeps full passes.
//
// The reference's per-node debug prints (solverUtilities3d.hpp:327,554,822) are
// compiled into a no-op stream: `cout` is redefined, after the standard headers are
// included, to an inline stream object whose operators do nothing.
#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>
#include <CL/sycl.hpp>

namespace std {
struct EikxNullStream {
    template <class V> EikxNullStream &operator<<(const V &) { return *this; }
    EikxNullStream &operator<<(std::ostream &(*)(std::ostream &)) { return *this; }
    std::streamsize precision(std::streamsize) { return 0; }
};
inline EikxNullStream eikx_null_cout;
}  // namespace std
#define cout eikx_null_cout

#include "eikonalxx/enums.hpp"
#include "eikonalxx/geometry2d.hpp"
#include "eikonalxx/geometry3d.hpp"
#include "eikonalxx/graph3d.hpp"
#include "eikonalxx/model2d.hpp"
#include "eikonalxx/model3d.hpp"
#include "eikonalxx/solverOptions.hpp"
#include "private/solver3d.hpp"
#undef HUGE
#include "private/solver2d.hpp"

using namespace EikonalXX;

// The sweep objects' setVelocityModel (LSM only) reads the model's slowness pointer;
// the FSM schedule here never calls it, so the model classes are not built.
namespace EikonalXX {
template <> const double *Model3D<double>::getSlownessPointer() const {
    throw std::runtime_error("not built in the oracle");
}
template <> const float *Model3D<float>::getSlownessPointer() const {
    throw std::runtime_error("not built in the oracle");
}
template <> const double *Model2D<double>::getSlownessPointer() const {
    throw std::runtime_error("not built in the oracle");
}
template <> const float *Model2D<float>::getSlownessPointer() const {
    throw std::runtime_error("not built in the oracle");
}
}  // namespace EikonalXX

namespace {

template <class T>
struct Sweeps3 {
    Solver3DSweep<T, SweepNumber3D::Sweep1> s1;
    Solver3DSweep<T, SweepNumber3D::Sweep2> s2;
    Solver3DSweep<T, SweepNumber3D::Sweep3> s3;
    Solver3DSweep<T, SweepNumber3D::Sweep4> s4;
    Solver3DSweep<T, SweepNumber3D::Sweep5> s5;
    Solver3DSweep<T, SweepNumber3D::Sweep6> s6;
    Solver3DSweep<T, SweepNumber3D::Sweep7> s7;
    Solver3DSweep<T, SweepNumber3D::Sweep8> s8;
    template <class F> void each(F f) { f(s1); f(s2); f(s3); f(s4); f(s5); f(s6); f(s7); f(s8); }
    void run(int e, const T *slow, T *tt, bool init) {
        switch (e) {
            case 0: s1.updateFSM(slow, tt, init); break;
            case 1: s2.updateFSM(slow, tt, init); break;
            case 2: s3.updateFSM(slow, tt, init); break;
            case 3: s4.updateFSM(slow, tt, init); break;
            case 4: s5.updateFSM(slow, tt, init); break;
            case 5: s6.updateFSM(slow, tt, init); break;
            case 6: s7.updateFSM(slow, tt, init); break;
            default: s8.updateFSM(slow, tt, init); break;
        }
    }
};

template <class T>
std::unique_ptr<Sweeps3<T>> setup3(int nx, int ny, int nz, double dx, double dy, double dz,
                                   int isx, int isy, int isz, double xo, double yo, double zo,
                                   int radius, T sSrc) {
    Geometry3D g;
    g.setNumberOfGridPointsInX(nx); g.setNumberOfGridPointsInY(ny); g.setNumberOfGridPointsInZ(nz);
    g.setGridSpacingInX(dx); g.setGridSpacingInY(dy); g.setGridSpacingInZ(dz);
    SolverOptions o;
    o.setAlgorithm(SolverAlgorithm::FastSweepingMethod);
    o.setFactoredEikonalEquationSolverRadius(radius);
    auto sw = std::make_unique<Sweeps3<T>>();
    sw->each([&](auto &s) {
        s.initialize(o, g);
        s.setSourceInformation(isx, isy, isz, static_cast<T>(xo), static_cast<T>(yo),
                               static_cast<T>(zo), sSrc);
    });
    return sw;
}

template <class T>
int solve3(int nx, int ny, int nz, double dx, double dy, double dz, int isx, int isy, int isz,
           double xo, double yo, double zo, const T *slow, int nSweeps, int radius,
           int doInitSweeps, T *tt) {
    try {
        const int ncx = nx - 1, ncy = ny - 1;
        const T sSrc = slow[static_cast<size_t>(isz) * ncx * ncy + static_cast<size_t>(isy) * ncx + isx];
        auto sw = setup3<T>(nx, ny, nz, dx, dy, dz, isx, isy, isz, xo, yo, zo, radius, sSrc);
        // src/solver3d.cpp:21-84
        std::fill(tt, tt + static_cast<size_t>(nx) * ny * nz, static_cast<T>(HUGE));
        for (int k = 0; k < 2; ++k)
            for (int j = 0; j < 2; ++j)
                for (int i = 0; i < 2; ++i) {
                    int ix = isx + i, iy = isy + j, iz = isz + k;
                    tt[gridToIndex(nx, ny, ix, iy, iz)] = computeAnalyticalTravelTime(
                        ix, iy, iz, static_cast<T>(dx), static_cast<T>(dy), static_cast<T>(dz),
                        static_cast<T>(xo), static_cast<T>(yo), static_cast<T>(zo), sSrc);
                }
        if (doInitSweeps)
            for (int e = 0; e < 8; ++e) sw->run(e, slow, tt, true);
        for (int k = 0; k < nSweeps; ++k)
            for (int e = 0; e < 8; ++e) sw->run(e, slow, tt, false);
    } catch (const std::exception &) {
        return -1;
    }
    return 0;
}

template <class T>
int sweep3(int e, int init, int nx, int ny, int nz, double dx, double dy, double dz, int isx,
           int isy, int isz, double xo, double yo, double zo, int radius, const T *slow, T *tt) {
    try {
        const int ncx = nx - 1, ncy = ny - 1;
        const T sSrc = slow[static_cast<size_t>(isz) * ncx * ncy + static_cast<size_t>(isy) * ncx + isx];
        auto sw = setup3<T>(nx, ny, nz, dx, dy, dz, isx, isy, isz, xo, yo, zo, radius, sSrc);
        sw->run(e, slow, tt, init != 0);
    } catch (const std::exception &) {
        return -1;
    }
    return 0;
}

template <class T>
struct Sweeps2 {
    Solver2DSweep<T, SweepNumber2D::Sweep1> s1;
    Solver2DSweep<T, SweepNumber2D::Sweep2> s2;
    Solver2DSweep<T, SweepNumber2D::Sweep3> s3;
    Solver2DSweep<T, SweepNumber2D::Sweep4> s4;
    template <class F> void each(F f) { f(s1); f(s2); f(s3); f(s4); }
    void run(int e, const T *slow, T *tt, bool init) {
        switch (e) {
            case 0: s1.updateFSM(slow, tt, init); break;
            case 1: s2.updateFSM(slow, tt, init); break;
            case 2: s3.updateFSM(slow, tt, init); break;
            default: s4.updateFSM(slow, tt, init); break;
        }
    }
};

template <class T>
int solve2(int nx, int nz, double dx, double dz, int isx, int isz, double xo, double zo,
           const T *slow, int nSweeps, int radius, int doInitSweeps, T *tt) {
    try {
        Geometry2D g;
        g.setNumberOfGridPointsInX(nx); g.setNumberOfGridPointsInZ(nz);
        g.setGridSpacingInX(dx); g.setGridSpacingInZ(dz);
        SolverOptions o;
        o.setAlgorithm(SolverAlgorithm::FastSweepingMethod);
        o.setFactoredEikonalEquationSolverRadius(radius);
        const T sSrc = slow[static_cast<size_t>(isz) * (nx - 1) + isx];
        auto sw = std::make_unique<Sweeps2<T>>();
        sw->each([&](auto &s) {
            s.initialize(g, o);
            s.setSourceInformation(isx, isz, static_cast<T>(xo), static_cast<T>(zo), sSrc);
        });
        // src/solver2d.cpp:61-105
        std::fill(tt, tt + static_cast<size_t>(nx) * nz, static_cast<T>(HUGE));
        for (int k = 0; k < 2; ++k)
            for (int i = 0; i < 2; ++i) {
                int ix = isx + i, iz = isz + k;
                tt[gridToIndex(nx, ix, iz)] = computeAnalyticalTravelTime(
                    ix, iz, static_cast<T>(dx), static_cast<T>(dz), static_cast<T>(xo),
                    static_cast<T>(zo), sSrc);
            }
        if (doInitSweeps)
            for (int e = 0; e < 4; ++e) sw->run(e, slow, tt, true);
        for (int k = 0; k < nSweeps; ++k)
            for (int e = 0; e < 4; ++e) sw->run(e, slow, tt, false);
    } catch (const std::exception &) {
        return -1;
    }
    return 0;
}

template <SweepNumber3D E>
int graph(int nx, int ny, int nz, int *levelStart, int *nodeToIndex, int *toX, int *toY,
          int *toZ, int *indexToLevel, int *maxLevelSize) {
    try {
        Graph3D<E> gr;
        gr.initialize(nx, ny, nz);
        const int nl = gr.getNumberOfLevels();
        const int n = gr.getNumberOfGridPoints();
        std::copy(gr.getLevelStartPointer(), gr.getLevelStartPointer() + nl + 1, levelStart);
        std::copy(gr.getNodeInLevelToIndexPointer(), gr.getNodeInLevelToIndexPointer() + n, nodeToIndex);
        std::copy(gr.getNodeInLevelToXGridPointPointer(), gr.getNodeInLevelToXGridPointPointer() + n, toX);
        std::copy(gr.getNodeInLevelToYGridPointPointer(), gr.getNodeInLevelToYGridPointPointer() + n, toY);
        std::copy(gr.getNodeInLevelToZGridPointPointer(), gr.getNodeInLevelToZGridPointPointer() + n, toZ);
        std::copy(gr.getIndexToLevelPointer(), gr.getIndexToLevelPointer() + n, indexToLevel);
        *maxLevelSize = gr.getMaximumLevelSize();
        return nl;
    } catch (const std::exception &) {
        return -1;
    }
}

}  // namespace

extern "C" {

int ref_solve3d_f64(int nx, int ny, int nz, double dx, double dy, double dz, int isx, int isy,
                    int isz, double xo, double yo, double zo, const double *slow, int nSweeps,
                    int radius, int doInitSweeps, double *tt) {
    return solve3<double>(nx, ny, nz, dx, dy, dz, isx, isy, isz, xo, yo, zo, slow, nSweeps, radius, doInitSweeps, tt);
}
int ref_solve3d_f32(int nx, int ny, int nz, double dx, double dy, double dz, int isx, int isy,
                    int isz, double xo, double yo, double zo, const float *slow, int nSweeps,
                    int radius, int doInitSweeps, float *tt) {
    return solve3<float>(nx, ny, nz, dx, dy, dz, isx, isy, isz, xo, yo, zo, slow, nSweeps, radius, doInitSweeps, tt);
}
int ref_sweep3d_f32(int e, int init, int nx, int ny, int nz, double dx, double dy, double dz,
                    int isx, int isy, int isz, double xo, double yo, double zo, int radius,
                    const float *slow, float *tt) {
    return sweep3<float>(e, init, nx, ny, nz, dx, dy, dz, isx, isy, isz, xo, yo, zo, radius, slow, tt);
}
int ref_sweep3d_f64(int e, int init, int nx, int ny, int nz, double dx, double dy, double dz,
                    int isx, int isy, int isz, double xo, double yo, double zo, int radius,
                    const double *slow, double *tt) {
    return sweep3<double>(e, init, nx, ny, nz, dx, dy, dz, isx, isy, isz, xo, yo, zo, radius, slow, tt);
}
int ref_solve2d_f64(int nx, int nz, double dx, double dz, int isx, int isz, double xo, double zo,
                    const double *slow, int nSweeps, int radius, int doInitSweeps, double *tt) {
    return solve2<double>(nx, nz, dx, dz, isx, isz, xo, zo, slow, nSweeps, radius, doInitSweeps, tt);
}
int ref_solve2d_f32(int nx, int nz, double dx, double dz, int isx, int isz, double xo, double zo,
                    const float *slow, int nSweeps, int radius, int doInitSweeps, float *tt) {
    return solve2<float>(nx, nz, dx, dz, isx, isz, xo, zo, slow, nSweeps, radius, doInitSweeps, tt);
}
int ref_graph3d(int e, int nx, int ny, int nz, int *levelStart, int *nodeToIndex, int *toX,
                int *toY, int *toZ, int *indexToLevel, int *maxLevelSize) {
    switch (e) {
        case 0: return graph<SweepNumber3D::Sweep1>(nx, ny, nz, levelStart, nodeToIndex, toX, toY, toZ, indexToLevel, maxLevelSize);
        case 1: return graph<SweepNumber3D::Sweep2>(nx, ny, nz, levelStart, nodeToIndex, toX, toY, toZ, indexToLevel, maxLevelSize);
        case 2: return graph<SweepNumber3D::Sweep3>(nx, ny, nz, levelStart, nodeToIndex, toX, toY, toZ, indexToLevel, maxLevelSize);
        case 3: return graph<SweepNumber3D::Sweep4>(nx, ny, nz, levelStart, nodeToIndex, toX, toY, toZ, indexToLevel, maxLevelSize);
        case 4: return graph<SweepNumber3D::Sweep5>(nx, ny, nz, levelStart, nodeToIndex, toX, toY, toZ, indexToLevel, maxLevelSize);
        case 5: return graph<SweepNumber3D::Sweep6>(nx, ny, nz, levelStart, nodeToIndex, toX, toY, toZ, indexToLevel, maxLevelSize);
        case 6: return graph<SweepNumber3D::Sweep7>(nx, ny, nz, levelStart, nodeToIndex, toX, toY, toZ, indexToLevel, maxLevelSize);
        default: return graph<SweepNumber3D::Sweep8>(nx, ny, nz, levelStart, nodeToIndex, toX, toY, toZ, indexToLevel, maxLevelSize);
    }
}

}  // extern "C"
