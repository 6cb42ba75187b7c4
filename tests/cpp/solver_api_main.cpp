// Drives the C++ drop-in API (Solver3D, Solver2D) the way a user of the reference would
// and writes the travel-time fields as raw binary for the Python test to compare
// against the oracle.  Usage: solver_api <outdir>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <random>
#include <string>
#include <vector>
#include "eikonalxx/geometry2d.hpp"
#include "eikonalxx/geometry3d.hpp"
#include "eikonalxx/model2d.hpp"
#include "eikonalxx/model3d.hpp"
#include "eikonalxx/solver2d.hpp"
#include "eikonalxx/solver3d.hpp"
#include "eikonalxx/solverOptions.hpp"
#include "eikonalxx/source3d.hpp"
#include "eikonalxx/station2d.hpp"

using namespace EikonalXX;

template <class T> void dump(const std::string &path, const std::vector<T> &v)
{
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char *>(v.data()), v.size() * sizeof(T));
}

template <class T> int run3(const std::string &out)
{
    const int nx = 21, ny = 17, nz = 13;
    Geometry3D g;
    g.setNumberOfGridPointsInX(nx); g.setNumberOfGridPointsInY(ny); g.setNumberOfGridPointsInZ(nz);
    g.setGridSpacingInX(50); g.setGridSpacingInY(50); g.setGridSpacingInZ(50);
    std::mt19937 rng(7);
    std::uniform_real_distribution<double> u(2500, 5500);
    std::vector<T> v(static_cast<size_t>(nx) * ny * nz);
    for (auto &x : v) x = static_cast<T>(u(rng));
    Model3D<T> m;
    m.initialize(g);
    m.setNodalVelocities(static_cast<int>(v.size()), v.data(), Ordering3D::Natural);
    SolverOptions o;
    o.setNumberOfSweeps(2);
    o.setConvergenceTolerance(0);
    o.setFactoredEikonalEquationSolverRadius(3);
    Solver3D<T> s;
    s.initialize(o, g);
    s.setVelocityModel(m);
    s.setSource(std::make_tuple(333.0, 421.0, 222.0));
    s.solve();
    dump(out + "/v3_" + std::to_string(sizeof(T)) + ".bin", v);
    dump(out + "/s3_" + std::to_string(sizeof(T)) + ".bin", m.getSlowness());
    dump(out + "/t3_" + std::to_string(sizeof(T)) + ".bin", s.getTravelTimeField());
    // the reference's error semantics
    bool threw = false;
    try { s.setSource(std::make_tuple(1e6, 0.0, 0.0)); } catch (const std::invalid_argument &) { threw = true; }
    if (!threw) { std::cerr << "out-of-range source did not throw" << std::endl; return 1; }
    Solver3D<T> empty;
    threw = false;
    try { empty.solve(); } catch (const std::runtime_error &) { threw = true; }
    if (!threw) { std::cerr << "solve before initialize did not throw" << std::endl; return 1; }
    return 0;
}

int run2(const std::string &out)
{
    const int nx = 61, nz = 37;
    Geometry2D g;
    g.setNumberOfGridPointsInX(nx); g.setNumberOfGridPointsInZ(nz);
    g.setGridSpacingInX(10); g.setGridSpacingInZ(10);
    std::vector<double> v(static_cast<size_t>(nx) * nz);
    for (int iz = 0; iz < nz; ++iz)
        for (int ix = 0; ix < nx; ++ix) v[iz * nx + ix] = 3000 + 0.5 * (iz * 10.0);
    Model2D<double> m;
    m.initialize(g);
    m.setNodalVelocities(nx * nz, v.data(), Ordering2D::Natural);
    SolverOptions o;
    o.setNumberOfSweeps(2);
    o.setConvergenceTolerance(0);
    Solver2D<double> s;
    s.initialize(o, g);
    s.setVelocityModel(m);
    s.setSource(std::make_pair(250.0, 130.0));
    std::vector<Station2D> st(2);
    st[0].setGeometry(g); st[0].setLocationInX(455.5); st[0].setLocationInZ(301.25);
    st[1].setGeometry(g); st[1].setLocationInX(251.0); st[1].setLocationInZ(131.0);   // in the source cell
    s.setStations(st);
    s.solve();
    s.computeTravelTimeGradientField();
    dump(out + "/s2.bin", m.getSlowness());
    dump(out + "/t2.bin", s.getTravelTimeField());
    dump(out + "/st2.bin", s.getTravelTimesAtStations());
    dump(out + "/g2.bin", s.getTravelTimeGradientField());
    s.writeVTK(out + "/t2.vtk", "travel time", true);   // src/solver2d.cpp:946-964
    return 0;
}

int main(int argc, char **argv)
{
    if (argc < 2) return 2;
    const std::string out = argv[1];
    try {
        if (run3<float>(out) || run3<double>(out) || run2(out)) return 1;
    } catch (const std::exception &e) {
        std::cerr << "error: " << e.what() << std::endl;
        return 1;
    }
    std::cout << "solver api ok" << std::endl;
    return 0;
}
