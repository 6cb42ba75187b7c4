// CPU driver of the C++ legacy-VTK writers (tests/test_vtk_cpp.py parses what it writes):
// Model3D/Model2D::writeVTK and the IO::VTKRectilinearGrid3D/2D and IO::VTKLines2D
// classes, binary and ASCII, natural and transposed orderings.  No GPU.
//   vtk_main <directory>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>
#include "eikonalxx/geometry2d.hpp"
#include "eikonalxx/geometry3d.hpp"
#include "eikonalxx/io/vtkLines2d.hpp"
#include "eikonalxx/io/vtkRectilinearGrid2d.hpp"
#include "eikonalxx/io/vtkRectilinearGrid3d.hpp"
#include "eikonalxx/model2d.hpp"
#include "eikonalxx/model3d.hpp"

using namespace EikonalXX;

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    const std::string dir = argv[1];
    const int nx = 5, ny = 4, nz = 3;
    Geometry3D g3;
    g3.setNumberOfGridPointsInX(nx); g3.setNumberOfGridPointsInY(ny); g3.setNumberOfGridPointsInZ(nz);
    g3.setGridSpacingInX(10); g3.setGridSpacingInY(20); g3.setGridSpacingInZ(25);
    g3.setOriginInX(100); g3.setOriginInY(-50); g3.setOriginInZ(5);
    // cell velocities v = 3000 + 10 * natural cell index
    const int nc3 = (nx - 1) * (ny - 1) * (nz - 1);
    std::vector<double> vc(nc3);
    for (int i = 0; i < nc3; ++i) vc[i] = 3000 + 10.0 * i;
    Model3D<double> m3;
    m3.initialize(g3);
    m3.setCellularVelocities(nc3, vc.data(), Ordering3D::Natural);
    m3.writeVTK(dir + "/sub/model3d.vtk", "velocity m/s");       // a directory the writer makes
    // nodal dataset t = natural node index, given in XYZ order (z fastest)
    std::vector<float> tXYZ(static_cast<size_t>(nx) * ny * nz);
    for (int ix = 0; ix < nx; ++ix)
        for (int iy = 0; iy < ny; ++iy)
            for (int iz = 0; iz < nz; ++iz) tXYZ[(ix * ny + iy) * nz + iz] = static_cast<float>((iz * ny + iy) * nx + ix);
    for (const bool binary : {true, false}) {
        IO::VTKRectilinearGrid3D w;
        w.open(dir + (binary ? "/grid3d_bin.vtk" : "/grid3d_ascii.vtk"), g3, "", binary);
        w.writeNodalDataset("index", tXYZ.data(), Ordering3D::XYZ);
        w.writeNodalDataset<double>("twice", std::vector<double>(tXYZ.size(), 2.5).data());
        w.writeCellularDataset("cells", vc.data());
        w.close();
        if (w.isOpen()) return 3;
    }
    // 2D
    const int mx = 6, mz = 4;
    Geometry2D g2;
    g2.setNumberOfGridPointsInX(mx); g2.setNumberOfGridPointsInZ(mz);
    g2.setGridSpacingInX(5); g2.setGridSpacingInZ(7.5);
    g2.setOriginInX(1); g2.setOriginInZ(2);
    const int nc2 = (mx - 1) * (mz - 1);
    std::vector<float> vc2(nc2);
    for (int i = 0; i < nc2; ++i) vc2[i] = 2000 + 100.0f * i;
    Model2D<float> m2;
    m2.initialize(g2);
    m2.setCellularVelocities(nc2, vc2.data(), Ordering2D::Natural);
    m2.writeVTK(dir + "/model2d.vtk");
    std::vector<double> grad(2 * static_cast<size_t>(mx) * mz);
    for (int i = 0; i < mx * mz; ++i) {
        grad[2 * i] = 0.5 * i;
        grad[2 * i + 1] = -0.25 * i;
    }
    {
        IO::VTKRectilinearGrid2D w;
        w.open(dir + "/grid2d.vtk", g2, "two d", true);
        std::vector<double> t(static_cast<size_t>(mx) * mz);
        for (int i = 0; i < mx * mz; ++i) t[i] = 0.001 * i;
        w.writeNodalDataset("t", t.data());
        w.writeNodalVectorDataset("t gradient", grad.data());
        w.writeCellularDataset("v", vc2.data());
        w.close();
    }
    {
        IO::VTKLines2D w;
        w.open(dir + "/rays.vtk", g2);
        w.write({{{0.0, 10.0}, {5.0, 12.5}, {7.5, 20.0}}, {{1.0, 2.0}, {3.0, 4.0}}});
        w.close();
    }
    // a model without velocities cannot be written
    try {
        Model3D<float> empty;
        empty.initialize(g3);
        empty.writeVTK(dir + "/never.vtk");
        return 4;
    } catch (const std::runtime_error &) {
    }
    std::printf("vtk ok\n");
    return 0;
}
