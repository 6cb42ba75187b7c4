#ifndef EIKONALXX_IO_VTK_RECTILINEAR_GRID_3D_HPP
#define EIKONALXX_IO_VTK_RECTILINEAR_GRID_3D_HPP
// Legacy-VTK rectilinear-grid writer of 3D nodal and cellular datasets, the drop-in for
// EikonalXX::IO::VTKRectilinearGrid3D (include/eikonalxx/io/vtkRectilinearGrid3d.hpp of
// the reference, src/io/vtkRectilinearGrid3d.cpp).  Files: "# vtk DataFile Version 3.0",
// the title with blanks as underscores, BINARY (big-endian float32) or ASCII, DATASET
// RECTILINEAR_GRID with x, y and z coordinates (z written as -depth), then POINT_DATA
// and CELL_DATA sections of SCALARS, each with "LOOKUP_TABLE default".
#include <memory>
#include <string>
#include "eikonalxx/enums.hpp"

namespace EikonalXX {
class Geometry3D;
}

namespace EikonalXX::IO {

class VTKRectilinearGrid3D {
public:
    VTKRectilinearGrid3D();
    ~VTKRectilinearGrid3D();
    /// Opens (truncates) fileName, making its directory if needed, and writes the grid.
    /// Throws std::invalid_argument if the geometry is incomplete, std::runtime_error if
    /// the file cannot be opened.
    void open(const std::string &fileName, const Geometry3D &geometry, const std::string &title = "traveltimes",
              bool writeBinary = true);
    [[nodiscard]] bool isOpen() const noexcept;
    /// nx*ny*nz values (float or double, written as float) in the given order.
    template <typename T>
    void writeNodalDataset(const std::string &name, const T *data, Ordering3D ordering = Ordering3D::Natural) const;
    /// (nx-1)*(ny-1)*(nz-1) values in the given order.
    template <typename T>
    void writeCellularDataset(const std::string &name, const T *data,
                              Ordering3D ordering = Ordering3D::Natural) const;
    void close() noexcept;
    VTKRectilinearGrid3D(const VTKRectilinearGrid3D &) = delete;
    VTKRectilinearGrid3D(VTKRectilinearGrid3D &&) noexcept = delete;
    VTKRectilinearGrid3D &operator=(const VTKRectilinearGrid3D &) = delete;
    VTKRectilinearGrid3D &operator=(VTKRectilinearGrid3D &&) noexcept = delete;

private:
    class VTKRectilinearGrid3DImpl;
    std::unique_ptr<VTKRectilinearGrid3DImpl> pImpl;
};

}  // namespace EikonalXX::IO
#endif
