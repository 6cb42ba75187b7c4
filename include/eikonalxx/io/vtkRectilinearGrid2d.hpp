#ifndef EIKONALXX_IO_VTK_RECTILINEAR_GRID_2D_HPP
#define EIKONALXX_IO_VTK_RECTILINEAR_GRID_2D_HPP
// Legacy-VTK rectilinear-grid writer of 2D nodal, nodal-vector and cellular datasets,
// the drop-in for EikonalXX::IO::VTKRectilinearGrid2D (the reference's
// include/eikonalxx/io/vtkRectilinearGrid2d.hpp, src/io/vtkRectilinearGrid2d.cpp).  The
// grid is written with one y coordinate (0); vectors (x, z) as (x, 0, z).
#include <memory>
#include <string>
#include "eikonalxx/enums.hpp"

namespace EikonalXX {
class Geometry2D;
}

namespace EikonalXX::IO {

class VTKRectilinearGrid2D {
public:
    VTKRectilinearGrid2D();
    ~VTKRectilinearGrid2D();
    void open(const std::string &fileName, const Geometry2D &geometry, const std::string &title = "traveltimes",
              bool writeBinary = true);
    [[nodiscard]] bool isOpen() const noexcept;
    /// nx*nz values.
    template <typename T>
    void writeNodalDataset(const std::string &name, const T *data, Ordering2D ordering = Ordering2D::Natural) const;
    /// 2*nx*nz values, (d/dx, d/dz) per node.
    template <typename T>
    void writeNodalVectorDataset(const std::string &name, const T *data,
                                 Ordering2D ordering = Ordering2D::Natural) const;
    /// (nx-1)*(nz-1) values.
    template <typename T>
    void writeCellularDataset(const std::string &name, const T *data,
                              Ordering2D ordering = Ordering2D::Natural) const;
    void close() noexcept;
    VTKRectilinearGrid2D(const VTKRectilinearGrid2D &) = delete;
    VTKRectilinearGrid2D(VTKRectilinearGrid2D &&) noexcept = delete;
    VTKRectilinearGrid2D &operator=(const VTKRectilinearGrid2D &) = delete;
    VTKRectilinearGrid2D &operator=(VTKRectilinearGrid2D &&) noexcept = delete;

private:
    class VTKRectilinearGrid2DImpl;
    std::unique_ptr<VTKRectilinearGrid2DImpl> pImpl;
};

}  // namespace EikonalXX::IO
#endif
