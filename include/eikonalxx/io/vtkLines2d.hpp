#ifndef EIKONALXX_IO_VTK_LINES_2D_HPP
#define EIKONALXX_IO_VTK_LINES_2D_HPP
// Legacy-VTK polyline writer of 2D ray paths, the drop-in for EikonalXX::IO::VTKLines2D
// (the reference's include/eikonalxx/io/vtkLines2d.hpp, src/io/vtkLines2d.cpp): ASCII
// DATASET POLYDATA, points (x, 0, -z), one LINES entry per path.
#include <memory>
#include <string>
#include <utility>
#include <vector>
#include "eikonalxx/enums.hpp"

namespace EikonalXX {
class Geometry2D;
}

namespace EikonalXX::IO {

class VTKLines2D {
public:
    VTKLines2D();
    ~VTKLines2D();
    void open(const std::string &fileName, const EikonalXX::Geometry2D &geometry,
              const std::string &title = "ray_paths");
    [[nodiscard]] bool isOpen() const noexcept;
    /// One polyline per path: its (x, z) points in metres.  Throws std::runtime_error if
    /// the file is not open.
    void write(const std::vector<std::vector<std::pair<double, double>>> &polygons) const;
    void close() noexcept;
    VTKLines2D(const VTKLines2D &) = delete;
    VTKLines2D(VTKLines2D &&) noexcept = delete;
    VTKLines2D &operator=(const VTKLines2D &) = delete;
    VTKLines2D &operator=(VTKLines2D &&) noexcept = delete;

private:
    class VTKLines2DImpl;
    std::unique_ptr<VTKLines2DImpl> pImpl;
};

}  // namespace EikonalXX::IO
#endif
