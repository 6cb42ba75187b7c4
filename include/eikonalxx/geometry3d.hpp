// 3D node-based grid geometry (drop-in for include/eikonalxx/geometry3d.hpp of the
// reference): at least 3 grid points and a positive spacing per axis; cells are the
// (n - 1) intervals between nodes; the origin defaults to 0.
#ifndef EIKONALXX_GEOMETRY_3D_HPP
#define EIKONALXX_GEOMETRY_3D_HPP
#include <memory>
namespace EikonalXX
{
class Geometry3D
{
public:
    Geometry3D();
    Geometry3D(const Geometry3D &geometry);
    Geometry3D(Geometry3D &&geometry) noexcept;
    Geometry3D& operator=(const Geometry3D &geometry);
    Geometry3D& operator=(Geometry3D &&geometry) noexcept;
    ~Geometry3D();
    void setNumberOfGridPointsInX(int nx);
    [[nodiscard]] int getNumberOfGridPointsInX() const;
    [[nodiscard]] int getNumberOfCellsInX() const;
    [[nodiscard]] bool haveNumberOfGridPointsInX() const noexcept;
    void setGridSpacingInX(double dx);
    [[nodiscard]] double getGridSpacingInX() const;
    [[nodiscard]] bool haveGridSpacingInX() const noexcept;
    void setOriginInX(double x0) noexcept;
    [[nodiscard]] double getOriginInX() const noexcept;
    void setNumberOfGridPointsInY(int ny);
    [[nodiscard]] int getNumberOfGridPointsInY() const;
    [[nodiscard]] int getNumberOfCellsInY() const;
    [[nodiscard]] bool haveNumberOfGridPointsInY() const noexcept;
    void setGridSpacingInY(double dy);
    [[nodiscard]] double getGridSpacingInY() const;
    [[nodiscard]] bool haveGridSpacingInY() const noexcept;
    void setOriginInY(double y0) noexcept;
    [[nodiscard]] double getOriginInY() const noexcept;
    void setNumberOfGridPointsInZ(int nz);
    [[nodiscard]] int getNumberOfGridPointsInZ() const;
    [[nodiscard]] int getNumberOfCellsInZ() const;
    [[nodiscard]] bool haveNumberOfGridPointsInZ() const noexcept;
    void setGridSpacingInZ(double dz);
    [[nodiscard]] double getGridSpacingInZ() const;
    [[nodiscard]] bool haveGridSpacingInZ() const noexcept;
    void setOriginInZ(double z0) noexcept;
    [[nodiscard]] double getOriginInZ() const noexcept;
    [[nodiscard]] int getNumberOfGridPoints() const;
    [[nodiscard]] int getNumberOfCells() const;
    void clear() noexcept;
private:
    class Geometry3DImpl;
    std::unique_ptr<Geometry3DImpl> pImpl;
};
/// Same grid: same point counts, spacings within 1e-8 m and origins within 1e-7 m.
bool operator==(const Geometry3D &lhs, const Geometry3D &rhs);
bool operator!=(const Geometry3D &lhs, const Geometry3D &rhs);
}
#endif
