// 2D node-based grid geometry (drop-in for include/eikonalxx/geometry2d.hpp of the
// reference): at least 3 grid points and a positive spacing per axis; cells are the
// (n - 1) intervals between nodes; the origin defaults to 0.
#ifndef EIKONALXX_GEOMETRY_2D_HPP
#define EIKONALXX_GEOMETRY_2D_HPP
#include <memory>
namespace EikonalXX
{
class Geometry2D
{
public:
    Geometry2D();
    Geometry2D(const Geometry2D &geometry);
    Geometry2D(Geometry2D &&geometry) noexcept;
    Geometry2D& operator=(const Geometry2D &geometry);
    Geometry2D& operator=(Geometry2D &&geometry) noexcept;
    ~Geometry2D();
    void setNumberOfGridPointsInX(int nx);
    [[nodiscard]] int getNumberOfGridPointsInX() const;
    [[nodiscard]] int getNumberOfCellsInX() const;
    [[nodiscard]] bool haveNumberOfGridPointsInX() const noexcept;
    void setGridSpacingInX(double dx);
    [[nodiscard]] double getGridSpacingInX() const;
    [[nodiscard]] bool haveGridSpacingInX() const noexcept;
    void setOriginInX(double x0) noexcept;
    [[nodiscard]] double getOriginInX() const noexcept;
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
    class Geometry2DImpl;
    std::unique_ptr<Geometry2DImpl> pImpl;
};
/// Same grid: same point counts, spacings within 1e-8 m and origins within 1e-7 m.
bool operator==(const Geometry2D &lhs, const Geometry2D &rhs);
bool operator!=(const Geometry2D &lhs, const Geometry2D &rhs);
}
#endif
