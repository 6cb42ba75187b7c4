// A point source in a 2D grid (drop-in for include/eikonalxx/source2d.hpp of the
// reference).  A location must lie inside the grid; its offset is location - origin and
// its cell min(nCell - 1, int(offset / spacing)) on each axis.
#ifndef EIKONALXX_SOURCE_2D_HPP
#define EIKONALXX_SOURCE_2D_HPP
#include <memory>
#include <ostream>
#include <string>
namespace EikonalXX
{
class Geometry2D;
class Source2D
{
public:
    Source2D();
    Source2D(const Source2D &other);
    Source2D(Source2D &&other) noexcept;
    Source2D& operator=(const Source2D &other);
    Source2D& operator=(Source2D &&other) noexcept;
    ~Source2D();
    void setGeometry(const Geometry2D &geometry);
    [[nodiscard]] Geometry2D getGeometry() const;
    [[nodiscard]] bool haveGeometry() const noexcept;
    void setLocationInX(double x);
    [[nodiscard]] double getLocationInX() const;
    [[nodiscard]] double getOffsetInX() const;
    [[nodiscard]] int getCellInX() const;
    [[nodiscard]] bool haveLocationInX() const noexcept;
    void setLocationInZ(double z);
    [[nodiscard]] double getLocationInZ() const;
    [[nodiscard]] double getOffsetInZ() const;
    [[nodiscard]] int getCellInZ() const;
    [[nodiscard]] bool haveLocationInZ() const noexcept;
    void setZToFreeSurface();
    [[nodiscard]] int getCell() const;
    void clear() noexcept;
private:
    class Source2DImpl;
    std::unique_ptr<Source2DImpl> pImpl;
};
std::ostream& operator<<(std::ostream &os, const Source2D &source);
}
#endif
