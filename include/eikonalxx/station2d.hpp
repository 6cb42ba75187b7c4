// A receiver in a 2D grid (drop-in for include/eikonalxx/station2d.hpp of the
// reference).  A location must lie inside the grid; its offset is location - origin and
// its cell min(nCell - 1, int(offset / spacing)) on each axis.
#ifndef EIKONALXX_STATION_2D_HPP
#define EIKONALXX_STATION_2D_HPP
#include <memory>
#include <ostream>
#include <string>
namespace EikonalXX
{
class Geometry2D;
class Station2D
{
public:
    Station2D();
    Station2D(const Station2D &other);
    Station2D(Station2D &&other) noexcept;
    Station2D& operator=(const Station2D &other);
    Station2D& operator=(Station2D &&other) noexcept;
    ~Station2D();
    void setGeometry(const Geometry2D &geometry);
    [[nodiscard]] Geometry2D getGeometry() const;
    [[nodiscard]] bool haveGeometry() const noexcept;
    void setName(const std::string &name) noexcept;
    [[nodiscard]] std::string getName() const noexcept;
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
    class Station2DImpl;
    std::unique_ptr<Station2DImpl> pImpl;
};
std::ostream& operator<<(std::ostream &os, const Station2D &station);
}
#endif
