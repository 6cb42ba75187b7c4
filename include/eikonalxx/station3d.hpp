// A receiver in a 3D grid (drop-in for include/eikonalxx/station3d.hpp of the
// reference).  A location must lie inside the grid; its offset is location - origin and
// its cell min(nCell - 1, int(offset / spacing)) on each axis.
#ifndef EIKONALXX_STATION_3D_HPP
#define EIKONALXX_STATION_3D_HPP
#include <memory>
#include <ostream>
#include <string>
namespace EikonalXX
{
class Geometry3D;
class Station3D
{
public:
    Station3D();
    Station3D(const Station3D &other);
    Station3D(Station3D &&other) noexcept;
    Station3D& operator=(const Station3D &other);
    Station3D& operator=(Station3D &&other) noexcept;
    ~Station3D();
    void setGeometry(const Geometry3D &geometry);
    [[nodiscard]] Geometry3D getGeometry() const;
    [[nodiscard]] bool haveGeometry() const noexcept;
    void setName(const std::string &name) noexcept;
    [[nodiscard]] std::string getName() const noexcept;
    void setLocationInX(double x);
    [[nodiscard]] double getLocationInX() const;
    [[nodiscard]] double getOffsetInX() const;
    [[nodiscard]] int getCellInX() const;
    [[nodiscard]] bool haveLocationInX() const noexcept;
    void setLocationInY(double y);
    [[nodiscard]] double getLocationInY() const;
    [[nodiscard]] double getOffsetInY() const;
    [[nodiscard]] int getCellInY() const;
    [[nodiscard]] bool haveLocationInY() const noexcept;
    void setLocationInZ(double z);
    [[nodiscard]] double getLocationInZ() const;
    [[nodiscard]] double getOffsetInZ() const;
    [[nodiscard]] int getCellInZ() const;
    [[nodiscard]] bool haveLocationInZ() const noexcept;
    void setZToFreeSurface();
    [[nodiscard]] int getCell() const;
    void clear() noexcept;
private:
    class Station3DImpl;
    std::unique_ptr<Station3DImpl> pImpl;
};
std::ostream& operator<<(std::ostream &os, const Station3D &station);
}
#endif
