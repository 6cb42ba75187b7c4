// A point of a 2D ray path (drop-in for include/eikonalxx/ray/point2d.hpp of the reference).
#ifndef EIKONALXX_RAY_POINT_2D_HPP
#define EIKONALXX_RAY_POINT_2D_HPP
#include <memory>
namespace EikonalXX::Ray
{
class Point2D
{
public:
    Point2D();
    Point2D(double x, double z);
    Point2D(const Point2D &point);
    Point2D(Point2D &&point) noexcept;
    Point2D &operator=(const Point2D &point);
    Point2D &operator=(Point2D &&point) noexcept;
    ~Point2D();
    void setPositionInX(double x) noexcept;
    [[nodiscard]] double getPositionInX() const;   // std::runtime_error when not set
    [[nodiscard]] bool havePositionInX() const noexcept;
    void setPositionInZ(double z) noexcept;
    [[nodiscard]] double getPositionInZ() const;
    [[nodiscard]] bool havePositionInZ() const noexcept;
    void clear() noexcept;
private:
    class Point2DImpl;
    std::unique_ptr<Point2DImpl> pImpl;
};
}
#endif
