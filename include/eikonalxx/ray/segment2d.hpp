// A straight piece of a 2D ray path with the slowness it travels in (drop-in for
// include/eikonalxx/ray/segment2d.hpp of the reference).
#ifndef EIKONALXX_RAY_SEGMENT_2D_HPP
#define EIKONALXX_RAY_SEGMENT_2D_HPP
#include <memory>
#include <ostream>
#include <utility>
namespace EikonalXX::Ray
{
class Point2D;
class Segment2D
{
public:
    Segment2D();
    Segment2D(const Segment2D &segment);
    Segment2D(Segment2D &&segment) noexcept;
    Segment2D &operator=(const Segment2D &segment);
    Segment2D &operator=(Segment2D &&segment) noexcept;
    ~Segment2D();
    /// std::invalid_argument when a point lacks a coordinate.
    void setStartAndEndPoint(const std::pair<Point2D, Point2D> &startAndEndPoint);
    [[nodiscard]] Point2D getStartPoint() const;
    [[nodiscard]] Point2D getEndPoint() const;
    [[nodiscard]] bool haveStartAndEndPoint() const noexcept;
    void reverse();
    [[nodiscard]] double getLength() const;
    void setVelocity(double velocity);    // std::runtime_error unless positive
    void setSlowness(double slowness);
    [[nodiscard]] double getVelocity() const;
    [[nodiscard]] double getSlowness() const;
    [[nodiscard]] bool haveVelocity() const noexcept;
    [[nodiscard]] double getTravelTime() const;   // slowness x length
    void setVelocityModelCellIndex(int index);
    [[nodiscard]] int getVelocityModelCellIndex() const;
    [[nodiscard]] bool haveVelocityModelCellIndex() const noexcept;
    void clear() noexcept;
private:
    friend void swap(Segment2D &lhs, Segment2D &rhs) noexcept;
    class Segment2DImpl;
    std::unique_ptr<Segment2DImpl> pImpl;
};
void swap(Segment2D &lhs, Segment2D &rhs) noexcept;
std::ostream &operator<<(std::ostream &os, const Segment2D &segment);
}
#endif
