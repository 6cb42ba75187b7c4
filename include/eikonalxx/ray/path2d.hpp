// A 2D ray path: segments joined end to start, with its travel time and length (drop-in
// for include/eikonalxx/ray/path2d.hpp of the reference).
#ifndef EIKONALXX_RAY_PATH_2D_HPP
#define EIKONALXX_RAY_PATH_2D_HPP
#include <memory>
#include <vector>
#include "eikonalxx/ray/segment2d.hpp"
namespace EikonalXX::Ray
{
class Path2D
{
private:
    using PathType = std::vector<Segment2D>;
public:
    using iterator = typename PathType::iterator;
    using const_iterator = typename PathType::const_iterator;
    Path2D();
    Path2D(const Path2D &path);
    Path2D(Path2D &&path) noexcept;
    Path2D &operator=(const Path2D &path);
    Path2D &operator=(Path2D &&path) noexcept;
    ~Path2D();
    void open();
    [[nodiscard]] bool isOpen() const noexcept;
    /// std::invalid_argument when the segment lacks points or velocity, or does not start
    /// at the previous segment's end point.
    void append(const Segment2D &segment);
    void append(Segment2D &&segment);
    void close();
    void set(const std::vector<Segment2D> &segments);
    void set(std::vector<Segment2D> &&segments);
    void reverse();
    [[nodiscard]] bool empty() const noexcept;
    [[nodiscard]] size_t size() const noexcept;
    [[nodiscard]] double getTravelTime() const;
    [[nodiscard]] double getLength() const;
    /// Degrees from the +z axis of the first segment of non-zero length.
    [[nodiscard]] double getTakeOffAngle() const;
    void clear() noexcept;
    iterator begin();
    const_iterator begin() const noexcept;
    const_iterator cbegin() const noexcept;
    iterator end();
    const_iterator end() const noexcept;
    const_iterator cend() const noexcept;
    Segment2D &at(size_t index);
    const Segment2D &at(size_t index) const;
private:
    class Path2DImpl;
    std::unique_ptr<Path2DImpl> pImpl;
};
}
#endif
