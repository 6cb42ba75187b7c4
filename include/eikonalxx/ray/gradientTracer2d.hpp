// Rays from stations to the source down a 2D travel-time gradient (drop-in for
// include/eikonalxx/ray/gradientTracer2d.hpp of the reference).  trace() runs on the GPU
// through eikx_trace_rays2d (include/eikx/eikx_c.h), one thread per station.
#ifndef EIKONALXX_RAY_GRADIENT_TRACER_2D_HPP
#define EIKONALXX_RAY_GRADIENT_TRACER_2D_HPP
#include <memory>
#include <string>
#include <vector>
#include "eikonalxx/abstractBaseClass/solver2d.hpp"
namespace EikonalXX
{
class Geometry2D;
class Station2D;
}
namespace EikonalXX::Ray
{
class GradientTracerOptions;
class Path2D;
class GradientTracer2D
{
public:
    GradientTracer2D();
    GradientTracer2D(const GradientTracer2D &tracer);
    GradientTracer2D(GradientTracer2D &&tracer) noexcept;
    GradientTracer2D &operator=(const GradientTracer2D &tracer);
    GradientTracer2D &operator=(GradientTracer2D &&tracer) noexcept;
    ~GradientTracer2D();
    void initialize(const GradientTracerOptions &options, const EikonalXX::Geometry2D &geometry);
    [[nodiscard]] bool isInitialized() const noexcept;
    void setStations(const std::vector<EikonalXX::Station2D> &stations);
    [[nodiscard]] bool haveStations() const noexcept;
    /// One path per station, source to station; a station whose ray does not reach the
    /// source gets an empty path and a message on std::cerr, as the reference prints.
    template <typename T> void trace(const EikonalXX::AbstractBaseClass::ISolver2D<T> &solver);
    [[nodiscard]] bool haveRayPaths() const noexcept;
    [[nodiscard]] std::vector<Path2D> getRayPaths() const;
    /// Writes the ray paths as ASCII legacy-VTK polylines (IO::VTKLines2D).  Throws
    /// std::runtime_error if no paths have been traced.
    void writeVTK(const std::string &fileName, const std::string &title = "ray_paths");
private:
    class GradientTracer2DImpl;
    std::unique_ptr<GradientTracer2DImpl> pImpl;
};
}
#endif
