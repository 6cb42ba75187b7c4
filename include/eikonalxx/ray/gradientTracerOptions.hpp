// Step rule of the gradient ray tracer (drop-in for
// include/eikonalxx/ray/gradientTracerOptions.hpp of the reference): within radius r cells
// of the source the ray steps scale x min(dx, dz).
#ifndef EIKONALXX_RAY_GRADIENT_TRACER_OPTIONS_HPP
#define EIKONALXX_RAY_GRADIENT_TRACER_OPTIONS_HPP
#include <memory>
#include <utility>
#include <vector>
namespace EikonalXX::Ray
{
class GradientTracerOptions
{
public:
    GradientTracerOptions();
    GradientTracerOptions(const GradientTracerOptions &options);
    GradientTracerOptions(GradientTracerOptions &&options) noexcept;
    GradientTracerOptions &operator=(const GradientTracerOptions &options);
    GradientTracerOptions &operator=(GradientTracerOptions &&options) noexcept;
    ~GradientTracerOptions();
    /// (radius, scale) pairs: radii non-negative and distinct, scales in (eps, 1); they are
    /// sorted by radius and a pair (INT_MAX, last scale) is added if missing.
    /// std::invalid_argument otherwise.
    void setRadiusScaleFactor(const std::vector<std::pair<int, double>> &radiusScaleFactor);
    [[nodiscard]] std::vector<std::pair<int, double>> getRadiusScaleFactor() const noexcept;
    void clear() noexcept;
private:
    class GradientTracerOptionsImpl;
    std::unique_ptr<GradientTracerOptionsImpl> pImpl;
};
}
#endif
