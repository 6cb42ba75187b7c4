// 3D eikonal solver (drop-in for include/eikonalxx/solver3d.hpp:20-178 of the reference).
//
// Workflow: initialize(options, geometry) -> setVelocityModel(model) -> setSource(...)
// -> solve() -> getTravelTimeField().  The solve runs on the GPU (device 0, or the
// index in the EIKX_DEVICE environment variable) through the C ABI of
// include/eikx/eikx_c.h: travel times initialised at the 8 corners of the source cell,
// one source-limited pass of the 8 sweeps, then up to getNumberOfSweeps() iterations of
// the 8 sweeps, stopping once each of the last 8 sweeps decreased no travel time by the
// convergence tolerance or more.  Solver3D<float> sweeps in FP32, Solver3D<double> in FP64.
// Errors are std::invalid_argument (bad input) and std::runtime_error (wrong order of
// calls, GPU failure), as the reference throws.  Not thread-safe.
#ifndef EIKONALXX_SOLVER_3D_HPP
#define EIKONALXX_SOLVER_3D_HPP
#include <memory>
#include <tuple>
#include <vector>
#include "eikonalxx/abstractBaseClass/solver3d.hpp"
namespace EikonalXX
{
class Geometry3D;
template<class T> class Model3D;
class Source3D;
class SolverOptions;
class Station3D;
template<class T>
class Solver3D : public EikonalXX::AbstractBaseClass::ISolver3D<T>
{
public:
    Solver3D();
    ~Solver3D() override;
    void initialize(const SolverOptions &options, const Geometry3D &geometry);
    [[nodiscard]] SolverOptions getOptions() const;
    [[nodiscard]] Geometry3D getGeometry() const;
    [[nodiscard]] bool isInitialized() const noexcept;
    void setVelocityModel(const Model3D<T> &velocityModel);
    [[nodiscard]] Model3D<T> getVelocityModel() const;
    [[nodiscard]] bool haveVelocityModel() const noexcept override;
    [[nodiscard]] T getSlowness(int iCellX, int iCellY, int iCellZ) const override;
    void setSource(const Source3D &source);
    void setSource(const std::tuple<double, double, double> &location);
    [[nodiscard]] Source3D getSource() const override;
    [[nodiscard]] bool haveSource() const noexcept override;
    void setStations(const std::vector<Station3D> &stations);
    [[nodiscard]] std::vector<Station3D> getStations() const;
    [[nodiscard]] const std::vector<Station3D>& getStationsReference() const;
    void solve();
    [[nodiscard]] std::vector<T> getTravelTimeField() const override;
    [[nodiscard]] const T* getTravelTimeFieldPointer() const override;
    [[nodiscard]] bool haveTravelTimeField() const noexcept override;
    [[nodiscard]] std::vector<T> getTravelTimeGradientField() const override;
    [[nodiscard]] const T *getTravelTimeGradientFieldPointer() const override;
    [[nodiscard]] bool haveTravelTimeGradientField() const noexcept override;
    /// Computes the gradient of the solved field on the GPU: (dT/dx, dT/dy, dT/dz) per node,
    /// natural order.  Central differences inside, second-order one-sided differences on
    /// the faces, the analytic gradient at the source cell's corners.  An addition: the
    /// reference declares the gradient getters but never computes the field.
    void computeTravelTimeGradientField();
    /// Travel times at the stations of setStations(): trilinear interpolation of the solved
    /// field, the straight-ray time in the source cell.  An addition, as for the gradient.
    [[nodiscard]] std::vector<T> getTravelTimesAtStations() const;
    void clear() noexcept;
private:
    class Solver3DImpl;
    std::unique_ptr<Solver3DImpl> pImpl;
};
}
#endif
