// 2D eikonal solver (drop-in for include/eikonalxx/solver2d.hpp:20-200 of the reference).
//
// Same workflow as Solver3D with the 4 sweeps of 2D; after a solve the travel times at
// the stations are interpolated bilinearly (src/solver2d.cpp:106-167).  Solver2D<double>
// sweeps in FP64 and Solver2D<float> in FP32, on the GPU.  The gradient field is central
// differences of the travel times (src/gradient.hpp).  writeVTK writes legacy-VTK files
// (IO::VTKRectilinearGrid2D).  Not copyable, not thread-safe.
#ifndef EIKONALXX_SOLVER_2D_HPP
#define EIKONALXX_SOLVER_2D_HPP
#include <memory>
#include <string>
#include <utility>
#include <vector>
#include "eikonalxx/abstractBaseClass/solver2d.hpp"
namespace EikonalXX
{
class Geometry2D;
template<class T> class Model2D;
class Source2D;
class SolverOptions;
class Station2D;
template<class T>
class Solver2D : public EikonalXX::AbstractBaseClass::ISolver2D<T>
{
public:
    Solver2D();
    ~Solver2D() override;
    Solver2D(const Solver2D &solver) = delete;
    Solver2D(Solver2D &&solver) noexcept = delete;
    Solver2D& operator=(const Solver2D &solver) = delete;
    Solver2D& operator=(Solver2D &&solver) noexcept = delete;
    void initialize(const SolverOptions &options, const Geometry2D &geometry);
    [[nodiscard]] SolverOptions getOptions() const;
    [[nodiscard]] Geometry2D getGeometry() const;
    [[nodiscard]] bool isInitialized() const noexcept;
    void setVelocityModel(const Model2D<T> &velocityModel);
    [[nodiscard]] Model2D<T> getVelocityModel() const;
    [[nodiscard]] bool haveVelocityModel() const noexcept override;
    [[nodiscard]] T getSlowness(int iCellX, int iCellZ) const override;
    void setSource(const Source2D &source);
    void setSource(const std::pair<double, double> &location);
    [[nodiscard]] Source2D getSource() const override;
    [[nodiscard]] bool haveSource() const noexcept override;
    void setStations(const std::vector<Station2D> &stations);
    [[nodiscard]] std::vector<Station2D> getStations() const;
    [[nodiscard]] const std::vector<Station2D>& getStationsReference() const;
    void solve();
    void computeTravelTimeGradientField();
    [[nodiscard]] std::vector<T> getTravelTimeField() const override;
    [[nodiscard]] const T* getTravelTimeFieldPointer() const override;
    [[nodiscard]] bool haveTravelTimeField() const noexcept override;
    [[nodiscard]] std::vector<T> getTravelTimesAtStations() const;
    [[nodiscard]] std::vector<T> getTravelTimeGradientField() const override;
    [[nodiscard]] const T *getTravelTimeGradientFieldPointer() const override;
    [[nodiscard]] bool haveTravelTimeGradientField() const noexcept override;
    /// Writes the travel-time field (and, with writeGradient, its gradient as vectors named
    /// title + "_gradient") to a binary legacy-VTK file (IO::VTKRectilinearGrid2D).
    /// Throws std::runtime_error if the field (or gradient) has not been computed.
    void writeVTK(const std::string &fileName, const std::string &title = "travel_time_field_s",
                  bool writeGradient = false) const;
    void clear() noexcept;
private:
    class Solver2DImpl;
    std::unique_ptr<Solver2DImpl> pImpl;
};
}
#endif
