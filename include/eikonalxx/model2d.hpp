// A 2D velocity model held as cell slowness (drop-in for include/eikonalxx/model2d.hpp
// of the reference).  Nodal velocities become cell slowness 4/(sum of the cell's corner
// velocities); cellular velocities become 1/v.  Velocities must be positive.
#ifndef EIKONALXX_MODEL_2D_HPP
#define EIKONALXX_MODEL_2D_HPP
#include <memory>
#include <string>
#include <vector>
#include "eikonalxx/enums.hpp"
namespace EikonalXX
{
class Geometry2D;
template<class T>
class Model2D
{
public:
    Model2D();
    Model2D(const Model2D &model);
    Model2D(Model2D &&model) noexcept;
    Model2D& operator=(const Model2D &model);
    Model2D& operator=(Model2D &&model) noexcept;
    ~Model2D();
    void initialize(const Geometry2D &geometry);
    [[nodiscard]] bool isInitialized() const noexcept;
    [[nodiscard]] int getNumberOfGridPoints() const;
    [[nodiscard]] int getNumberOfCells() const;
    [[nodiscard]] Geometry2D getGeometry() const;
    void setNodalVelocities(int nGrid, const T velocity[], EikonalXX::Ordering2D ordering);
    template<typename U>
    void setCellularVelocities(int nCell, const U velocity[], EikonalXX::Ordering2D ordering);
    [[nodiscard]] bool haveVelocities() const noexcept;
    [[nodiscard]] std::vector<T> getSlowness() const;
    [[nodiscard]] const T* getSlownessPointer() const;
    [[nodiscard]] std::vector<T> getVelocities() const;
    [[nodiscard]] T getSlowness(int iCellX, int iCellZ) const;
    /// Writes the cell velocities to a binary legacy-VTK rectilinear-grid file
    /// (IO::VTKRectilinearGrid2D).  Throws std::runtime_error if no model is set.
    void writeVTK(const std::string &fileName, const std::string &title = "velocity_m/s") const;
    void clear() noexcept;
private:
    class Model2DImpl;
    std::unique_ptr<Model2DImpl> pImpl;
};
}
#endif
