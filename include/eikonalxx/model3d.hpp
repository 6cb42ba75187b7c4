// A 3D velocity model held as cell slowness (drop-in for include/eikonalxx/model3d.hpp
// of the reference).  Nodal velocities become cell slowness 8/(sum of the cell's corner
// velocities); cellular velocities become 1/v.  Velocities must be positive.
#ifndef EIKONALXX_MODEL_3D_HPP
#define EIKONALXX_MODEL_3D_HPP
#include <memory>
#include <string>
#include <vector>
#include "eikonalxx/enums.hpp"
namespace EikonalXX
{
class Geometry3D;
template<class T>
class Model3D
{
public:
    Model3D();
    Model3D(const Model3D &model);
    Model3D(Model3D &&model) noexcept;
    Model3D& operator=(const Model3D &model);
    Model3D& operator=(Model3D &&model) noexcept;
    ~Model3D();
    void initialize(const Geometry3D &geometry);
    [[nodiscard]] bool isInitialized() const noexcept;
    [[nodiscard]] int getNumberOfGridPoints() const;
    [[nodiscard]] int getNumberOfCells() const;
    [[nodiscard]] Geometry3D getGeometry() const;
    void setNodalVelocities(int nGrid, const T velocity[], EikonalXX::Ordering3D ordering);
    template<typename U>
    void setCellularVelocities(int nCell, const U velocity[], EikonalXX::Ordering3D ordering);
    [[nodiscard]] bool haveVelocities() const noexcept;
    [[nodiscard]] std::vector<T> getSlowness() const;
    [[nodiscard]] const T* getSlownessPointer() const;
    [[nodiscard]] std::vector<T> getVelocities() const;
    [[nodiscard]] T getSlowness(int iCellX, int iCellY, int iCellZ) const;
    /// Writes the cell velocities to a binary legacy-VTK rectilinear-grid file
    /// (IO::VTKRectilinearGrid3D).  Throws std::runtime_error if no model is set.
    void writeVTK(const std::string &fileName, const std::string &title = "velocity_m/s") const;
    void clear() noexcept;
private:
    class Model3DImpl;
    std::unique_ptr<Model3DImpl> pImpl;
};
}
#endif
