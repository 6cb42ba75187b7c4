// Interface of a 3D travel-time solver (drop-in for the reference's
// include/eikonalxx/abstractBaseClass/solver3d.hpp).
#ifndef EIKONALX_ABSTRACT_BASE_CLASS_SOLVER_3D_HPP
#define EIKONALX_ABSTRACT_BASE_CLASS_SOLVER_3D_HPP
#include <vector>
namespace EikonalXX { class Source3D; }
namespace EikonalXX::AbstractBaseClass
{
template<class T>
class ISolver3D
{
public:
    virtual ~ISolver3D() = default;
    virtual bool haveVelocityModel() const noexcept = 0;
    virtual std::vector<T> getTravelTimeField() const = 0;
    virtual const T* getTravelTimeFieldPointer() const = 0;
    virtual std::vector<T> getTravelTimeGradientField() const = 0;
    virtual const T* getTravelTimeGradientFieldPointer() const = 0;
    virtual bool haveTravelTimeField() const noexcept = 0;
    virtual bool haveTravelTimeGradientField() const noexcept = 0;
    virtual Source3D getSource() const = 0;
    virtual bool haveSource() const noexcept = 0;
    virtual T getSlowness(int iCellX, int iCellY, int iCellZ) const = 0;
};
}
#endif
