// Interface of a 2D travel-time solver (drop-in for the reference's
// include/eikonalxx/abstractBaseClass/solver2d.hpp).
#ifndef EIKONALX_ABSTRACT_BASE_CLASS_SOLVER_2D_HPP
#define EIKONALX_ABSTRACT_BASE_CLASS_SOLVER_2D_HPP
#include <vector>
namespace EikonalXX { class Source2D; }
namespace EikonalXX::AbstractBaseClass
{
template<class T>
class ISolver2D
{
public:
    virtual ~ISolver2D() = default;
    virtual bool haveVelocityModel() const noexcept = 0;
    virtual std::vector<T> getTravelTimeField() const = 0;
    virtual const T* getTravelTimeFieldPointer() const = 0;
    virtual std::vector<T> getTravelTimeGradientField() const = 0;
    virtual const T *getTravelTimeGradientFieldPointer() const = 0;
    virtual bool haveTravelTimeField() const noexcept = 0;
    virtual bool haveTravelTimeGradientField() const noexcept = 0;
    virtual Source2D getSource() const = 0;
    virtual bool haveSource() const noexcept = 0;
    virtual T getSlowness(int iCellX, int iCellZ) const = 0;
};
}
#endif
