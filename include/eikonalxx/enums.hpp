// Enumerations of the solver API (drop-in for uofuseismo/eikonalxx,
// include/eikonalxx/enums.hpp:7-90): the same names and values.
#ifndef EIKONALXX_ENUMS_HPP
#define EIKONALXX_ENUMS_HPP
namespace EikonalXX
{
/// Memory order of a 2D array: Natural/ZX = x fastest; XZ = z fastest.
enum class Ordering2D { Natural = 0, ZX = 0, XZ = 1 };
/// Memory order of a 3D array: Natural/ZYX = x fastest, then y; XYZ = z fastest.
enum class Ordering3D { Natural = 0, ZYX = 0, XYZ = 1 };
/// LevelSetMethod: nodes of one wavefront level are updated in parallel (on the GPU);
/// FastSweepingMethod: the serial sweep order.  Both orders give identical travel
/// times; this library always runs the level-set order on the GPU.
enum class SolverAlgorithm { LevelSetMethod, FastSweepingMethod };
/// Sweep1 increases x and z; Sweep2 decreases x; Sweep3 decreases z; Sweep4 both.
enum class SweepNumber2D { Sweep1 = 0, Sweep2 = 1, Sweep3 = 2, Sweep4 = 3 };
/// Bit 0 of (Sweep - 1) flips x, bit 1 flips y, bit 2 flips z.
enum class SweepNumber3D { Sweep1 = 0, Sweep2 = 1, Sweep3 = 2, Sweep4 = 3,
                           Sweep5 = 4, Sweep6 = 5, Sweep7 = 6, Sweep8 = 7 };
/// Logging level.
enum class Verbosity { Error, Warning, Info, Debug };
}
#endif
