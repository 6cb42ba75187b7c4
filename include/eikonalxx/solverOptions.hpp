// Solver options (drop-in for include/eikonalxx/solverOptions.hpp:11-111 of the
// reference).  Defaults as src/solverOptions.cpp:5-21: 5 refinement iterations,
// tolerance 1e-5 s, factored-eikonal radius 3, level-set algorithm, Error verbosity.
// Unlike the reference, the tolerance is applied: a solve ends once each of its last
// 8 (3D) / 4 (2D) refinement sweeps decreased no travel time by the tolerance or more.
#ifndef EIKONALXX_SOLVER_OPTIONS_HPP
#define EIKONALXX_SOLVER_OPTIONS_HPP
#include <cstdint>
#include <memory>
#include <ostream>
#include "eikonalxx/enums.hpp"
namespace EikonalXX
{
class SolverOptions
{
public:
    SolverOptions();
    SolverOptions(const SolverOptions &options);
    SolverOptions(SolverOptions &&options) noexcept;
    SolverOptions& operator=(const SolverOptions &options);
    SolverOptions& operator=(SolverOptions &&options) noexcept;
    ~SolverOptions();
    void setNumberOfSweeps(uint16_t nSweeps) noexcept;
    [[nodiscard]] int getNumberOfSweeps() const noexcept;
    void setConvergenceTolerance(double tolerance) noexcept;
    [[nodiscard]] double getConvergenceTolerance() const noexcept;
    void setFactoredEikonalEquationSolverRadius(int radius) noexcept;
    [[nodiscard]] int getFactoredEikonalEquationSolverRadius() const noexcept;
    void setVerbosity(EikonalXX::Verbosity verbosity) noexcept;
    [[nodiscard]] EikonalXX::Verbosity getVerbosity() const noexcept;
    void setAlgorithm(EikonalXX::SolverAlgorithm algorithm) noexcept;
    [[nodiscard]] EikonalXX::SolverAlgorithm getAlgorithm() const noexcept;
    void clear() noexcept;
private:
    class SolverOptionsImpl;
    std::unique_ptr<SolverOptionsImpl> pImpl;
};
std::ostream& operator<<(std::ostream &os, const SolverOptions &options);
}
#endif
