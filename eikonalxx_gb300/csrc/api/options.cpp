// SolverOptions (reference: src/solverOptions.cpp).
#include <string>
#include "eikonalxx/solverOptions.hpp"

using namespace EikonalXX;

class SolverOptions::SolverOptionsImpl
{
public:
    double tolerance{1.e-5};
    int radius{3};
    SolverAlgorithm algorithm{SolverAlgorithm::LevelSetMethod};
    Verbosity verbosity{Verbosity::Error};
    uint16_t sweeps{5};
};

SolverOptions::SolverOptions() : pImpl(std::make_unique<SolverOptionsImpl>()) {}
SolverOptions::SolverOptions(const SolverOptions &o) { *this = o; }
SolverOptions::SolverOptions(SolverOptions &&o) noexcept { *this = std::move(o); }
SolverOptions &SolverOptions::operator=(const SolverOptions &o)
{
    if (&o != this) pImpl = std::make_unique<SolverOptionsImpl>(*o.pImpl);
    return *this;
}
SolverOptions &SolverOptions::operator=(SolverOptions &&o) noexcept
{
    if (&o != this) pImpl = std::move(o.pImpl);
    return *this;
}
SolverOptions::~SolverOptions() = default;
void SolverOptions::setNumberOfSweeps(uint16_t n) noexcept { pImpl->sweeps = n; }
int SolverOptions::getNumberOfSweeps() const noexcept { return pImpl->sweeps; }
void SolverOptions::setConvergenceTolerance(double t) noexcept { pImpl->tolerance = t; }
double SolverOptions::getConvergenceTolerance() const noexcept { return pImpl->tolerance; }
void SolverOptions::setFactoredEikonalEquationSolverRadius(int r) noexcept { pImpl->radius = r; }
int SolverOptions::getFactoredEikonalEquationSolverRadius() const noexcept { return pImpl->radius; }
void SolverOptions::setVerbosity(Verbosity v) noexcept { pImpl->verbosity = v; }
Verbosity SolverOptions::getVerbosity() const noexcept { return pImpl->verbosity; }
void SolverOptions::setAlgorithm(SolverAlgorithm a) noexcept { pImpl->algorithm = a; }
SolverAlgorithm SolverOptions::getAlgorithm() const noexcept { return pImpl->algorithm; }
void SolverOptions::clear() noexcept { pImpl = std::make_unique<SolverOptionsImpl>(); }

std::ostream &EikonalXX::operator<<(std::ostream &os, const SolverOptions &o)
{
    std::string r = "Solver Options:\n";
    r += "    Number of sweeps: " + std::to_string(o.getNumberOfSweeps()) + "\n";
    r += o.getAlgorithm() == SolverAlgorithm::LevelSetMethod ? "    Solver type: Level-set method\n"
                                                              : "    Solver type: Fast-sweeping method\n";
    r += "    Convergence (seconds): " + std::to_string(o.getConvergenceTolerance()) + "\n";
    r += "    Factored-eikonal equation radius (grid points): " +
         std::to_string(o.getFactoredEikonalEquationSolverRadius()) + "\n";
    r += "    Verbosity: " + std::to_string(static_cast<int>(o.getVerbosity())) + "\n";
    return os << r;
}
