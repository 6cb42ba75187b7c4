// Graph3D<E> (reference: src/graph3d.cpp:120-340) over eikx_graph3d_tables.
#include <stdexcept>
#include <string>
#include <vector>
#include "eikonalxx/graph3d.hpp"
#include "eikx/eikx_c.h"

using namespace EikonalXX;

template <SweepNumber3D E>
class Graph3D<E>::Graph3DImpl
{
public:
    std::vector<int> levelStart, nodeToIndex, toX, toY, toZ, indexToLevel;
    int nLevels{0}, nGrid{0}, maxLevelSize{0};
    bool initialized{false};
};

template <SweepNumber3D E> Graph3D<E>::Graph3D() : pImpl(std::make_unique<Graph3DImpl>()) {}
template <SweepNumber3D E> Graph3D<E>::Graph3D(const Graph3D &g) { *this = g; }
template <SweepNumber3D E> Graph3D<E>::Graph3D(Graph3D &&g) noexcept { *this = std::move(g); }
template <SweepNumber3D E> Graph3D<E> &Graph3D<E>::operator=(const Graph3D &g)
{
    if (&g != this) pImpl = std::make_unique<Graph3DImpl>(*g.pImpl);
    return *this;
}
template <SweepNumber3D E> Graph3D<E> &Graph3D<E>::operator=(Graph3D &&g) noexcept
{
    if (&g != this) pImpl = std::move(g.pImpl);
    return *this;
}
template <SweepNumber3D E> Graph3D<E>::~Graph3D() = default;
template <SweepNumber3D E> void Graph3D<E>::clear() noexcept { pImpl = std::make_unique<Graph3DImpl>(); }

template <SweepNumber3D E> void Graph3D<E>::initialize(const int nx, const int ny, const int nz)
{
    clear();
    if (nx < 3) throw std::invalid_argument("nx must be at least 3");
    if (ny < 3) throw std::invalid_argument("ny must be at least 3");
    if (nz < 3) throw std::invalid_argument("nz must be at least 3");
    const size_t n = static_cast<size_t>(nx) * ny * nz;
    auto &p = *pImpl;
    p.levelStart.resize(nx + ny + nz - 1);
    p.nodeToIndex.resize(n); p.toX.resize(n); p.toY.resize(n); p.toZ.resize(n); p.indexToLevel.resize(n);
    const int nl = eikx_graph3d_tables(static_cast<int>(E), nx, ny, nz, p.levelStart.data(), p.nodeToIndex.data(),
                                       p.toX.data(), p.toY.data(), p.toZ.data(), p.indexToLevel.data(),
                                       &p.maxLevelSize);
    if (nl < 0) throw std::invalid_argument("grid too large for level tables");
    p.nLevels = nl;
    p.nGrid = static_cast<int>(n);
    p.initialized = true;
}
template <SweepNumber3D E> bool Graph3D<E>::isInitialized() const noexcept { return pImpl->initialized; }
#define EIKX_NEED_INIT                                                                             \
    if (!isInitialized()) throw std::runtime_error("Class not initialized")
template <SweepNumber3D E> int Graph3D<E>::getNumberOfGridPoints() const { EIKX_NEED_INIT; return pImpl->nGrid; }
template <SweepNumber3D E> int Graph3D<E>::getNumberOfLevels() const { EIKX_NEED_INIT; return pImpl->nLevels; }
template <SweepNumber3D E> int Graph3D<E>::getMaximumLevelSize() const { EIKX_NEED_INIT; return pImpl->maxLevelSize; }
template <SweepNumber3D E> int Graph3D<E>::getNumberOfNodesInLevel(const int level) const
{
    EIKX_NEED_INIT;
    if (level < 0 || level >= pImpl->nLevels)
        throw std::invalid_argument("level = " + std::to_string(level) + " must be in range [0," +
                                    std::to_string(pImpl->nLevels - 1) + "]");
    return pImpl->levelStart[level + 1] - pImpl->levelStart[level];
}
template <SweepNumber3D E> const int *Graph3D<E>::getIndexToLevelPointer() const { EIKX_NEED_INIT; return pImpl->indexToLevel.data(); }
template <SweepNumber3D E> const int *Graph3D<E>::getLevelStartPointer() const { EIKX_NEED_INIT; return pImpl->levelStart.data(); }
template <SweepNumber3D E> const int *Graph3D<E>::getNodeInLevelToIndexPointer() const { EIKX_NEED_INIT; return pImpl->nodeToIndex.data(); }
template <SweepNumber3D E> const int *Graph3D<E>::getNodeInLevelToXGridPointPointer() const { EIKX_NEED_INIT; return pImpl->toX.data(); }
template <SweepNumber3D E> const int *Graph3D<E>::getNodeInLevelToYGridPointPointer() const { EIKX_NEED_INIT; return pImpl->toY.data(); }
template <SweepNumber3D E> const int *Graph3D<E>::getNodeInLevelToZGridPointPointer() const { EIKX_NEED_INIT; return pImpl->toZ.data(); }

int EikonalXX::computeNumberOfLevels(const int nx, const int ny, const int nz) noexcept { return nx + ny + nz - 2; }

template class EikonalXX::Graph3D<SweepNumber3D::Sweep1>;
template class EikonalXX::Graph3D<SweepNumber3D::Sweep2>;
template class EikonalXX::Graph3D<SweepNumber3D::Sweep3>;
template class EikonalXX::Graph3D<SweepNumber3D::Sweep4>;
template class EikonalXX::Graph3D<SweepNumber3D::Sweep5>;
template class EikonalXX::Graph3D<SweepNumber3D::Sweep6>;
template class EikonalXX::Graph3D<SweepNumber3D::Sweep7>;
template class EikonalXX::Graph3D<SweepNumber3D::Sweep8>;
