// Level-set tables of one 3D sweep (drop-in for include/eikonalxx/graph3d.hpp:11-121 of
// the reference): level L holds the nodes whose sweep-permuted indices sum to L, sorted
// by natural index.  The GPU sweeps do not need these tables (their levels are implicit);
// they are computed on the host by eikx_graph3d_tables for callers of the reference API.
#ifndef EIKONALXX_GRAPH_3D_HPP
#define EIKONALXX_GRAPH_3D_HPP
#include <memory>
#include "eikonalxx/enums.hpp"
namespace EikonalXX
{
template<EikonalXX::SweepNumber3D E>
class Graph3D
{
public:
    Graph3D();
    Graph3D(const Graph3D &graph);
    Graph3D(Graph3D &&graph) noexcept;
    Graph3D& operator=(const Graph3D &graph);
    Graph3D& operator=(Graph3D &&graph) noexcept;
    ~Graph3D();
    void initialize(int nx, int ny, int nz);
    bool isInitialized() const noexcept;
    [[nodiscard]] int getNumberOfGridPoints() const;
    [[nodiscard]] int getMaximumLevelSize() const;
    [[nodiscard]] int getNumberOfLevels() const;
    [[nodiscard]] int getNumberOfNodesInLevel(int level) const;
    [[nodiscard]] const int *getIndexToLevelPointer() const;
    [[nodiscard]] const int *getLevelStartPointer() const;
    [[nodiscard]] const int *getNodeInLevelToIndexPointer() const;
    [[nodiscard]] const int *getNodeInLevelToXGridPointPointer() const;
    [[nodiscard]] const int *getNodeInLevelToYGridPointPointer() const;
    [[nodiscard]] const int *getNodeInLevelToZGridPointPointer() const;
    void clear() noexcept;
private:
    class Graph3DImpl;
    std::unique_ptr<Graph3DImpl> pImpl;
};
/// nx + ny + nz - 2 (src/graph3d.cpp:324-329).
int computeNumberOfLevels(const int nx, const int ny, const int nz) noexcept;
}
#endif
