// Level-set tables on the host: the 3D Graph3D tables and the 2D level order.
//
// The GPU sweep never reads these tables -- its levels are implicit in the warp-block
// wavefront -- but callers of the reference's Graph3D<E> (src/graph3d.cpp:120-317) and
// of the 2D level helpers (solverUtilities2d.hpp:1063-1266) get the same integers.
#include <algorithm>
#include <vector>

#include "eikx/eikx_c.h"

namespace {

// Sweep-permuted coordinate of axis index i (permuteGrid, solverUtilities3d.hpp:1197-1257).
inline int perm(int i, int n, int flip) { return flip ? n - 1 - i : i; }

}  // namespace

extern "C" int eikx_graph3d_tables(int sweep, int nx, int ny, int nz, int *levelStart, int *nodeToIndex,
                                   int *toX, int *toY, int *toZ, int *indexToLevel, int *maxLevelSize) {
    if (sweep < 0 || sweep > 7) return EIKX_ERR_INVALID;
    if (nx < 3 || ny < 3 || nz < 3) return EIKX_ERR_INVALID;
    if (!levelStart || !nodeToIndex || !toX || !toY || !toZ || !indexToLevel || !maxLevelSize)
        return EIKX_ERR_INVALID;
    const long long nGrid = static_cast<long long>(nx) * ny * nz;
    if (nGrid > (1LL << 31) - 1) return EIKX_ERR_INVALID;
    const int fx = sweep & 1, fy = (sweep >> 1) & 1, fz = (sweep >> 2) & 1;
    const int nLevels = nx + ny + nz - 2;
    const int nxy = nx * ny;
    // Level L holds the nodes whose permuted coordinates sum to L.  Walk the permuted
    // (jz, jy) pairs of the level, emit the natural indices, then sort them ascending:
    // the same content and order as the reference's table.
    int offset = 0, maxSize = 0;
    levelStart[0] = 0;
    for (int level = 0; level < nLevels; ++level) {
        int count = 0;
        const int zLo = std::max(0, level - (nx - 1) - (ny - 1)), zHi = std::min(nz - 1, level);
        for (int jz = zLo; jz <= zHi; ++jz) {
            const int yLo = std::max(0, level - jz - (nx - 1)), yHi = std::min(ny - 1, level - jz);
            for (int jy = yLo; jy <= yHi; ++jy) {
                const int jx = level - jz - jy;
                const int ix = perm(jx, nx, fx), iy = perm(jy, ny, fy), iz = perm(jz, nz, fz);
                nodeToIndex[offset + count] = iz * nxy + iy * nx + ix;
                // filled by node position, as the reference (src/graph3d.cpp:177)
                indexToLevel[offset + count] = level;
                ++count;
            }
        }
        std::sort(nodeToIndex + offset, nodeToIndex + offset + count);
        for (int i = offset; i < offset + count; ++i) {
            const int idx = nodeToIndex[i];
            const int iz = idx / nxy, r = idx - iz * nxy, iy = r / nx;
            toX[i] = r - iy * nx;
            toY[i] = iy;
            toZ[i] = iz;
        }
        offset += count;
        levelStart[level + 1] = offset;
        maxSize = std::max(maxSize, count);
    }
    *maxLevelSize = maxSize;
    return nLevels;
}

extern "C" int eikx_levels2d(int sweep, int nx, int nz, int *levelStart, int *orderIx, int *orderIz) {
    if (sweep < 0 || sweep > 3) return EIKX_ERR_INVALID;
    if (nx < 3 || nz < 3) return EIKX_ERR_INVALID;
    if (!levelStart || !orderIx || !orderIz) return EIKX_ERR_INVALID;
    const int fx = sweep & 1, fz = (sweep >> 1) & 1;
    const int nLevels = nx + nz - 1;  // computeNumberOfLevels, solverUtilities2d.hpp:1241-1244
    int k = 0;
    levelStart[0] = 0;
    for (int level = 0; level < nLevels; ++level) {
        // level slice [max(0, L+1-nx), min(nz, L+1)) over the permuted z index
        // (getLevelStartStopIndices, solverUtilities2d.hpp:1230-1235)
        const int i0 = std::max(0, level + 1 - nx), i1 = std::min(nz, level + 1);
        for (int jz = i0; jz < i1; ++jz) {
            orderIx[k] = perm(level - jz, nx, fx);
            orderIz[k] = perm(jz, nz, fz);
            ++k;
        }
        levelStart[level + 1] = k;
    }
    return nLevels;
}
