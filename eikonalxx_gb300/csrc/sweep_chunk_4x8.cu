// Chunk-step 3D sweep kernels with 4 x 8 pencils per warp (sweep_chunk.cuh).
#include "sweep_chunk.cuh"

namespace eikx {
EIKX_CHUNK_SHAPE(4, 8)
}  // namespace eikx
