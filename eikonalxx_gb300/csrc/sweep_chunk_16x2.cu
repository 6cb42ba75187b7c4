// Chunk-step 3D sweep kernels with 16 x 2 pencils per warp (sweep_chunk.cuh).
#include "sweep_chunk.cuh"

namespace eikx {
EIKX_CHUNK_SHAPE(16, 2)
}  // namespace eikx
