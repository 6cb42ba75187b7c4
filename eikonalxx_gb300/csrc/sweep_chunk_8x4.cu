// Chunk-step 3D sweep kernels with 8 x 4 pencils per warp (sweep_chunk.cuh).
#include "sweep_chunk.cuh"

namespace eikx {
EIKX_CHUNK_SHAPE(8, 4)
}  // namespace eikx
