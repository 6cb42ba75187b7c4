// ORACLE SHIM — test infrastructure only: stand-in for tbb::cache_aligned_allocator.
#ifndef EIKX_ORACLE_SHIM_TBB_CACHE_ALIGNED_ALLOCATOR_H
#define EIKX_ORACLE_SHIM_TBB_CACHE_ALIGNED_ALLOCATOR_H
#include <memory>
namespace tbb {
template <class T> using cache_aligned_allocator = std::allocator<T>;
}  // namespace tbb
#endif
