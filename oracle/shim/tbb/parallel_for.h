// ORACLE SHIM — test infrastructure only: serial stand-in for tbb::parallel_for.
#ifndef EIKX_ORACLE_SHIM_TBB_PARALLEL_FOR_H
#define EIKX_ORACLE_SHIM_TBB_PARALLEL_FOR_H
#include "tbb/blocked_range.h"
namespace tbb {
template <class R, class F> void parallel_for(const R &r, const F &f) { f(r); }
}  // namespace tbb
#endif
