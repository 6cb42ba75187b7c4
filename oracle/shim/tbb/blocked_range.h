// ORACLE SHIM — test infrastructure only: serial stand-in for tbb::blocked_range.
#ifndef EIKX_ORACLE_SHIM_TBB_BLOCKED_RANGE_H
#define EIKX_ORACLE_SHIM_TBB_BLOCKED_RANGE_H
namespace tbb {
template <class V> class blocked_range {
public:
    blocked_range(V b, V e) : b_(b), e_(e) {}
    V begin() const { return b_; }
    V end() const { return e_; }
private:
    V b_, e_;
};
}  // namespace tbb
#endif
