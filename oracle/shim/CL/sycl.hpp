// ORACLE SHIM — test infrastructure only.
// A serial host stand-in for the few SYCL names the reference's hot-path headers use
// (include/private/solverUtilities{2,3}d.hpp, include/private/solver{2,3}d.hpp), so
// those headers compile unchanged with g++ for the reference build under oracle/_ref.
// Math maps onto the C++ standard library (IEEE, correctly rounded sqrt); queues run
// kernels serially on the calling thread.
#ifndef EIKX_ORACLE_SHIM_SYCL_HPP
#define EIKX_ORACLE_SHIM_SYCL_HPP
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <cstddef>
#include <functional>

namespace sycl {
using std::fmin;
using std::fmax;
using std::sqrt;
using std::hypot;
using std::acosh;
using std::abs;
template <class T> inline T min(T a, T b) { return std::min(a, b); }
template <class T> inline T max(T a, T b) { return std::max(a, b); }

template <int D = 1> struct id {
    std::size_t v{0};
    operator std::size_t() const { return v; }
};
template <int D = 1> struct range {
    std::size_t n{0};
    range(std::size_t n_) : n(n_) {}
};
range(std::size_t) -> range<1>;
struct event {
    void wait() {}
};
struct handler {
    void depends_on(const event &) {}
    template <class K> void parallel_for(range<1> r, K k) {
        for (std::size_t i = 0; i < r.n; ++i) k(id<1>{i});
    }
    void memcpy(void *d, const void *s, std::size_t n) { std::memcpy(d, s, n); }
};
struct device {};
struct cpu_selector_t {};
inline constexpr cpu_selector_t cpu_selector_v{};
struct queue {
    queue() = default;
    template <class S> explicit queue(const S &) {}
    template <class F> event submit(F f) { handler h; f(h); return {}; }
    event memcpy(void *d, const void *s, std::size_t n) { std::memcpy(d, s, n); return {}; }
    void wait() {}
};
template <class T> T *malloc_device(std::size_t n, queue &) { return static_cast<T *>(std::calloc(n ? n : 1, sizeof(T))); }
template <class T> T *malloc_shared(std::size_t n, queue &) { return static_cast<T *>(std::calloc(n ? n : 1, sizeof(T))); }
inline void free(void *p, queue &) { std::free(p); }
}  // namespace sycl
#endif
