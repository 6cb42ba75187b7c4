// Shared helpers of the C++ solver classes: one eikx_ctx per solver object and the
// mapping of eikx_status to the reference's exception types.
#pragma once
#include <cstdlib>
#include <stdexcept>
#include <string>
#include "eikx/eikx_c.h"

namespace EikonalXX::Detail
{
/// Throws std::invalid_argument for EIKX_ERR_INVALID and std::runtime_error otherwise.
inline void check(eikx_status rc)
{
    if (rc == EIKX_OK) return;
    const std::string msg = eikx_last_error();
    if (rc == EIKX_ERR_INVALID) throw std::invalid_argument(msg);
    throw std::runtime_error(msg);
}

/// GPU context owned by one solver object; created on first use on device 0 or the
/// device named by the EIKX_DEVICE environment variable.
class GpuContext
{
public:
    GpuContext() = default;
    GpuContext(const GpuContext &) = delete;
    GpuContext &operator=(const GpuContext &) = delete;
    ~GpuContext() { reset(); }
    eikx_ctx *get()
    {
        if (!ctx_) {
            int device = 0;
            if (const char *d = std::getenv("EIKX_DEVICE")) device = std::atoi(d);
            check(eikx_create(&ctx_, device));
        }
        return ctx_;
    }
    void reset() noexcept
    {
        if (ctx_) eikx_destroy(ctx_);
        ctx_ = nullptr;
    }
private:
    eikx_ctx *ctx_{nullptr};
};

template <class T> constexpr int dtypeOf() { return sizeof(T) == 4 ? EIKX_F32 : EIKX_F64; }

/// SolverOptions -> eikx_options (the GPU knobs keep their defaults).
template <class O> eikx_options toOptions(const O &o)
{
    eikx_options r;
    eikx_options_default(&r);
    r.n_sweeps = o.getNumberOfSweeps();
    r.tolerance = o.getConvergenceTolerance();
    r.factored_radius = o.getFactoredEikonalEquationSolverRadius();
    return r;
}
}
