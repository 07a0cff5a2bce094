// wc_util.h — error reporting helpers shared by the host translation units.
#pragma once

#include <nvtx3/nvToolsExt.h>

#include "../../include/watercube.h"

namespace wc {

// Record a message for wc_last_error() and return `s`.
wc_status fail(wc_status s, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
void clear_error();
const char* last_error();

// NVTX range for the duration of a scope: the library's entry points appear by name on an
// Nsight timeline (header-only NVTX3; nothing is recorded unless a tool is attached).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};
#define WC_NVTX(name) ::wc::NvtxRange wc_nvtx_range_(name)

// cudaMalloc of every device buffer the library owns (WC_ERR_OOM on failure); the allocation
// failure test hook (wc_debug_fail_allocations) acts here.
wc_status device_alloc(void** p, size_t bytes);

}  // namespace wc

// Return WC_ERR_CUDA (with the call text and CUDA's message) when a runtime call fails.
#define WC_CUDA_TRY(call)                                                                        \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess)                                                                   \
            return ::wc::fail(e_ == cudaErrorMemoryAllocation ? WC_ERR_OOM : WC_ERR_CUDA,        \
                              "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

// Return a non-OK status from the enclosing function.
#define WC_TRY(expr)                \
    do {                            \
        wc_status s_ = (expr);      \
        if (s_ != WC_OK) return s_; \
    } while (0)
