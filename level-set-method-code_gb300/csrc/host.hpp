// host.hpp -- helpers shared by the host-side translation units (api.cu,
// sample_api.cu): error reporting with a thread-local message and the
// status-returning CUDA call wrappers.
#pragma once

#include <string>

#include "common.cuh"

namespace lsgb {

extern thread_local std::string g_err;
// Records the message for lsgb_last_error and returns code.
int fail(int code, const char* fmt, ...);
// LSGB_OK if ptr is device (or managed) memory, else LSGB_ERR_INVALID.
int check_dev(const void* ptr, const char* name);

#define LSGB_CUDA(call)                                                                  \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess)                                                           \
            return fail(LSGB_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                        __FILE__, __LINE__);                                             \
    } while (0)

#define LSGB_TRY(call)             \
    do {                           \
        int rc_ = (call);          \
        if (rc_ != LSGB_OK) return rc_; \
    } while (0)

}  // namespace lsgb
