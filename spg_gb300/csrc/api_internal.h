// Error plumbing shared by the C ABI implementation files.
#pragma once

#include <string>

#include "spgx.h"

namespace spgx {

void set_error(const std::string &msg);
void clear_error();

}  // namespace spgx

// Evaluates a CUDA runtime call; on failure records the message and returns SPGX_ERR_CUDA.
#define SPGX_CUDA(call)                                                                              \
    do {                                                                                             \
        cudaError_t spgx_e_ = (call);                                                                \
        if (spgx_e_ != cudaSuccess) {                                                                \
            ::spgx::set_error(std::string(#call) + ": " + cudaGetErrorString(spgx_e_));              \
            return SPGX_ERR_CUDA;                                                                    \
        }                                                                                            \
    } while (0)

#define SPGX_TRY_STATUS(expr)                 \
    do {                                      \
        spgx_status spgx_s_ = (expr);         \
        if (spgx_s_ != SPGX_OK) return spgx_s_; \
    } while (0)

// Wraps a C ABI body so no C++ exception crosses the boundary.
#define SPGX_GUARD_BEGIN try {
#define SPGX_GUARD_END                                      \
    }                                                       \
    catch (const std::bad_alloc &) {                        \
        ::spgx::set_error("host allocation failed");        \
        return SPGX_ERR_INVALID_ARG;                        \
    }                                                       \
    catch (const std::exception &ex) {                      \
        ::spgx::set_error(ex.what());                       \
        return SPGX_ERR_INVALID_ARG;                        \
    }
