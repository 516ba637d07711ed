// Kernel timing hooks (see evx_prof.cu).
#pragma once

#include "evx_common.cuh"

namespace evx {

struct ProfTok {
    int slot;
    cudaEvent_t ev;
};

ProfTok prof_begin(const char* name, cudaStream_t st);
void prof_end(const ProfTok& t, cudaStream_t st);
void count_launch(unsigned n = 1);

// Launch a kernel (or run a library call) bracketed by timing events.
#define EVX_TIMED(name, st, ...)                          \
    do {                                                  \
        ::evx::ProfTok _evx_t = ::evx::prof_begin(name, st); \
        __VA_ARGS__;                                      \
        ::evx::prof_end(_evx_t, st);                      \
    } while (0)

}  // namespace evx
