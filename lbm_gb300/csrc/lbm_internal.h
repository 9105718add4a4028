// Internal declarations shared by the translation units of liblbm_gb300.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include "../../include/lbm_gb300.h"

namespace lbm {
// Thread-local last-error message (lbm_last_error_string).
void set_error(const char* fmt, ...);
// Argument checks of an lbm_problem (lbm_api.cu).
int problem_check(const lbm_problem* p, const char* fn);
// Fused engine (lbm_fused.cu).
size_t fused_scratch_bytes(const lbm_problem* p);
int fused_enqueue(const lbm_problem* p, int mode, long long it0, int n_steps, int parity,
                  unsigned flags, bool set_it, cudaStream_t st, cudaEvent_t* ev = nullptr);
int fused_kernels_per_step(const lbm_problem* p, int mode);
int fused_set_it(const lbm_problem* p, long long value, cudaStream_t st);
// FP64 steps it0 + 1 .. it0 + n_steps - 1 along a chain of state slots:
// step m reads states + (m - 1) * stride and writes states + m * stride (no
// drag history).  The arguments are built once for the whole chain.
int fused_enqueue_chain(const lbm_problem* p, long long it0, int n_steps, double* states,
                        long long stride, cudaStream_t st);
}  // namespace lbm

#define LBM_CUDA_CHECK(call, what)                                              \
  do {                                                                          \
    cudaError_t e_ = (call);                                                    \
    if (e_ != cudaSuccess) {                                                    \
      ::lbm::set_error("%s: %s", what, cudaGetErrorString(e_));                 \
      return LBM_ERR_CUDA;                                                      \
    }                                                                           \
  } while (0)
