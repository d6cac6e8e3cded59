// Tensor-core trailing update of the complex64 LU (tcgen05), see below.
#include "m25_internal.h"

namespace m25 {

bool lu_tc_available() { return false; }

int lu_gemm_tc(m25_ctx*, zf*, int64_t, int, int, int) {
  set_error("tensor-core LU update not built");
  return M25_ERR_CUDA;
}

}  // namespace m25
