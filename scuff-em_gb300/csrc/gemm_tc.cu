// gemm_tc.cu -- tensor-core trailing update of the complex-FP32 LU.
#include "bem_math.cuh"
#include "gbem_internal.h"

namespace gbem {

size_t tc_gemm_ws_bytes(int m, int n, int k) { (void)m; (void)n; (void)k; return 0; }

bool tc_gemm_update(cx<float>* C, long long ldc, const cx<float>* A, long long lda, const cx<float>* B, long long ldb,
                    int m, int n, int k, void* ws, size_t ws_bytes, cudaStream_t s, cudaError_t* err) {
  (void)C; (void)ldc; (void)A; (void)lda; (void)B; (void)ldb; (void)m; (void)n; (void)k; (void)ws; (void)ws_bytes; (void)s;
  *err = cudaSuccess;
  return false;
}

}  // namespace gbem
