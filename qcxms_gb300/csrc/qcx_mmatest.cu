// Self-check of the tensor-core GEMM (qcx_mma.cuh) through the C ABI: one CTA
// multiplies host matrices. Used by the tests to compare the split-TF32
// tcgen05 product with an FP64 reference product before the SCC kernel relies
// on it, and by the profiles to time the product alone.
#include <cuda_runtime.h>

#include <string>

#include "../../include/qcxgpu.h"
#include "qcx_kernels.h"
#include "qcx_mma.cuh"

namespace qcx {

constexpr int kMmaTestThreads = 512;

__global__ void __launch_bounds__(kMmaTestThreads) k_mma_selftest(int M, int N, int K, const float* A, int ta,
                                                                   const float* B, int tb, float* C, int reps,
                                                                   int* ok) {
  extern __shared__ __align__(1024) char smem[];
  __shared__ uint32_t tmem_slot;
  __shared__ __align__(8) uint64_t mbar;
  MmaCtx c;
  mma_setup(c, &tmem_slot, &mbar, smem);
  const int lda = ta ? M : K, ldb = tb ? K : N;
  for (int r = 0; r < reps; ++r) mma_gemm_tf32(c, M, N, K, A, lda, ta != 0, B, ldb, tb != 0, C, N);
  mma_teardown(c);
  if (threadIdx.x == 0) *ok = c.ok;
}

}  // namespace qcx

extern "C" int qcx_mma_selftest(int M, int N, int K, const float* A, int ta, const float* B, int tb, float* C,
                                int reps, float* ms) {
  using namespace qcx;
  if (M < 1 || M > 512 || N < 1 || N > 256 || K < 1 || !A || !B || !C || reps < 1) {
    set_last_error("qcx_mma_selftest: 1 <= M <= 512, 1 <= N <= 256, K >= 1, reps >= 1");
    return -1;
  }
  float *dA = nullptr, *dB = nullptr, *dC = nullptr;
  int* dok = nullptr;
  cudaError_t e = cudaMalloc(&dA, sizeof(float) * M * K);
  if (e == cudaSuccess) e = cudaMalloc(&dB, sizeof(float) * K * N);
  if (e == cudaSuccess) e = cudaMalloc(&dC, sizeof(float) * M * N);
  if (e == cudaSuccess) e = cudaMalloc(&dok, sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpy(dA, A, sizeof(float) * M * K, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dB, B, sizeof(float) * K * N, cudaMemcpyHostToDevice);
  const int smem = mma_stage_bytes(256);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_mma_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  if (e == cudaSuccess) e = cudaEventCreate(&t0);
  if (e == cudaSuccess) e = cudaEventCreate(&t1);
  if (e == cudaSuccess) {
    cudaEventRecord(t0);
    k_mma_selftest<<<1, kMmaTestThreads, smem>>>(M, N, K, dA, ta, dB, tb, dC, reps, dok);
    cudaEventRecord(t1);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaEventSynchronize(t1);
  if (e == cudaSuccess && ms) e = cudaEventElapsedTime(ms, t0, t1);
  int ok = 0;
  if (e == cudaSuccess) e = cudaMemcpy(C, dC, sizeof(float) * M * N, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&ok, dok, sizeof(int), cudaMemcpyDeviceToHost);
  if (t0) cudaEventDestroy(t0);
  if (t1) cudaEventDestroy(t1);
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dC);
  cudaFree(dok);
  if (e != cudaSuccess) {
    set_last_error(std::string("qcx_mma_selftest: ") + cudaGetErrorString(e));
    return -1;
  }
  if (!ok) {
    set_last_error("qcx_mma_selftest: the tensor-core completion wait ran out");
    return -2;
  }
  return 0;
}
