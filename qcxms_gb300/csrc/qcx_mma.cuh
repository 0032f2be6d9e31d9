// CTA-wide GEMM on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// C[M][N] = A[M][K] * B[K][N] for N <= 256, any M and K (tiles of 128 rows), FP32 in and out,
// computed as split-TF32: every operand is split into a TF32 head and an FP32
// tail (x = hi + lo, lo exact), and the product accumulates hi*hi + hi*lo + lo*hi
// (the lo*lo term is below FP32 rounding) in FP32 in tensor memory. The result
// carries about 21 significant bits, which is what the FP32 SCC iterations need.
//
// Operands are staged chunk by chunk (16 values of K) into shared memory in the
// canonical K-major layout without swizzle: core matrices of 8 rows x 16 bytes
// (4 TF32 values), the next core matrix along K 128 bytes on (leading byte
// offset), the next group of 8 rows 512 bytes on (stride byte offset). One
// elected thread issues tcgen05.mma.cta_group::1.kind::tf32 for the 2 K-steps
// of 8 and the 3 split products, commits to an mbarrier, and every thread waits
// on it with a bounded number of polls. The accumulator (128 lanes x N columns)
// is read back with tcgen05.ld by the first four warps' lane quarters.
#pragma once
#include <cstdint>

namespace qcx {

// staging bytes for one K chunk: A hi/lo (128 x 16) and B hi/lo (nmax x 16)
constexpr int kMmaKc = 16;
__host__ __device__ constexpr int mma_stage_bytes(int nmax) { return 2 * 128 * kMmaKc * 4 + 2 * nmax * kMmaKc * 4; }

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: K-major, no swizzle, descriptor version 1
__device__ __forceinline__ uint64_t mma_sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo & 0x3FFFFu) >> 4) << 16;
  d |= (uint64_t)((sbo & 0x3FFFFu) >> 4) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// instruction descriptor, kind::tf32: D FP32, A and B TF32, both K-major
__device__ __forceinline__ uint32_t mma_idesc_tf32(int m, int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ float tf32_hi(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

struct MmaCtx {
  uint32_t tmem;    // accumulator base address in tensor memory
  uint64_t* mbar;   // completion barrier (shared memory)
  uint32_t phase;   // parity of the next completion
  char* stage;      // staging buffer, mma_stage_bytes(nmax) bytes, 1024-byte aligned
  int ok;           // 0 after a wait ran out: the caller must not trust the results
};

// Tensor-memory columns of the accumulator (a power of two >= 32): the largest
// N a caller may pass (rounded up to 16), and the MMA's own limit for M = 128
constexpr int kMmaTmemCols = 256;

// Warp 0 allocates the accumulator; the address goes through shared memory.
// Thread 0 initialises the barrier. Call from all threads.
__device__ inline void mma_setup(MmaCtx& c, uint32_t* tmem_slot, uint64_t* mbar, char* stage) {
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(kMmaTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  c.tmem = *tmem_slot;
  c.mbar = mbar;
  c.phase = 0;
  c.stage = stage;
  c.ok = 1;
}

// Warp 0 frees the accumulator. Call from all threads, after the last read.
__device__ inline void mma_teardown(MmaCtx& c) {
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(c.tmem), "r"(kMmaTmemCols));
  }
}

// Wait for the committed MMAs: bounded polling (each try_wait also suspends for
// a while), so a lost arrival ends as c.ok = 0 instead of a hang.
__device__ inline void mma_wait(MmaCtx& c) {
  const uint32_t addr = smem_u32(c.mbar);
  uint32_t done = 0;
  for (int i = 0; i < (1 << 22) && !done; ++i) {
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(addr), "r"(c.phase));
  }
  if (!done) c.ok = 0;
  c.phase ^= 1u;
  asm volatile("tcgen05.fence::after_thread_sync;");
}

// Core-matrix offset (bytes) of element (row r, k) of a staged K chunk
__device__ __forceinline__ int mma_off(int r, int k) {
  return (r >> 3) * (kMmaKc / 4) * 128 + (k >> 2) * 128 + (r & 7) * 16 + (k & 3) * 4;
}

// C = A B with A(i,k) = ta ? A[k*lda + i] : A[i*lda + k] and
// B(k,j) = tb ? B[j*ldb + k] : B[k*ldb + j]; C row-major (ldc), M <= 128,
// N <= 256. All threads call it; blockDim.x must be a multiple of 128.
template <typename TA, typename TB>
__device__ void mma_gemm_tile(MmaCtx& c, int M, int N, int K, const TA* A, int lda, bool ta, const TB* B, int ldb,
                              bool tb, float* C, int ldc) {
  const int Np = (N + 15) & ~15;  // N multiple of 16 for M = 128
  float* a_hi = (float*)c.stage;
  float* a_lo = (float*)(c.stage + 128 * kMmaKc * 4);
  float* b_hi = (float*)(c.stage + 2 * 128 * kMmaKc * 4);
  float* b_lo = (float*)(c.stage + 2 * 128 * kMmaKc * 4 + Np * kMmaKc * 4);
  const uint32_t idesc = mma_idesc_tf32(128, Np);
  const uint32_t sbo = (kMmaKc / 4) * 128, lbo = 128;
  for (int k0 = 0; k0 < K; k0 += kMmaKc) {
    // stage the chunk (zero outside M, N, K)
    for (int e = threadIdx.x; e < 128 * kMmaKc; e += blockDim.x) {
      const int r = e / kMmaKc, k = e - r * kMmaKc, kk = k0 + k;
      float x = 0.0f;
      if (r < M && kk < K) x = (float)(ta ? A[(long long)kk * lda + r] : A[(long long)r * lda + kk]);
      const float h = tf32_hi(x);
      const int o = mma_off(r, k) >> 2;
      a_hi[o] = h;
      a_lo[o] = x - h;
    }
    for (int e = threadIdx.x; e < Np * kMmaKc; e += blockDim.x) {
      int j, k;
      if (tb) {
        j = e / kMmaKc;
        k = e - j * kMmaKc;
      } else {
        k = e / Np;
        j = e - k * Np;
      }
      const int kk = k0 + k;
      float x = 0.0f;
      if (j < N && kk < K) x = (float)(tb ? B[(long long)j * ldb + kk] : B[(long long)kk * ldb + j]);
      const float h = tf32_hi(x);
      const int o = mma_off(j, k) >> 2;
      b_hi[o] = h;
      b_lo[o] = x - h;
    }
    // generic-proxy writes -> visible to the tensor core's async proxy
    asm volatile("fence.proxy.async.shared::cta;");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (threadIdx.x == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t ah = smem_u32(a_hi), al = smem_u32(a_lo), bh = smem_u32(b_hi), bl = smem_u32(b_lo);
      for (int ks = 0; ks < kMmaKc / 8; ++ks) {
        const uint32_t step = ks * 2 * 128;  // 8 TF32 values of K = two core matrices
        const uint64_t dah = mma_sdesc(ah + step, lbo, sbo), dal = mma_sdesc(al + step, lbo, sbo);
        const uint64_t dbh = mma_sdesc(bh + step, lbo, sbo), dbl = mma_sdesc(bl + step, lbo, sbo);
        const uint32_t acc0 = (k0 > 0 || ks > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(c.tmem),
            "l"(dah), "l"(dbh), "r"(idesc), "r"(acc0));
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, 1, 0;\n"
            " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n"
            " tcgen05.mma.cta_group::1.kind::tf32 [%0], %4, %5, %3, p;\n}" ::"r"(c.tmem),
            "l"(dah), "l"(dbl), "r"(idesc), "l"(dal), "l"(dbh));
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(c.mbar)));
    }
    mma_wait(c);  // the staging buffer is reused by the next chunk
  }
  // read the accumulator: warp w takes lanes 32 (w % 4) .. + 31 and every
  // (blockDim.x / 128)-th group of 8 columns
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int quarter = w & 3, nslab = blockDim.x >> 7;
  const int row = quarter * 32 + lane;
  for (int c8 = (w >> 2) * 8; c8 < Np; c8 += nslab * 8) {
    uint32_t v[8];
    const uint32_t taddr = c.tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)c8;
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;");
    if (row < M)
      for (int q = 0; q < 8; ++q)
        if (c8 + q < N) C[(long long)row * ldc + c8 + q] = __uint_as_float(v[q]);
  }
  // the next GEMM may overwrite the accumulator only after every read
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
}

// C = op(A) op(B) for any M: tiles of 128 rows of op(A) and C
template <typename TA, typename TB>
__device__ void mma_gemm_tf32(MmaCtx& c, int M, int N, int K, const TA* A, int lda, bool ta, const TB* B, int ldb,
                              bool tb, float* C, int ldc) {
  for (int m0 = 0; m0 < M; m0 += 128) {
    const int mt = M - m0 < 128 ? M - m0 : 128;
    const TA* Am = ta ? A + m0 : A + (long long)m0 * lda;
    mma_gemm_tile(c, mt, N, K, Am, lda, ta, B, ldb, tb, C + (long long)m0 * ldc, ldc);
  }
}

}  // namespace qcx
