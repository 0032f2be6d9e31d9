// Self-consistent-charge loop: one CTA per molecule runs the whole SCC
// (potentials, Fock build, generalized eigensolve, Fermi smearing, density,
// Mulliken moments, modified Broyden mixing) without returning to the host,
// so a batch of uneven molecules advances in one launch and molecules that
// converge early simply retire their CTA.
//
// Generalized eigenproblem F C = S C e: S = L L^T (Cholesky, once per
// geometry), X = L^-T, A = X^T F X, cyclic parallel Jacobi on A (round-robin
// pair ordering, n/2 disjoint rotations per round), C = X V. Later iterations
// refine the previous coefficients: B = C^T F C is nearly diagonal, and a
// first-order (GEMM) refinement, exact rotations of hard pairs, or a warm
// Jacobi sweep on B updates them.
#include <atomic>
#include <cfloat>
#include <type_traits>

#include "qcx_batch.cuh"
#include "qcx_kernels.h"
#include "qcx_mma.cuh"

namespace qcx {

// warm FP32 Jacobi sweeps (at most) when the first-order refinement cannot
// update the eigenvectors: a single sweep left errors of order 1e-2 in the
// density of molecules with near-degenerate orbitals at the Fermi level, which
// stalled the FP32 phase (measured on 5-40-atom cations: 43 iterations per
// evaluation with one sweep, 38 with two or three, and fewer stopped
// trajectories). A sweep costs ~n^2 cycles, so molecules above
// QCX_JAC32_WARM2_MAX_NAO AOs take one (collision workload, 18-281 AOs: 907
// trajectory-steps/s with one sweep for every molecule against 818 with two)
#ifndef QCX_JAC32_WARM_SWEEPS
#define QCX_JAC32_WARM_SWEEPS 2
#endif
#ifndef QCX_JAC32_WARM2_MAX_NAO
#define QCX_JAC32_WARM2_MAX_NAO 128
#endif
#ifndef QCX_JAC32_COLD_TOL
#define QCX_JAC32_COLD_TOL 2e-6
#endif
#ifndef QCX_MIXED_SWITCH
#define QCX_MIXED_SWITCH 1e-4
#endif
#ifndef QCX_SCC_THREADS
#define QCX_SCC_THREADS 512
#endif
#ifndef QCX_SCC_MINBLOCKS
#define QCX_SCC_MINBLOCKS 1
#endif
#ifndef QCX_SCC_SMEM_KB
#define QCX_SCC_SMEM_KB 220
#endif
#ifndef QCX_REFINE32_KFAIL
#define QCX_REFINE32_KFAIL 0.1
#endif
#ifndef QCX_REFINE32_PASSES
#define QCX_REFINE32_PASSES 2
#endif
#ifndef QCX_REFINE32_BACKOFF
#define QCX_REFINE32_BACKOFF 6
#endif
#ifndef QCX_REFINE32_KTOL
#define QCX_REFINE32_KTOL 1e-3
#endif
// rounds of exact rotations on the pairs that first-order refinement cannot
// handle, before the refinement gives up and a Jacobi sweep takes over
// items per batch of the Jacobi update loops, and whether the sweep is a
// separate function (its own register allocation; the caller saves its live
// registers around the call, once per sweep)
#ifndef QCX_JAC_UNROLL
#define QCX_JAC_UNROLL 1
#endif
#ifndef QCX_JAC_INLINE
#define QCX_JAC_INLINE __noinline__
#endif
// rounds of the Jacobi sweep with compacted lists of active rotations
#ifndef QCX_JAC_COMPACT
#define QCX_JAC_COMPACT 1
#endif
#ifndef QCX_HARD_ROUNDS
#define QCX_HARD_ROUNDS 6
#endif
// FP32 refinement: pairs of orbitals both further than this from the previous
// Fermi level, on the same side, are not rotated (negative: all pairs rotate).
// Off: the Fermi level of the previous iteration can move by 0.1 Eh in the
// early SCC iterations, so an orbital judged fully occupied may not be, and
// rotating all pairs measured 6-9 % faster on the 256-trajectory workload.
#ifndef QCX_OCC_GAP_KT
#define QCX_OCC_GAP_KT -1.0
#endif
#ifndef QCX_OCC_GAP_ABS
#define QCX_OCC_GAP_ABS 0.0
#endif
// Newton-Schulz steps (at most) after a first-order refinement step in FP64
// and in double-float
#ifndef QCX_NS64_STEPS
#define QCX_NS64_STEPS 4
#endif
// a stalled FP32 phase hands over to the finishing iterations once its
// residual is below this
#ifndef QCX_STALL_HANDOVER
#define QCX_STALL_HANDOVER 1e-3
#endif
// an FP32 phase that has not reached the hand-over residual after this many
// iterations hands over anyway (a hard SCC continues in the accurate arithmetic)
#ifndef QCX_FP32_MAXIT
#define QCX_FP32_MAXIT 1000
#endif
// FP32 products of the FP32 iterations on the tcgen05 tensor cores (split-TF32)
// when the CTA has room to stage them; 0: CUDA cores only
#ifndef QCX_SCC_MMA
#define QCX_SCC_MMA 1
#endif
constexpr int kSccThreads = QCX_SCC_THREADS;
constexpr int kWarps = kSccThreads / 32;

// ---------------------------------------------------------------------------
// CTA helpers
// ---------------------------------------------------------------------------
__device__ inline double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ inline double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Sum K values over the CTA; result valid in all threads. red: K*kWarps doubles.
template <int K>
__device__ void cta_sum(double (&v)[K], double* red) {
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double s = warp_sum(v[k]);
    if (lane == 0) red[k * kWarps + w] = s;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double s = 0.0;
    for (int i = 0; i < kWarps; ++i) s += red[k * kWarps + i];
    v[k] = s;
  }
  __syncthreads();
}

__device__ double cta_max(double v, double* red) {
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  double s = warp_max(v);
  if (lane == 0) red[w] = s;
  __syncthreads();
  double m = red[0];
  for (int i = 1; i < kWarps; ++i) m = fmax(m, red[i]);
  __syncthreads();
  return m;
}

// C[M][N] = op(A) op(B), row-major; inputs converted to ACC on load.
// ta: A is stored K x M; tb: B is stored N x K. 2x2 register tile per thread.
template <typename TA, typename TB, typename TC, typename ACC>
__device__ void cta_gemm(int M, int N, int K, const TA* A, int lda, bool ta, const TB* B, int ldb, bool tb, TC* C,
                         int ldc) {
  int tilesM = (M + 1) / 2, tilesN = (N + 1) / 2;
  for (int t = threadIdx.x; t < tilesM * tilesN; t += blockDim.x) {
    int i0 = (t / tilesN) * 2, j0 = (t % tilesN) * 2;
    ACC c00 = 0, c01 = 0, c10 = 0, c11 = 0;
    bool i1ok = i0 + 1 < M, j1ok = j0 + 1 < N;
    int i1 = i1ok ? i0 + 1 : i0, j1 = j1ok ? j0 + 1 : j0;
    for (int k = 0; k < K; ++k) {
      ACC a0 = (ACC)(ta ? A[(long long)k * lda + i0] : A[(long long)i0 * lda + k]);
      ACC a1 = (ACC)(ta ? A[(long long)k * lda + i1] : A[(long long)i1 * lda + k]);
      ACC b0 = (ACC)(tb ? B[(long long)j0 * ldb + k] : B[(long long)k * ldb + j0]);
      ACC b1 = (ACC)(tb ? B[(long long)j1 * ldb + k] : B[(long long)k * ldb + j1]);
      c00 = fma(a0, b0, c00);
      c01 = fma(a0, b1, c01);
      c10 = fma(a1, b0, c10);
      c11 = fma(a1, b1, c11);
    }
    C[(long long)i0 * ldc + j0] = (TC)c00;
    if (j1ok) C[(long long)i0 * ldc + j1] = (TC)c01;
    if (i1ok) {
      C[(long long)i1 * ldc + j0] = (TC)c10;
      if (j1ok) C[(long long)i1 * ldc + j1] = (TC)c11;
    }
  }
}

// Products of the FP32 iterations: on the tensor cores (qcx_mma.cuh, split-TF32)
// when the CTA holds a tcgen05 context and N fits the accumulator, else on the
// CUDA cores. FP64 products always take the CUDA cores.
template <typename T>
__device__ __forceinline__ void gemm_t(MmaCtx* mc, int M, int N, int K, const T* A, int lda, bool ta, const T* B,
                                       int ldb, bool tb, T* C, int ldc) {
  if constexpr (std::is_same<T, float>::value) {
    if (mc && ((N + 15) & ~15) <= kMmaTmemCols) {
      mma_gemm_tf32(*mc, M, N, K, A, lda, ta, B, ldb, tb, C, ldc);
      return;
    }
  }
  cta_gemm<T, T, T, T>(M, N, K, A, lda, ta, B, ldb, tb, C, ldc);
}

// ---------------------------------------------------------------------------
// shared-memory layout
// ---------------------------------------------------------------------------
struct SccShared {
  int* ao_sh;      // [n] local shell of each AO
  int* ao_at;      // [n] local atom of each AO
  int* perm;       // [np]
  int* rp;         // [np/2] rotation pair p
  int* rq;         // [np/2] rotation pair q
  int* rskip;      // [np/2] 1 if the rotation is the identity
  double* rc;      // [np/2]
  double* rs;      // [np/2]
  double* mom;     // [10][n] per-AO moment partials
  double* red;     // [16*kWarps] reductions
  double* scal;    // [32] scalars
  double* jac;     // Jacobi region (A, maybe V)
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

__host__ __device__ inline size_t scc_fixed_bytes(int n) {
  int np = n + (n & 1);
  size_t b = 0;
  b += align16(sizeof(int) * n) * 2;
  b += align16(sizeof(int) * np);
  b += align16(sizeof(int) * (np / 2)) * 3;
  b += align16(sizeof(double) * (np / 2)) * 2;
  b += align16(sizeof(double) * 10 * n);
  b += align16(sizeof(double) * 16 * kWarps);
  b += align16(sizeof(double) * 32);
  return b;
}

constexpr size_t kSmemCap = QCX_SCC_SMEM_KB * 1024;

// Jacobi storage mode for a molecule with n AOs given the granted dynamic
// shared memory: 0 = A and V in shared memory, 1 = A shared / V global,
// 2 = both global (L2 resident).
__host__ __device__ inline int jacobi_mode(int n, size_t granted) {
  int np = n + (n & 1);
  size_t fixed = scc_fixed_bytes(n);
  size_t m2 = sizeof(double) * (size_t)np * np;
  if (fixed + 2 * m2 <= granted) return 0;
  if (fixed + m2 <= granted) return 1;
  return 2;
}

size_t scc_smem_bytes(int max_nao, int precision) {
  (void)precision;
  int n = max_nao;
  int np = n + (n & 1);
  // both Jacobi matrices, then the staging buffer of the tensor-core products
  size_t want = ((scc_fixed_bytes(n) + 2 * sizeof(double) * (size_t)np * np + 127) & ~(size_t)127) +
                (size_t)mma_stage_bytes((n + 15) & ~15);
  return want < kSmemCap ? want : kSmemCap;
}

__device__ SccShared carve(char* base, int n) {
  int np = n + (n & 1);
  SccShared s;
  size_t o = 0;
  s.ao_sh = (int*)(base + o); o += align16(sizeof(int) * n);
  s.ao_at = (int*)(base + o); o += align16(sizeof(int) * n);
  s.perm = (int*)(base + o); o += align16(sizeof(int) * np);
  s.rp = (int*)(base + o); o += align16(sizeof(int) * (np / 2));
  s.rq = (int*)(base + o); o += align16(sizeof(int) * (np / 2));
  s.rskip = (int*)(base + o); o += align16(sizeof(int) * (np / 2));
  s.rc = (double*)(base + o); o += align16(sizeof(double) * (np / 2));
  s.rs = (double*)(base + o); o += align16(sizeof(double) * (np / 2));
  s.mom = (double*)(base + o); o += align16(sizeof(double) * 10 * n);
  s.red = (double*)(base + o); o += align16(sizeof(double) * 16 * kWarps);
  s.scal = (double*)(base + o); o += align16(sizeof(double) * 32);
  s.jac = (double*)(base + o);
  return s;
}

// ---------------------------------------------------------------------------
// electrostatic + dispersion potentials of a moment vector x
// ---------------------------------------------------------------------------
struct MolView {
  const DevBatch* bt;
  MolDesc md;
  VecLayout vl;
  double* vec;
  const int* Z;      // Z of local atoms (pointer offset)
  const double* xyz;  // local atoms
};

// energies: [0]=ies [1]=e3 [2]=aes [3]=axc [4]=disp
__device__ void potentials(const MolView& mv, const double* x, double* en, double* red) {
  const Params& P = *mv.bt->prm;
  const int nat = mv.md.nat, nsh = mv.md.nsh;
  const double* qsh = x;
  const double* dp = x + nsh;
  const double* qp = x + nsh + 3 * nat;
  double* vec = mv.vec;
  double* qat = vec + mv.vl.qat;
  double* vat = vec + mv.vl.vat;
  double* vsh = vec + mv.vl.vsh;
  double* vdp = vec + mv.vl.vdp;
  double* vqp = vec + mv.vl.vqp;
  double* wq = vec + mv.vl.wq;    // [nat][kMaxRef] gw zeta(q)
  double* dwq = vec + mv.vl.dwq;  // [nat][kMaxRef] gw dzeta/dq
  double* zq = vec + mv.vl.zq;    // [nat][kMaxRef] zeta(q)
  const double* gam = vec + mv.vl.gam;
  const double* gdm = vec + mv.vl.gdisp;
  const double* f3m = vec + mv.vl.f3;
  const double* f5m = vec + mv.vl.f5;
  const int* sh_k = mv.bt->sh_k + mv.md.sh_off;
  const int* sh_atom = mv.bt->sh_atom + mv.md.sh_off;
  const int aoff = mv.md.atom_off;
  // atomic charges and the charge scaling of every D4 reference (edisp /
  // disppot, src/dftd4.f90:807-1034)
  for (int a = threadIdx.x; a < nat; a += blockDim.x) {
    double q = 0.0;
    for (int s = 0; s < nsh; ++s)
      if (sh_atom[s] - aoff == a) q += qsh[s];
    qat[a] = q;
    const int z = mv.Z[a];
    const double* gw = mv.bt->w4 + (long long)(aoff + a) * kMaxRef;
    for (int i = 0; i < kMaxRef; ++i) {
      double zt = 0.0, dzt = 0.0;
      if (i < P.d4_refn[z]) d4_zeta(P, z, i, q, zt, dzt);
      zq[kMaxRef * a + i] = zt;
      wq[kMaxRef * a + i] = gw[i] * zt;
      dwq[kMaxRef * a + i] = gw[i] * dzt;
    }
  }
  __syncthreads();
  double e[5] = {0, 0, 0, 0, 0};
  // atom-resolved terms. First the on-atom multipole XC kernels (which also
  // initialise the potentials), then the pair terms spread over all threads
  // (atom pairs b-major, so that consecutive threads add into different atoms).
  for (int a = threadIdx.x; a < nat; a += blockDim.x) {
    const double* ma = dp + 3 * a;
    const double* ta = qp + 6 * a;
    int z = mv.Z[a];
    double fd = P.aes_dk[z], fq = P.aes_qk[z];
    e[3] += fd * (ma[0] * ma[0] + ma[1] * ma[1] + ma[2] * ma[2]) +
            fq * (ta[0] * ta[0] + ta[1] * ta[1] + ta[2] * ta[2] + 2.0 * (ta[3] * ta[3] + ta[4] * ta[4] + ta[5] * ta[5]));
    vat[a] = 0.0;
    for (int k = 0; k < 3; ++k) vdp[3 * a + k] = 2.0 * fd * ma[k];
    for (int q = 0; q < 3; ++q) vqp[6 * a + q] = 2.0 * fq * ta[q];
    for (int q = 3; q < 6; ++q) vqp[6 * a + q] = 4.0 * fq * ta[q];
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < nat * nat; idx += blockDim.x) {
    int b = idx / nat, a = idx - b * nat;
    if (b == a) continue;
    const double* ma = dp + 3 * a;
    const double* ta = qp + 6 * a;
    double r[3] = {mv.xyz[3 * a] - mv.xyz[3 * b], mv.xyz[3 * a + 1] - mv.xyz[3 * b + 1],
                   mv.xyz[3 * a + 2] - mv.xyz[3 * b + 2]};
    double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    double f3 = f3m[a * nat + b], f5 = f5m[a * nat + b];
    const double* mb = dp + 3 * b;
    const double* tb = qp + 6 * b;
    double mar = ma[0] * r[0] + ma[1] * r[1] + ma[2] * r[2];
    double mbr = mb[0] * r[0] + mb[1] * r[1] + mb[2] * r[2];
    double mab = ma[0] * mb[0] + ma[1] * mb[1] + ma[2] * mb[2];
    double rr[6] = {r[0] * r[0], r[1] * r[1], r[2] * r[2], 2 * r[0] * r[1], 2 * r[0] * r[2], 2 * r[1] * r[2]};
    double rta = 0, rtb = 0;
    for (int q = 0; q < 6; ++q) {
      rta += ta[q] * rr[q];
      rtb += tb[q] * rr[q];
    }
    // dispersion: E_ab = -g_ab sum_ij wq_ai wq_bj C6_ij; the a-side charge derivative
    const double gd = gdm[a * nat + b];
    const int za = mv.Z[a], zb = mv.Z[b];
    double c6, dc6;
    d4_c6_pair(P, za, wq + kMaxRef * a, dwq + kMaxRef * a, zb, wq + kMaxRef * b, c6, dc6);
    e[2] += 0.5 * (f3 * (qat[a] * mbr - qat[b] * mar) + f5 * (qat[a] * rtb + qat[b] * rta + mab * r2 - 3.0 * mar * mbr));
    e[4] += -0.5 * gd * c6;
    atomicAdd(&vat[a], f3 * mbr + f5 * rtb - gd * dc6);
    for (int k = 0; k < 3; ++k) atomicAdd(&vdp[3 * a + k], -f3 * qat[b] * r[k] + f5 * (mb[k] * r2 - 3.0 * mbr * r[k]));
    for (int q = 0; q < 6; ++q) atomicAdd(&vqp[6 * a + q], f5 * qat[b] * rr[q]);
  }
  __syncthreads();
  // shell-resolved isotropic electrostatics and third order
  for (int s = threadIdx.x; s < nsh; s += blockDim.x) {
    double v = 0.0;
    for (int t = 0; t < nsh; ++t) v += gam[s * nsh + t] * qsh[t];
    int a = sh_atom[s] - aoff;
    double g3 = P.gamma3[mv.Z[a]][sh_k[s]];
    e[0] += 0.5 * qsh[s] * v;
    e[1] += g3 * qsh[s] * qsh[s] * qsh[s] / 3.0;
    vsh[s] = v + g3 * qsh[s] * qsh[s] + vat[a];
  }
  cta_sum<5>(e, red);
  for (int k = 0; k < 5; ++k) en[k] = e[k];
}

// ---------------------------------------------------------------------------
// FP32 potentials for the FP32 iterations: the potential terms of
// potentials() (no energies, which only the FP64 convergence test uses), in
// FP32, written to shared memory for the FP32 Fock build, with shared-memory
// atomics for the pair sums. Layout of v32: shell potentials [nsh], dipole
// [3 nat] and quadrupole [6 nat] potentials, atom positions [3 nat], then
// scratch (dipoles, quadrupoles, charges, atom potentials); the D4 reference
// weights times the charge scaling and its derivative go to the vector block
// (as FP32, in the space of the FP64 weights, which the FP64 potentials rewrite).
// Returns false, writing nothing, when the scratch (nsh + 23 nat floats)
// exceeds the 20 n floats available.
// ---------------------------------------------------------------------------
__device__ bool potentials32(const MolView& mv, const double* x, float* v32, int n) {
  const Params& P = *mv.bt->prm;
  const int nat = mv.md.nat, nsh = mv.md.nsh;
  if (nsh + 23 * nat > 20 * n) return false;
  float* vs32 = v32;
  float* vd32 = vs32 + nsh;
  float* vq32 = vd32 + 3 * nat;
  float* r32 = vq32 + 6 * nat;
  float* m32 = r32 + 3 * nat;
  float* t32 = m32 + 3 * nat;
  float* q32 = t32 + 6 * nat;
  float* va32 = q32 + nat;
  const double* qsh = x;
  const double* dp = x + nsh;
  const double* qp = x + nsh + 3 * nat;
  double* vec = mv.vec;
  float* wq32 = (float*)(vec + mv.vl.wq);  // [nat][kMaxRef]
  float* dwq32 = wq32 + kMaxRef * nat;     // [nat][kMaxRef]
  const double* gam = vec + mv.vl.gam;
  const double* gdm = vec + mv.vl.gdisp;
  const double* f3m = vec + mv.vl.f3;
  const double* f5m = vec + mv.vl.f5;
  const int* sh_k = mv.bt->sh_k + mv.md.sh_off;
  const int* sh_atom = mv.bt->sh_atom + mv.md.sh_off;
  const int aoff = mv.md.atom_off;
  for (int a = threadIdx.x; a < nat; a += blockDim.x) {
    double q = 0.0;
    for (int t = 0; t < nsh; ++t)
      if (sh_atom[t] - aoff == a) q += qsh[t];
    const int z = mv.Z[a];
    const double* gw = mv.bt->w4 + (long long)(aoff + a) * kMaxRef;
    for (int i = 0; i < kMaxRef; ++i) {
      double zt = 0.0, dzt = 0.0;
      if (i < P.d4_refn[z]) d4_zeta(P, z, i, q, zt, dzt);
      wq32[kMaxRef * a + i] = (float)(gw[i] * zt);
      dwq32[kMaxRef * a + i] = (float)(gw[i] * dzt);
    }
    q32[a] = (float)q;
    va32[a] = 0.f;
    const float fd = (float)P.aes_dk[mv.Z[a]], fq = (float)P.aes_qk[mv.Z[a]];
    for (int k = 0; k < 3; ++k) {
      r32[3 * a + k] = (float)mv.xyz[3 * a + k];
      m32[3 * a + k] = (float)dp[3 * a + k];
      vd32[3 * a + k] = 2.f * fd * m32[3 * a + k];
    }
    for (int c = 0; c < 6; ++c) {
      t32[6 * a + c] = (float)qp[6 * a + c];
      vq32[6 * a + c] = (c < 3 ? 2.f : 4.f) * fq * t32[6 * a + c];
    }
  }
  __syncthreads();
  // pair terms (atom pairs b-major, so that consecutive threads add into different atoms)
  for (int idx = threadIdx.x; idx < nat * nat; idx += blockDim.x) {
    int b = idx / nat, a = idx - b * nat;
    if (b == a) continue;
    float r[3] = {r32[3 * a] - r32[3 * b], r32[3 * a + 1] - r32[3 * b + 1], r32[3 * a + 2] - r32[3 * b + 2]};
    float r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    float f3 = (float)f3m[a * nat + b], f5 = (float)f5m[a * nat + b], gd = (float)gdm[a * nat + b];
    const float dc6 = d4_c6(P, mv.Z[a], dwq32 + kMaxRef * a, mv.Z[b], wq32 + kMaxRef * b);
    const float* mb = m32 + 3 * b;
    const float* tb = t32 + 6 * b;
    float mbr = mb[0] * r[0] + mb[1] * r[1] + mb[2] * r[2];
    float rr[6] = {r[0] * r[0], r[1] * r[1], r[2] * r[2], 2.f * r[0] * r[1], 2.f * r[0] * r[2], 2.f * r[1] * r[2]};
    float rtb = 0.f;
    for (int c = 0; c < 6; ++c) rtb += tb[c] * rr[c];
    const float qb = q32[b];
    atomicAdd(&va32[a], f3 * mbr + f5 * rtb - gd * dc6);
    for (int k = 0; k < 3; ++k) atomicAdd(&vd32[3 * a + k], -f3 * qb * r[k] + f5 * (mb[k] * r2 - 3.f * mbr * r[k]));
    for (int c = 0; c < 6; ++c) atomicAdd(&vq32[6 * a + c], f5 * qb * rr[c]);
  }
  __syncthreads();
  // shell-resolved isotropic electrostatics and third order
  for (int t = threadIdx.x; t < nsh; t += blockDim.x) {
    double v = 0.0;
    for (int u = 0; u < nsh; ++u) v += gam[t * nsh + u] * qsh[u];
    int a = sh_atom[t] - aoff;
    double g3 = P.gamma3[mv.Z[a]][sh_k[t]];
    vs32[t] = (float)(v + g3 * qsh[t] * qsh[t]) + va32[a];
  }
  __syncthreads();
  return true;
}

// s != 0 for a rotation sine that is either exactly +0 (a skipped rotation)
// or nonzero, tested on the bit pattern: an FP64 compare would run at the FP64 rate
__device__ __forceinline__ bool nonzero(float s) { return __float_as_int(s) != 0; }
__device__ __forceinline__ bool nonzero(double s) { return __double_as_longlong(s) != 0; }

// ---------------------------------------------------------------------------
// cyclic parallel Jacobi on the symmetric np x np matrix A (lda = np).
// Vt (ld = np) holds eigenvectors as rows; with warm = false it starts as the
// identity, with warm = true it keeps its rows (a previous orthonormal basis in
// which A was expressed) and the rotations are accumulated onto them.
// Rounds use the round-robin pairing: n/2 disjoint (p,q) rotations each.
// Returns the number of sweeps, or -1 if max_sweeps were not enough.
// ---------------------------------------------------------------------------
template <typename T>
__device__ QCX_JAC_INLINE int jacobi(T* A, T* Vt, int n, bool warm, double reltol, SccShared& sh, int max_sweeps) {
  const int np = n + (n & 1);
  const int half = np / 2;
  const int m = np - 1;
  for (int i = threadIdx.x; i < np * np; i += blockDim.x) {
    int r = i / np, c = i % np;
    if (!warm || r >= n || c >= n) Vt[i] = (r == c) ? T(1) : T(0);
    if (r >= n || c >= n) A[i] = T(0);
  }
  __syncthreads();
  double amax = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) amax = fmax(amax, fabs((double)A[i * np + i]));
  amax = cta_max(amax, sh.red);
  const T tol = (T)(reltol * fmax(1.0, amax));
  // rotations below a tenth of the tolerance are skipped (threshold Jacobi);
  // they cannot change the result at the tolerance level
  const T tiny = (T)(0.1 * reltol * fmax(1.0, amax));
  // quadratic convergence: once a sweep starts below sqrt(tol * scale), one
  // more sweep reaches tol, so that sweep is the last and needs no check sweep
  const double last_below = sqrt(reltol) * fmax(1.0, amax);
  bool last = false;
  // rotation table of a round: (p, q) pairs and (c, s), s == 0 for a skipped
  // rotation (rp/rq and rc/rs are contiguous, so they hold half int2 / T2)
  using T2 = typename std::conditional<sizeof(T) == 4, float2, double2>::type;
  int2* pq = (int2*)sh.rp;
  T2* csr = (T2*)sh.rc;
  // per-thread start of the block items (k1, k2) and of the row items (k, j);
  // items advance by blockDim.x, i.e. by (dk1, dk2) and (dk, dj)
  const int b1 = threadIdx.x / half, b2 = threadIdx.x - b1 * half;
  const int db1 = blockDim.x / half, db2 = blockDim.x - db1 * half;
  const int v1 = threadIdx.x / np, v2 = threadIdx.x - v1 * np;
  const int dv1 = blockDim.x / np, dv2 = blockDim.x - dv1 * np;
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    T offmax = 0;
#if QCX_JAC_COMPACT
    // (FP64 sweeps only: most rotations of an FP32 warm sweep are active, and
    // there the list building costs more than the skipped items save)
    if (sizeof(T) == 8 && half <= (int)blockDim.x) {
      // Rounds with compacted rotation lists: the parameter phase also sorts the
      // rotations into active (s != 0) and skipped ones (warp ballots and a
      // prefix over the warps), and the update touches only the 2x2 blocks and
      // coefficient rows that an active rotation changes.
      const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
      int* act = sh.rskip;        // [half] active rotations of the round
      int* inact = sh.perm;       // [half] skipped rotations
      int* wcnt = (int*)sh.red;   // [2 kWarps] per-warp counts
      for (int r = 0; r < m; ++r) {
        bool on = false;
        const int k = threadIdx.x;
        if (k < half) {
          int p, q;
          if (k == 0) {
            p = m;
            q = r;
          } else {
            p = r + k;
            if (p >= m) p -= m;
            q = r - k;
            if (q < 0) q += m;
          }
          if (p > q) {
            int t = p;
            p = q;
            q = t;
          }
          T apq = A[p * np + q];
          T aa = apq < T(0) ? -apq : apq;
          offmax = aa > offmax ? aa : offmax;
          T c = 1, s = 0;
          if (aa > tiny) {
            T app = A[p * np + p], aqq = A[q * np + q];
            T theta = (aqq - app) / (T(2) * apq);
            T at = theta < T(0) ? -theta : theta;
            T t = (theta >= T(0) ? T(1) : T(-1)) / (at + sqrt(T(1) + theta * theta));
            c = T(1) / sqrt(T(1) + t * t);
            s = t * c;
          }
          pq[k] = make_int2(p, q);
          T2 cs;
          cs.x = c;
          cs.y = s;
          csr[k] = cs;
          on = nonzero(s);
        }
        const unsigned ba = __ballot_sync(0xffffffffu, on);
        const unsigned bi = __ballot_sync(0xffffffffu, !on && k < half);
        if (lane == 0) {
          wcnt[wid] = __popc(ba);
          wcnt[kWarps + wid] = __popc(bi);
        }
        __syncthreads();
        int offa = 0, offi = 0, na = 0, ni = 0;
        for (int w2 = 0; w2 < kWarps; ++w2) {
          const int ca = wcnt[w2], ci = wcnt[kWarps + w2];
          if (w2 < wid) {
            offa += ca;
            offi += ci;
          }
          na += ca;
          ni += ci;
        }
        const unsigned lt = (1u << lane) - 1u;
        if (on) act[offa + __popc(ba & lt)] = k;
        else if (k < half) inact[offi + __popc(bi & lt)] = k;
        __syncthreads();
        if (na == 0) continue;  // nothing changes this round (uniform)
        // blocks in the rows of an active rotation (all columns), then blocks in
        // the rows of a skipped rotation and the columns of an active one
        const int tot1 = na * half, tot2 = ni * na;
        for (int e = threadIdx.x; e < tot1 + tot2; e += blockDim.x) {
          int k1, k2;
          if (e < tot1) {
            const int a1 = e / half;
            k1 = act[a1];
            k2 = e - a1 * half;
          } else {
            const int f = e - tot1, i1 = f / na;
            k1 = inact[i1];
            k2 = act[f - i1 * na];
          }
          const T2 r1 = csr[k1], r2 = csr[k2];
          const int2 e1 = pq[k1], e2 = pq[k2];
          T* row_p = A + e1.x * np;
          T* row_q = A + e1.y * np;
          T a = row_p[e2.x], b = row_p[e2.y], c = row_q[e2.x], d = row_q[e2.y];
          T ra = r1.x * a - r1.y * c, rb = r1.x * b - r1.y * d;
          T rc = r1.y * a + r1.x * c, rd = r1.y * b + r1.x * d;
          row_p[e2.x] = r2.x * ra - r2.y * rb;
          row_p[e2.y] = r2.y * ra + r2.x * rb;
          row_q[e2.x] = r2.x * rc - r2.y * rd;
          row_q[e2.y] = r2.y * rc + r2.x * rd;
        }
        for (int e = threadIdx.x; e < na * np; e += blockDim.x) {
          const int a1 = e / np, j = e - a1 * np;
          const int kk = act[a1];
          const T2 rr = csr[kk];
          const int2 ee = pq[kk];
          T vp = Vt[ee.x * np + j], vq = Vt[ee.y * np + j];
          Vt[ee.x * np + j] = rr.x * vp - rr.y * vq;
          Vt[ee.y * np + j] = rr.y * vp + rr.x * vq;
        }
        __syncthreads();
      }
    } else
#endif
    {
    for (int r = 0; r < m; ++r) {
      for (int k = threadIdx.x; k < half; k += blockDim.x) {
        int p, q;
        if (k == 0) {
          p = m;
          q = r;
        } else {
          p = r + k;
          if (p >= m) p -= m;
          q = r - k;
          if (q < 0) q += m;
        }
        if (p > q) {
          int t = p;
          p = q;
          q = t;
        }
        T apq = A[p * np + q];
        T aa = apq < T(0) ? -apq : apq;
        offmax = aa > offmax ? aa : offmax;
        T c = 1, s = 0;
        if (aa > tiny) {
          T app = A[p * np + p], aqq = A[q * np + q];
          T theta = (aqq - app) / (T(2) * apq);
          T at = theta < T(0) ? -theta : theta;
          T t = (theta >= T(0) ? T(1) : T(-1)) / (at + sqrt(T(1) + theta * theta));
          c = T(1) / sqrt(T(1) + t * t);
          s = t * c;
        }
        pq[k] = make_int2(p, q);
        T2 cs;
        cs.x = c;
        cs.y = s;
        csr[k] = cs;
      }
      __syncthreads();
      // One fused phase per round: every 2x2 block A[{p1,q1}][{p2,q2}] of a pair
      // of pairs becomes R1 * block * R2^T (each element belongs to exactly one
      // block), and the rows p,q of Vt are rotated by R.
      // Items are taken U at a time with all their shared-memory loads issued
      // before any use, so that the latencies overlap (a round is otherwise
      // bound by one dependent load chain per item).
      constexpr int U = sizeof(T) == 4 ? QCX_JAC_UNROLL : 2;
      for (int k1 = b1, k2 = b2; k1 < half;) {
        int ka[U], kb[U];
        bool ok[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          ok[u] = k1 < half;
          ka[u] = ok[u] ? k1 : 0;
          kb[u] = k2;
          k1 += db1;
          k2 += db2;
          if (k2 >= half) {
            k2 -= half;
            ++k1;
          }
        }
        T2 r1[U], r2[U];
        int2 e1[U], e2[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          r1[u] = csr[ka[u]];
          r2[u] = csr[kb[u]];
          e1[u] = pq[ka[u]];
          e2[u] = pq[kb[u]];
        }
        T a[U], b[U], c[U], d[U];
        bool act[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          act[u] = ok[u] && (nonzero(r1[u].y) || nonzero(r2[u].y));
          if (act[u]) {
            a[u] = A[e1[u].x * np + e2[u].x];
            b[u] = A[e1[u].x * np + e2[u].y];
            c[u] = A[e1[u].y * np + e2[u].x];
            d[u] = A[e1[u].y * np + e2[u].y];
          }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          if (act[u]) {
            // rows: R1 = [[c1,-s1],[s1,c1]]; columns: multiply by R2^T
            T ra = r1[u].x * a[u] - r1[u].y * c[u], rb = r1[u].x * b[u] - r1[u].y * d[u];
            T rc = r1[u].y * a[u] + r1[u].x * c[u], rd = r1[u].y * b[u] + r1[u].x * d[u];
            A[e1[u].x * np + e2[u].x] = r2[u].x * ra - r2[u].y * rb;
            A[e1[u].x * np + e2[u].y] = r2[u].y * ra + r2[u].x * rb;
            A[e1[u].y * np + e2[u].x] = r2[u].x * rc - r2[u].y * rd;
            A[e1[u].y * np + e2[u].y] = r2[u].y * rc + r2[u].x * rd;
          }
        }
      }
      for (int k = v1, j = v2; k < half;) {
        int kk[U], jj[U];
        bool ok[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          ok[u] = k < half;
          kk[u] = ok[u] ? k : 0;
          jj[u] = j;
          k += dv1;
          j += dv2;
          if (j >= np) {
            j -= np;
            ++k;
          }
        }
        T2 rr[U];
        int2 e[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          rr[u] = csr[kk[u]];
          e[u] = pq[kk[u]];
        }
        T vp[U], vq[U];
        bool act[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          act[u] = ok[u] && nonzero(rr[u].y);
          if (act[u]) {
            vp[u] = Vt[e[u].x * np + jj[u]];
            vq[u] = Vt[e[u].y * np + jj[u]];
          }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          if (act[u]) {
            Vt[e[u].x * np + jj[u]] = rr[u].x * vp[u] - rr[u].y * vq[u];
            Vt[e[u].y * np + jj[u]] = rr[u].y * vp[u] + rr[u].x * vq[u];
          }
        }
      }
      __syncthreads();
    }
    }
    double om = cta_max((double)offmax, sh.red);
    if (om <= (double)tol || last) return sweep + 1;
    if (om <= last_below) last = true;
  }
  return -1;
}

// ---------------------------------------------------------------------------
// Fermi level by safeguarded Newton/bisection (one warp); returns -T S.
// ---------------------------------------------------------------------------
__device__ double fermi_warp(int n, const double* eps, double nel, double kT, double* focc, double* efermi,
                             double rtol = 1e-13, double mu_guess = 0.0, bool have_guess = false) {
  int lane = threadIdx.x & 31;
  if (nel <= 0.0) {
    for (int i = lane; i < n; i += 32) focc[i] = 0.0;
    *efermi = eps[0];
    return 0.0;
  }
  if (nel >= 2.0 * n) {
    for (int i = lane; i < n; i += 32) focc[i] = 2.0;
    *efermi = eps[n - 1];
    return 0.0;
  }
  int ho = (int)ceil(nel / 2.0) - 1;
  if (ho < 0) ho = 0;
  int lu = ho + 1 < n ? ho + 1 : n - 1;
  double lo = eps[0] - 1.0, hi = eps[n - 1] + 1.0;
  double mu = 0.5 * (eps[ho] + eps[lu]);
  if (have_guess && mu_guess > lo && mu_guess < hi) mu = mu_guess;  // Fermi level of the previous iteration
  for (int it = 0; it < QCX_FERMI_ITERS; ++it) {
    double N = 0.0, dN = 0.0;
    for (int i = lane; i < n; i += 32) {
      double f = 1.0 / (1.0 + exp((eps[i] - mu) / kT));
      N += 2.0 * f;
      dN += 2.0 * f * (1.0 - f) / kT;
    }
    N = warp_sum(N);
    dN = warp_sum(dN);
    double r = N - nel;
    if (fabs(r) < rtol * (nel > 1.0 ? nel : 1.0)) break;
    if (r < 0) lo = mu;
    else hi = mu;
    double mn = (dN > 1e-300) ? mu - r / dN : 0.5 * (lo + hi);
    if (!(mn > lo && mn < hi)) mn = 0.5 * (lo + hi);
    mu = mn;
  }
  double ts = 0.0;
  for (int i = lane; i < n; i += 32) {
    double x = (eps[i] - mu) / kT, ax = fabs(x);
    double fs = 1.0 / (1.0 + exp(ax));
    double s = -(fs * ax + log1p(exp(-ax)));
    focc[i] = 2.0 / (1.0 + exp(x));
    ts += 2.0 * kT * s;
  }
  ts = warp_sum(ts);
  *efermi = mu;
  return ts;
}

// FP32 Fermi level for the FP32 SCC iterations (one warp). Orbital energies
// are shifted by the starting guess once in FP64; the Newton/bisection runs in
// FP32 on the shifted values held in registers (n <= 512), to an electron-count
// accuracy of 1e-6 * nel. Returns -T S.
__device__ double fermi_warp32(int n, const double* eps, double nel, double kT, double* focc, double* efermi,
                               double mu_guess, bool have_guess) {
  int lane = threadIdx.x & 31;
  if (nel <= 0.0 || nel >= 2.0 * n || n > 512)
    return fermi_warp(n, eps, nel, kT, focc, efermi, 1e-13, mu_guess, have_guess);
  int ho = (int)ceil(nel / 2.0) - 1;
  if (ho < 0) ho = 0;
  int lu = ho + 1 < n ? ho + 1 : n - 1;
  double mu0 = 0.5 * (eps[ho] + eps[lu]);
  if (have_guess && mu_guess > eps[0] - 1.0 && mu_guess < eps[n - 1] + 1.0) mu0 = mu_guess;
  float d[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    int i = lane + 32 * k;
    d[k] = i < n ? (float)(eps[i] - mu0) : 1e30f;
  }
  const float ikT = (float)(1.0 / kT);
  const float fnel = (float)nel;
  float lo = (float)(eps[0] - mu0) - 1.0f, hi = (float)(eps[n - 1] - mu0) + 1.0f, mu = 0.0f;
  for (int it = 0; it < QCX_FERMI_ITERS; ++it) {
    float N = 0.0f, dN = 0.0f;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      // fast exp and division: the FP32 iterations need the level to ~1e-6 electrons
      float f = __fdividef(1.0f, 1.0f + __expf((d[k] - mu) * ikT));
      N += 2.0f * f;
      dN += 2.0f * f * (1.0f - f) * ikT;
    }
    for (int o = 16; o > 0; o >>= 1) {
      N += __shfl_xor_sync(0xffffffffu, N, o);
      dN += __shfl_xor_sync(0xffffffffu, dN, o);
    }
    float r = N - fnel;
    if (fabsf(r) < 1e-6f * (fnel > 1.0f ? fnel : 1.0f)) break;
    if (r < 0.0f) lo = mu;
    else hi = mu;
    float mn = (dN > 1e-30f) ? mu - r / dN : 0.5f * (lo + hi);
    if (!(mn > lo && mn < hi)) mn = 0.5f * (lo + hi);
    mu = mn;
  }
  float ts = 0.0f;
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    int i = lane + 32 * k;
    if (i >= n) continue;
    float x = (d[k] - mu) * ikT, ax = fabsf(x);
    float fs = 1.0f / (1.0f + expf(ax));
    ts += -(fs * ax + log1pf(expf(-ax)));
    focc[i] = (double)(2.0f / (1.0f + expf(x)));
  }
  for (int o = 16; o > 0; o >>= 1) ts += __shfl_xor_sync(0xffffffffu, ts, o);
  *efermi = mu0 + (double)mu;
  return 2.0 * kT * (double)ts;
}

// ---------------------------------------------------------------------------
// Solves M x = b for a symmetric positive definite k x k matrix (k <= 32, row
// major, FP64) with one warp: an FP32 Cholesky factor held one row per lane,
// then two steps of iterative refinement with FP64 residuals (Wilkinson), which
// recover the FP64 solution for condition numbers far below 1/eps_FP32^2. The
// factorisation and triangular solves run on the FP32 pipes; a serial FP64
// elimination on one warp is latency-bound at the FP64 rate.
// ---------------------------------------------------------------------------
// L L^T x = b with the Cholesky factor held one row per lane (row[c] = L[lane][c])
// and the right-hand side held one element per lane
template <int NM>
__device__ __forceinline__ float chol_solve_lane(const float (&row)[NM], float b, int k) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int j = 0; j < NM; ++j) {
    if (j < k) {
      float yj = __shfl_sync(full, b, j) / __shfl_sync(full, row[j], j);
      if (lane == j) b = yj;
      else if (lane > j) b = fmaf(-row[j], yj, b);
    }
  }
#pragma unroll
  for (int j = NM - 1; j >= 0; --j) {
    if (j < k) {
      float t = (lane > j && lane < k) ? row[j] * b : 0.f;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(full, t, o);
      float yj = __shfl_sync(full, b, j), ljj = __shfl_sync(full, row[j], j);
      if (lane == j) b = (yj - t) / ljj;
    }
  }
  return b;
}

template <int NM>
__device__ __noinline__ void spd_solve_warp(const double* M, double* rhs, int k) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  float row[NM];
#pragma unroll
  for (int c = 0; c < NM; ++c) row[c] = (lane < k && c < k) ? (float)M[lane * k + c] : 0.f;
#pragma unroll
  for (int j = 0; j < NM; ++j) {
    if (j < k) {
      float ljj = sqrtf(fmaxf(__shfl_sync(full, row[j], j), 1e-30f));
      float lj = lane > j ? row[j] / ljj : 0.f;
      if (lane == j) row[j] = ljj;
      else if (lane > j) row[j] = lj;
#pragma unroll
      for (int c = j + 1; c < NM; ++c) {
        if (c < k) {
          float lcj = __shfl_sync(full, lj, c);
          if (lane >= c) row[c] = fmaf(-lj, lcj, row[c]);
        }
      }
    }
  }
  const double bd = lane < k ? rhs[lane] : 0.0;
  double xd = (double)chol_solve_lane<NM>(row, (float)bd, k);
  for (int it = 0; it < 2; ++it) {
    double r = bd;
    for (int c = 0; c < k; ++c) {
      double xc = __shfl_sync(full, xd, c);
      if (lane < k) r -= M[lane * k + c] * xc;
    }
    xd += (double)chol_solve_lane<NM>(row, (float)r, k);
  }
  if (lane < k) rhs[lane] = xd;
}

// ---------------------------------------------------------------------------
// modified Broyden update of x (len) given x_out; it = number of previous updates
// ---------------------------------------------------------------------------
__device__ void broyden(const MolView& mv, double* x, const double* xout, int it, double alpha, SccShared& sh) {
  const int len = mv.md.len, nmem = mv.md.nmem;
  double* vec = mv.vec;
  double* df = vec + mv.vl.bdf;
  double* u = vec + mv.vl.bu;
  double* a = vec + mv.vl.ba;
  double* xl = vec + mv.vl.bxl;
  double* fl = vec + mv.vl.bfl;
  double* cvec = vec + mv.vl.bc;
  if (it == 0) {
    for (int i = threadIdx.x; i < len; i += blockDim.x) {
      double f = xout[i] - x[i];
      xl[i] = x[i];
      fl[i] = f;
      x[i] += alpha * f;
    }
    __syncthreads();
    return;
  }
  // sliding window: slot of this update, number of valid slots
  int m = (it - 1) % nmem;
  int k = it < nmem ? it : nmem;
  double* dfm = df + (long long)m * len;
  double* um = u + (long long)m * len;
  // the residual f and the new difference vector are read by every dot product
  // below: keep them in shared memory (the moment scratch holds 10 n >= len
  // doubles; the second vector only when both fit)
  double* fs = sh.mom;
  double* ds = 2 * len <= 10 * mv.md.nao ? sh.mom + len : nullptr;
  double nrm[1] = {0.0};
  for (int i = threadIdx.x; i < len; i += blockDim.x) {
    double f = xout[i] - x[i];
    double d = f - fl[i];
    fs[i] = f;
    dfm[i] = d;
    nrm[0] += d * d;
  }
  cta_sum<1>(nrm, sh.red);
  double nr = sqrt(nrm[0]);
  if (nr < 1e-300) nr = 1e-300;
  for (int i = threadIdx.x; i < len; i += blockDim.x) {
    const double d = dfm[i] / nr;
    dfm[i] = d;
    if (ds) ds[i] = d;
    um[i] = alpha * d + (x[i] - xl[i]) / nr;
  }
  __syncthreads();
  const double* dv = ds ? ds : dfm;
  // a[j][m] = df_j . df_m ; c_j = df_j . f   (one warp per j)
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int j = w; j < k; j += kWarps) {
    const double* dfj = df + (long long)j * len;
    double s1 = 0.0, s2 = 0.0;
    for (int i = lane; i < len; i += 32) {
      const double dj = dfj[i];
      s1 += dj * dv[i];
      s2 += dj * fs[i];
    }
    s1 = warp_sum(s1);
    s2 = warp_sum(s2);
    if (lane == 0) {
      a[j * nmem + m] = s1;
      a[m * nmem + j] = s1;
      cvec[j] = s2;
    }
  }
  __syncthreads();
  // solve (w0^2 I + a) gamma = c (symmetric positive definite): one warp, FP32
  // Cholesky with FP64 refinement; Gaussian elimination with partial pivoting
  // for histories longer than a warp
  double* Ms = vec + mv.vl.bm;
  double* rhs = Ms + k * k;
  for (int i = threadIdx.x; i < k * k; i += blockDim.x) {
    int r = i / k, c = i % k;
    Ms[i] = a[r * nmem + c] + (r == c ? QCX_BROYDEN_W0 * QCX_BROYDEN_W0 : 0.0);
  }
  for (int i = threadIdx.x; i < k; i += blockDim.x) rhs[i] = cvec[i];
  __syncthreads();
  if (k <= 32 && QCX_BROYDEN_WINDOW <= 32) {
    if (w == 0) spd_solve_warp<(QCX_BROYDEN_WINDOW < 32 ? QCX_BROYDEN_WINDOW : 32)>(Ms, rhs, k);
  } else if (w == 0) {
    for (int col = 0; col < k; ++col) {
      // pivot search
      double best = -1.0;
      int bi = col;
      for (int r = col + lane; r < k; r += 32) {
        double v = fabs(Ms[r * k + col]);
        if (v > best) {
          best = v;
          bi = r;
        }
      }
      for (int o = 16; o > 0; o >>= 1) {
        double ov = __shfl_xor_sync(0xffffffffu, best, o);
        int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > best || (ov == best && oi < bi)) {
          best = ov;
          bi = oi;
        }
      }
      if (bi != col) {
        for (int c = lane; c < k; c += 32) {
          double t = Ms[col * k + c];
          Ms[col * k + c] = Ms[bi * k + c];
          Ms[bi * k + c] = t;
        }
        if (lane == 0) {
          double t = rhs[col];
          rhs[col] = rhs[bi];
          rhs[bi] = t;
        }
      }
      __syncwarp();
      double piv = Ms[col * k + col];
      for (int r = col + 1 + lane; r < k; r += 32) {
        double f = Ms[r * k + col] / piv;
        for (int c = col; c < k; ++c) Ms[r * k + c] -= f * Ms[col * k + c];
        rhs[r] -= f * rhs[col];
      }
      __syncwarp();
    }
    if (lane == 0) {
      for (int r = k - 1; r >= 0; --r) {
        double s = rhs[r];
        for (int c = r + 1; c < k; ++c) s -= Ms[r * k + c] * rhs[c];
        rhs[r] = s / Ms[r * k + r];
      }
    }
    __syncwarp();
  }
  __syncthreads();
  for (int i = threadIdx.x; i < len; i += blockDim.x) {
    double f = fs[i];
    double s = 0.0;
    for (int j = 0; j < k; ++j) s += rhs[j] * u[(long long)j * len + i];
    xl[i] = x[i];
    fl[i] = f;
    x[i] += alpha * f - s;
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Exact Jacobi rotations on the pairs that are too far from diagonal for the
// first-order refinement: Km (ld n) holds the first-order coefficients, row i
// picks its partner j with the largest |K_ij| above khard, and thread 0 keeps
// a set of disjoint pairs (rows in index order, so the choice is
// deterministic). Each kept pair (p, q) gets the rotation that zeroes B_pq; B
// is rotated on both sides (all rows first, then all columns, which is
// R B R^T for commuting disjoint rotations) and so are the coefficient rows,
// with the conventions of jacobi(). Returns the number of rotations.
// ---------------------------------------------------------------------------
template <typename T>
__device__ int rotate_hard_pairs(T* JA, T* JV, const T* Km, int n, T khard, SccShared& sh) {
  const int np = n + (n & 1);
  int* best = sh.perm;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    T bk = khard;
    int bj = -1;
    for (int j = 0; j < n; ++j) {
      T k = Km[(long long)i * n + j];
      k = k < T(0) ? -k : k;
      if (k > bk) {
        bk = k;
        bj = j;
      }
    }
    best[i] = bj;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned* used = (unsigned*)sh.red;  // one bit per orbital: 16 kWarps doubles hold 1024 kWarps bits
    const int words = (n + 31) >> 5;
    for (int w = 0; w < words; ++w) used[w] = 0u;
    int cnt = 0;
    for (int i = 0; i < n; ++i) {
      int j = best[i];
      if (j < 0) continue;
      if (((used[i >> 5] >> (i & 31)) | (used[j >> 5] >> (j & 31))) & 1u) continue;
      used[i >> 5] |= 1u << (i & 31);
      used[j >> 5] |= 1u << (j & 31);
      sh.rp[cnt] = i < j ? i : j;
      sh.rq[cnt] = i < j ? j : i;
      ++cnt;
    }
    sh.rskip[0] = cnt;
  }
  __syncthreads();
  const int cnt = sh.rskip[0];
  T* rc = (T*)sh.rc;
  T* rs = (T*)sh.rs;
  for (int k = threadIdx.x; k < cnt; k += blockDim.x) {
    int p = sh.rp[k], q = sh.rq[k];
    T apq = T(0.5) * (JA[p * np + q] + JA[q * np + p]);
    T app = JA[p * np + p], aqq = JA[q * np + q];
    T c = 1, s = 0;
    if (apq != T(0)) {
      T theta = (aqq - app) / (T(2) * apq);
      T at = theta < T(0) ? -theta : theta;
      T t = (theta >= T(0) ? T(1) : T(-1)) / (at + sqrt(T(1) + theta * theta));
      c = T(1) / sqrt(T(1) + t * t);
      s = t * c;
    }
    rc[k] = c;
    rs[k] = s;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < cnt * n; e += blockDim.x) {
    int k = e / n, j = e - k * n;
    int p = sh.rp[k], q = sh.rq[k];
    T c = rc[k], s = rs[k];
    T ap = JA[p * np + j], aq = JA[q * np + j];
    JA[p * np + j] = c * ap - s * aq;
    JA[q * np + j] = s * ap + c * aq;
    T vp = JV[p * np + j], vq = JV[q * np + j];
    JV[p * np + j] = c * vp - s * vq;
    JV[q * np + j] = s * vp + c * vq;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < cnt * n; e += blockDim.x) {
    int k = e / n, i = e - k * n;
    int p = sh.rp[k], q = sh.rq[k];
    T c = rc[k], s = rs[k];
    T ap = JA[i * np + p], aq = JA[i * np + q];
    JA[i * np + p] = c * ap - s * aq;
    JA[i * np + q] = s * ap + c * aq;
  }
  __syncthreads();
  return cnt;
}

// ---------------------------------------------------------------------------
// GEMM-form eigenvector refinement in a nearly diagonal basis (T = float or
// double).
//
// JA holds B = C^T F C (ld np) for the current coefficient rows JV (= C^T,
// S-orthonormal). First-order perturbation theory gives the eigenvectors of
// B as I + K with K_ij = B_ij / (B_jj - B_ii), so C^T <- (I + K^T) C^T
// followed by one Newton-Schulz step that restores S-orthonormality, and the
// eigenvalues as B_jj + sum_i B_ij K_ij. A pass leaves an error of order
// max|K|^2; passes repeat (recomputing B) until the max|K| of a pass is below
// ktol (the remaining error is then below ktol^2). In FP32, pairs with
// |K| > kfail are first rotated exactly (rotate_hard_pairs, up to
// QCX_HARD_ROUNDS rounds per call).
// Returns false when the basis stays too far from diagonal or the passes do
// not reach ktol; JA then holds B for the current rows of JV and the caller
// runs Jacobi on it. On success JA's diagonal holds the eigenvalues.
// ---------------------------------------------------------------------------
#ifdef QCX_SCC_PHASE_TIMING
// FP32 refinement outcomes (diagnostic builds): [0] max|K| above the limit at
// the first pass, [1] above it at a later pass, [2] success, [3] passes
// exhausted, [4..8] first max|K| < 1e-3, < 1e-2, < 0.1, < 1, larger, [9] hard
// rounds before outcome [0]
__device__ unsigned long long g_refine32[16];
#define REFINE32_COUNT(i) \
  do {                     \
    if (sizeof(T) == 4 && threadIdx.x == 0) atomicAdd(&g_refine32[i], 1ull); \
  } while (0)
#else
#define REFINE32_COUNT(i)
#endif

template <typename T>
__device__ bool refine(T* JA, T* JV, const T* F, const T* S, T* Tm, T* Cm, double* tmp, int n,
                       double kfail, double ktol, int max_pass, double ns_min, SccShared& sh,
                       double mu = 0.0, double occ_gap = -1.0, MmaCtx* mc = nullptr) {
  const int np = n + (n & 1);
  int hard = 0;       // rounds of exact rotations so far
  bool fresh = true;  // JA holds B for the current rows of JV
  for (int pass = 0; pass < max_pass; ++pass) {
    if (pass > 0 && !fresh) {
      gemm_t<T>(mc, n, n, n, F, n, false, JV, np, true, Tm, n);
      __syncthreads();
      gemm_t<T>(mc, n, n, n, JV, np, false, Tm, n, false, JA, np);
      __syncthreads();
    }
    fresh = false;
    // K^T[j][i] = K_ij = B_ij / (B_jj - B_ii) into Tm (ld n). All arithmetic
    // in T: FP64 instructions inside the FP32 iterations cost the FP64 rate.
    T kmax_t = T(0);
    const T mu_t = (T)mu, gap_t = (T)occ_gap;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      int j = e / n, i = e - j * n;
      T k = T(0);
      if (i != j) {
        T b = T(0.5) * (JA[i * np + j] + JA[j * np + i]);
        T d = JA[j * np + j] - JA[i * np + i];
        // occ_gap > 0: mixing two orbitals that are both fully occupied or both
        // empty (further than occ_gap from mu, same side) leaves the density
        // unchanged, so such pairs are not rotated
        bool same = false;
        if (gap_t > T(0)) {
          T ei = JA[i * np + i] - mu_t, ej = JA[j * np + j] - mu_t;
          same = (ei > gap_t && ej > gap_t) || (ei < -gap_t && ej < -gap_t);
        }
        if (b != T(0) && !same) k = (d > T(1e-30) || d < T(-1e-30)) ? b / d : T(1e30);
      }
      Tm[e] = k;
      T ka = k < T(0) ? -k : k;
      kmax_t = ka > kmax_t ? ka : kmax_t;
    }
    double kmax = cta_max((double)kmax_t, sh.red);
#ifdef QCX_SCC_PHASE_TIMING
    if (pass == 0 && hard == 0)
      REFINE32_COUNT(kmax < 1e-3 ? 4 : kmax < 1e-2 ? 5 : kmax < 0.1 ? 6 : kmax < 1.0 ? 7 : 8);
#endif
    if (kmax > kfail) {
      // rotate the offending pairs exactly (B stays expressed in the rotated
      // basis, so no recomputation) and look again
      if (sizeof(T) == 4 && hard < QCX_HARD_ROUNDS && rotate_hard_pairs<T>(JA, JV, Tm, n, (T)kfail, sh) > 0) {
        ++hard;
        --pass;
        fresh = true;
        continue;
      }
      if (pass == 0) {
        REFINE32_COUNT(0);
#ifdef QCX_SCC_PHASE_TIMING
        if (sizeof(T) == 4 && threadIdx.x == 0) atomicAdd(&g_refine32[9], (unsigned long long)hard);
#endif
        return false;
      }
      REFINE32_COUNT(1);
      // the basis moved but did not converge: give the current B to Jacobi
      for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        int i = e / n, j = e % n;
        if (j < i) {
          T s = T(0.5) * (JA[i * np + j] + JA[j * np + i]);
          JA[i * np + j] = s;
          JA[j * np + i] = s;
        }
      }
      __syncthreads();
      return false;
    }
    // second-order eigenvalues onto the diagonal of B
    T* lamv = (T*)tmp;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
      T lam = JA[j * np + j];
      for (int i = 0; i < n; ++i)
        if (i != j) lam += T(0.5) * (JA[i * np + j] + JA[j * np + i]) * Tm[(long long)j * n + i];
      lamv[j] = lam;
    }
    __syncthreads();
    for (int j = threadIdx.x; j < n; j += blockDim.x) JA[j * np + j] = lamv[j];
    if (kmax == 0.0) {
      REFINE32_COUNT(2);
      return true;
    }
    // C^T <- C^T + K^T C^T
    gemm_t<T>(mc, n, n, n, Tm, n, false, JV, np, false, Cm, n);
    __syncthreads();
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) JV[(e / n) * np + (e % n)] += Cm[e];
    __syncthreads();
    // restore S-orthonormality: C^T <- (3I - C^T S C)/2 C^T. (I + K) is orthogonal
    // to first order (K is antisymmetric), so below ns_min the O(K^2) defect is
    // left for a later pass or iteration.
    if (kmax < ns_min) {
      if (kmax < ktol) {
        REFINE32_COUNT(2);
        return true;
      }
      continue;
    }
    // A first-order step of size K leaves an S-orthonormality defect of order
    // K^2 and one Newton-Schulz step squares it: after a step with K ~ 0.1 one
    // step still leaves ~1e-4. The Jacobi fallback and the next passes treat
    // B = V F V^T as a standard eigenproblem, so a defect left here becomes an
    // eigenvalue error of the same order (measured: 3e-4 Eh, which stalled the
    // SCC). Steps therefore repeat until the defect predicted from the
    // measured one (3/4 n E^2) is below the precision's floor.
    const int ns_steps = sizeof(T) == 4 ? 3 : QCX_NS64_STEPS;
    const double ns_floor = sizeof(T) == 4 ? 1e-9 : 1e-13;
    for (int st = 0; st < ns_steps; ++st) {
      gemm_t<T>(mc, n, n, n, S, n, false, JV, np, true, Tm, n);
      __syncthreads();
      gemm_t<T>(mc, n, n, n, JV, np, false, Tm, n, false, Cm, n);
      __syncthreads();
      T emax_t = T(0);
      for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        int i = e / n, j = e % n;
        T d = Cm[e] - (i == j ? T(1) : T(0));
        T ad = d < T(0) ? -d : d;
        emax_t = ad > emax_t ? ad : emax_t;
        Cm[e] = (i == j ? T(1) : T(0)) - T(0.5) * d;
      }
      double emax = cta_max((double)emax_t, sh.red);
      __syncthreads();
      gemm_t<T>(mc, n, n, n, Cm, n, false, JV, np, false, Tm, n);
      __syncthreads();
      for (int e = threadIdx.x; e < n * n; e += blockDim.x) JV[(e / n) * np + (e % n)] = Tm[e];
      __syncthreads();
      // predicted defect of the next step: 3/4 E^2, with the entries of E^2
      // summing sqrt(n) terms of random sign (n terms bound it; measured
      // steps shrink as 0.8 E^2 in the max norm)
      if (0.75 * (sizeof(T) == 4 ? (double)n : sqrt((double)n)) * emax * emax < ns_floor) break;
    }
    // the remaining off-diagonal is of order kmax^2: stop once that is below ktol^2
    if (kmax < ktol) {
      REFINE32_COUNT(2);
      return true;
    }
  }
  REFINE32_COUNT(3);
  // passes exhausted: recompute B in the final basis for the caller's Jacobi
  gemm_t<T>(mc, n, n, n, F, n, false, JV, np, true, Tm, n);
  __syncthreads();
  gemm_t<T>(mc, n, n, n, JV, np, false, Tm, n, false, JA, np);
  __syncthreads();
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    int i = e / n, j = e % n;
    if (j < i) {
      T s = T(0.5) * (JA[i * np + j] + JA[j * np + i]);
      JA[i * np + j] = s;
      JA[j * np + i] = s;
    }
  }
  __syncthreads();
  return false;
}

// ---------------------------------------------------------------------------
// Double-float arithmetic for the finishing iterations of mixed mode.
//
// A value is held as an unevaluated sum hi + lo of two FP32 numbers (Dekker
// 1971; the "double-single" or "df64" representation), about 48 significant
// bits. Products use the exact FMA splitting of hi*hi and sums use Knuth's
// two-sum, so a dot product of length n carries a relative error of order
// n 2^-46 while running on the FP32 pipes, which GB300 executes at 58 times
// the FP64 rate. All steps use explicitly rounded intrinsics so that the
// compiler cannot contract or reorder them.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void dd_split(double x, float& hi, float& lo) {
  hi = __double2float_rn(x);
  lo = __double2float_rn(x - (double)hi);
}

// (sh, sl) += (ah + al) (bh + bl), dropping al*bl
__device__ __forceinline__ void dd_fma(float& sh, float& sl, float ah, float al, float bh, float bl) {
  float p = __fmul_rn(ah, bh);
  float e = __fmaf_rn(ah, bh, -p);
  e = __fmaf_rn(ah, bl, e);
  e = __fmaf_rn(al, bh, e);
  float s = __fadd_rn(sh, p);
  float v = __fsub_rn(s, sh);
  float t = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, v)), __fsub_rn(p, v));
  sl = __fadd_rn(sl, __fadd_rn(t, e));
  sh = s;
}

// renormalise so that |lo| <= ulp(hi) / 2 (fast two-sum; |hi| >= |lo| holds)
__device__ __forceinline__ void dd_norm(float& hi, float& lo) {
  float s = __fadd_rn(hi, lo);
  lo = __fsub_rn(lo, __fsub_rn(s, hi));
  hi = s;
}

// (h, l) += d
__device__ __forceinline__ void dd_add(float& h, float& l, float d) {
  float s = __fadd_rn(h, d);
  float v = __fsub_rn(s, h);
  float t = __fadd_rn(__fsub_rn(h, __fsub_rn(s, v)), __fsub_rn(d, v));
  l = __fadd_rn(l, t);
  h = s;
  dd_norm(h, l);
}

// C = op(A) op(B) in double-float, with the index conventions of cta_gemm
// (ta: A stored K x M; tb: B stored N x K). Each element is a float2 (hi, lo),
// so one 8-byte load brings both parts. The result goes to C, or, when Cd is
// given, to Cd as FP64.
__device__ void cta_gemm_dd(int M, int N, int K, const float2* A, int lda, bool ta, const float2* B, int ldb,
                            bool tb, float2* C, double* Cd, int ldc) {
  int tilesM = (M + 1) / 2, tilesN = (N + 1) / 2;
  for (int t = threadIdx.x; t < tilesM * tilesN; t += blockDim.x) {
    int i0 = (t / tilesN) * 2, j0 = (t % tilesN) * 2;
    bool i1ok = i0 + 1 < M, j1ok = j0 + 1 < N;
    int i1 = i1ok ? i0 + 1 : i0, j1 = j1ok ? j0 + 1 : j0;
    float h00 = 0.f, l00 = 0.f, h01 = 0.f, l01 = 0.f, h10 = 0.f, l10 = 0.f, h11 = 0.f, l11 = 0.f;
    for (int k = 0; k < K; ++k) {
      const float2 a0 = A[ta ? (long long)k * lda + i0 : (long long)i0 * lda + k];
      const float2 a1 = A[ta ? (long long)k * lda + i1 : (long long)i1 * lda + k];
      const float2 b0 = B[tb ? (long long)j0 * ldb + k : (long long)k * ldb + j0];
      const float2 b1 = B[tb ? (long long)j1 * ldb + k : (long long)k * ldb + j1];
      dd_fma(h00, l00, a0.x, a0.y, b0.x, b0.y);
      dd_fma(h01, l01, a0.x, a0.y, b1.x, b1.y);
      dd_fma(h10, l10, a1.x, a1.y, b0.x, b0.y);
      dd_fma(h11, l11, a1.x, a1.y, b1.x, b1.y);
    }
    dd_norm(h00, l00);
    dd_norm(h01, l01);
    dd_norm(h10, l10);
    dd_norm(h11, l11);
    auto put = [&](int i, int j, float h, float l) {
      long long c = (long long)i * ldc + j;
      if (Cd) Cd[c] = (double)h + (double)l;
      else C[c] = make_float2(h, l);
    };
    put(i0, j0, h00, l00);
    if (j1ok) put(i0, j1, h01, l01);
    if (i1ok) {
      put(i1, j0, h10, l10);
      if (j1ok) put(i1, j1, h11, l11);
    }
  }
}

// C = A B_hi in FP32 (A: M x K, ld lda; B: K x N float2, ld ldb, hi parts only)
__device__ void cta_gemm_hi(int M, int N, int K, const float* A, int lda, const float2* B, int ldb, float* C,
                            int ldc) {
  int tilesM = (M + 1) / 2, tilesN = (N + 1) / 2;
  for (int t = threadIdx.x; t < tilesM * tilesN; t += blockDim.x) {
    int i0 = (t / tilesN) * 2, j0 = (t % tilesN) * 2;
    bool i1ok = i0 + 1 < M, j1ok = j0 + 1 < N;
    int i1 = i1ok ? i0 + 1 : i0, j1 = j1ok ? j0 + 1 : j0;
    float c00 = 0.f, c01 = 0.f, c10 = 0.f, c11 = 0.f;
    for (int k = 0; k < K; ++k) {
      const float a0 = A[(long long)i0 * lda + k], a1 = A[(long long)i1 * lda + k];
      const float b0 = B[(long long)k * ldb + j0].x, b1 = B[(long long)k * ldb + j1].x;
      c00 = fmaf(a0, b0, c00);
      c01 = fmaf(a0, b1, c01);
      c10 = fmaf(a1, b0, c10);
      c11 = fmaf(a1, b1, c11);
    }
    C[(long long)i0 * ldc + j0] = c00;
    if (j1ok) C[(long long)i0 * ldc + j1] = c01;
    if (i1ok) {
      C[(long long)i1 * ldc + j0] = c10;
      if (j1ok) C[(long long)i1 * ldc + j1] = c11;
    }
  }
}

// Double-float coefficient rows and the matrices of one molecule's finishing
// iterations (mixed mode), each element a float2 (hi, lo): V (rows = MOs, ld
// np) and its transpose Vt (ld n, kept in step with V so that the products with
// V^T read their operand along rows), B = V F V^T (ld np), F and S (ld n), T and
// M scratch (ld n); Kf and dV are FP32 scratch (ld n).
struct DDMats {
  float2 *V, *Vt, *B, *F, *S, *T, *M;
  float *Kf, *dV;
};

// Vt = V^T
__device__ void dd_transpose(const DDMats& d, int n, int np) {
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    int k = e / n, j = e - k * n;
    d.Vt[e] = d.V[(long long)j * np + k];
  }
  __syncthreads();
}

// V <- V + dV (dV FP32, ld n) in double-float, and the same into Vt
__device__ void dd_add_rows(const DDMats& d, int n, int np) {
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    int i = e / n, j = e - i * n;
    long long x = (long long)i * np + j;
    float2 v = d.V[x];
    dd_add(v.x, v.y, d.dV[e]);
    d.V[x] = v;
    d.Vt[(long long)j * n + i] = v;
  }
  __syncthreads();
}

// B = V F V^T
__device__ void dd_rotate_fock(const DDMats& d, int n, int np) {
  cta_gemm_dd(n, n, n, d.F, n, false, d.Vt, n, false, d.T, nullptr, n);
  __syncthreads();
  cta_gemm_dd(n, n, n, d.V, np, false, d.T, n, false, d.B, nullptr, np);
  __syncthreads();
}

// Newton-Schulz steps V <- (3I - V S V^T)/2 V: the overlap V S V^T in
// double-float, the (small) correction -(V S V^T - I)/2 V in FP32. Returns the
// largest |V S V^T - I| seen before the last step.
__device__ double dd_orthonormalize(const DDMats& d, int n, int np, int steps, SccShared& sh,
                                   double floor = 1e-26) {
  double emax = 0.0;
  for (int st = 0; st < steps; ++st) {
    cta_gemm_dd(n, n, n, d.S, n, false, d.Vt, n, false, d.T, nullptr, n);
    __syncthreads();
    cta_gemm_dd(n, n, n, d.V, np, false, d.T, n, false, d.M, nullptr, n);
    __syncthreads();
    float em = 0.f;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      int i = e / n, j = e - i * n;
      const float2 m = d.M[e];
      float dev = __fadd_rn(__fsub_rn(m.x, i == j ? 1.f : 0.f), m.y);
      em = fmaxf(em, fabsf(dev));
      d.Kf[e] = -0.5f * dev;
    }
    emax = cta_max((double)em, sh.red);
    cta_gemm_hi(n, n, n, d.Kf, n, d.V, np, d.dV, n);
    __syncthreads();
    dd_add_rows(d, n, np);
    // the defect left is about 3/4 emax^2, times sqrt(n) for the sum of n
    // terms of random sign in every entry of E^2 (n terms bound it)
    if (0.75 * sqrt((double)n) * emax * emax < floor) break;
  }
  return emax;
}

// First-order refinement of the double-float rows V against B = V F V^T (held
// in d.B on entry), as refine() does in FP32/FP64: K_ij = B_ij / (B_jj - B_ii)
// in FP32 from the double-float B, V <- V + K^T V with the product in FP32
// (K is small, so its rounding is far below the double-float level of V), and
// Newton-Schulz in double-float when max|K| >= ns_min. Eigenvalues (second
// order) go to lam. Returns false if max|K| exceeds kfail or the passes do not
// reach ktol; B then holds V F V^T for the current rows.
__device__ bool refine_dd(const DDMats& d, int n, double* lam, double kfail, double ktol, int max_pass,
                          double ns_min, SccShared& sh) {
  const int np = n + (n & 1);
  for (int pass = 0; pass < max_pass; ++pass) {
    if (pass > 0) dd_rotate_fock(d, n, np);
    // diagonal in FP64
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const float2 b = d.B[(long long)i * np + i];
      lam[i] = (double)b.x + (double)b.y;
    }
    __syncthreads();
    float km = 0.f;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      int j = e / n, i = e - j * n;
      float k = 0.f;
      if (i != j) {
        float b = 0.5f * (d.B[(long long)i * np + j].x + d.B[(long long)j * np + i].x);
        float dd = __double2float_rn(lam[j] - lam[i]);
        if (b != 0.f) k = (dd > 1e-30f || dd < -1e-30f) ? b / dd : 1e30f;
      }
      d.Kf[e] = k;  // K^T[j][i] = K_ij
      km = fmaxf(km, fabsf(k));
    }
    double kmax = cta_max((double)km, sh.red);
    if (kmax > kfail) return false;
    // second-order eigenvalues
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
      float c = 0.f;
      for (int i = 0; i < n; ++i)
        if (i != j)
          c += 0.5f * (d.B[(long long)i * np + j].x + d.B[(long long)j * np + i].x) * d.Kf[(long long)j * n + i];
      d.dV[j] = c;
    }
    __syncthreads();
    for (int j = threadIdx.x; j < n; j += blockDim.x) lam[j] += (double)d.dV[j];
    __syncthreads();
    if (kmax == 0.0) return true;
    // K^T V with the hi parts of V
    cta_gemm_hi(n, n, n, d.Kf, n, d.V, np, d.dV, n);
    __syncthreads();
    dd_add_rows(d, n, np);
    // as in refine(): remove the O(K^2) defect completely, the fallback Jacobi
    // and the next passes need an S-orthonormal basis
    if (kmax >= ns_min) dd_orthonormalize(d, n, np, QCX_NS64_STEPS, sh, 1e-13);
    if (kmax < ktol) return true;
  }
  dd_rotate_fock(d, n, np);
  return false;
}

// Cd = sum_{k < nocc} w_k v_k^T v_k (FP64 result, ld n) for the double-float
// rows v_k = V[perm[k]]: G_k = w_k v_k goes to T, the rows in order to M, and
// one double-float product G^T V_occ forms the matrix.
__device__ void dd_density(const DDMats& d, int n, int nocc, const int* perm, const double* w, double* Cd,
                           SccShared& sh) {
  const int np = n + (n & 1);
  float* wh = (float*)sh.rc;  // np floats each: the rotation scratch is free here
  float* wl = (float*)sh.rs;
  for (int k = threadIdx.x; k < nocc; k += blockDim.x) dd_split(w[k], wh[k], wl[k]);
  __syncthreads();
  for (int e = threadIdx.x; e < nocc * n; e += blockDim.x) {
    int k = e / n, j = e - k * n;
    const float2 v = d.V[(long long)perm[k] * np + j];
    float p = __fmul_rn(wh[k], v.x);
    float er = __fmaf_rn(wh[k], v.x, -p);
    er = __fmaf_rn(wh[k], v.y, er);
    er = __fmaf_rn(wl[k], v.x, er);
    dd_norm(p, er);
    d.T[e] = make_float2(p, er);
    d.M[e] = v;
  }
  __syncthreads();
  cta_gemm_dd(n, n, nocc, d.T, n, true, d.M, n, false, nullptr, Cd, n);
  __syncthreads();
}

// ---------------------------------------------------------------------------
// the SCC kernel
//
// MIXED = 0: every iteration in FP64.
// MIXED = 1: iterations run the Fock build, potentials, transforms, the
//   Jacobi eigensolve, Fermi level, density and moments in FP32 until the
//   moment residual drops below kMixedSwitch; the remaining iterations (at
//   least two, and always the final one) keep the coefficient rows and their
//   O(n^3) products in double-float (hi + lo FP32), warm-started from the FP32
//   eigenvectors after two Newton-Schulz re-orthonormalisations. The Fock
//   build, potentials, moments, Fermi level, energies of those iterations and
//   the Broyden mixing are FP64.
// ---------------------------------------------------------------------------
constexpr double kMixedSwitch = QCX_MIXED_SWITCH;

// Optional per-phase cycle counters (diagnostic builds only: -DQCX_SCC_PHASE_TIMING).
#ifdef QCX_SCC_PHASE_TIMING
__device__ unsigned long long g_phase_cycles[24];
__device__ unsigned long long g_mol_cycles[4096];
__device__ unsigned long long g_counts[8];  // refine64 ok, jacobi64 fallbacks
#define PHASE_BEGIN() long long _pt = clock64()
#define PHASE_MARK(i)                                                 \
  do {                                                                \
    if (threadIdx.x == 0) {                                           \
      long long _n = clock64();                                       \
      atomicAdd(&g_phase_cycles[i], (unsigned long long)(_n - _pt)); \
      _pt = _n;                                                       \
    }                                                                 \
  } while (0)
#else
#define PHASE_BEGIN()
#define PHASE_MARK(i)
#endif
// Optional per-iteration trace of molecule 0 (diagnostic builds only: -DQCX_SCC_TRACE):
// residual, energy change, electronic energy, FP32 phase, Fermi level, highest occupied + 1
#ifdef QCX_SCC_TRACE
__device__ double g_trace[QCX_SCC_MAXITER + 1][6];
// orbital energies, occupations, input and output moment vectors (first 128 entries)
__device__ double g_trace_vec[QCX_SCC_MAXITER + 1][4][128];
#endif

template <int MIXED>
__global__ void __launch_bounds__(kSccThreads, QCX_SCC_MINBLOCKS) k_scc(DevBatch bt) {
  extern __shared__ __align__(16) char smem_raw[];
  // largest molecules first, so that the longest CTAs start in the first wave
  const int mol = bt.order ? bt.order[blockIdx.x] : blockIdx.x;
  if (!bt.active[mol]) return;
  // an SCC suspended at the previous launch's budget continues from its state
  const bool resume = bt.carry != nullptr && scc_pending(bt, mol);
  SccCarry cr{};
  if (resume) cr = bt.carry[mol];
  MolView mv;
  mv.bt = &bt;
  mv.md = bt.mol[mol];
  const MolDesc& md = mv.md;
  const int n = md.nao, nat = md.nat, nsh = md.nsh, len = md.len;
  const int np = n + (n & 1);
  mv.vl = VecLayout::make(nat, nsh, n, len, md.nmem);
  mv.vec = bt.vecs + md.vec_off;
  mv.Z = bt.Z + md.atom_off;
  mv.xyz = bt.xyz + 3LL * md.atom_off;
  const Params& P = *bt.prm;
  SccShared sh = carve(smem_raw, n);
  double* vec = mv.vec;
  const long long nn = (long long)n * n;
  double* S = mat_ptr(bt, md, kS);
  double* H0 = mat_ptr(bt, md, kH0);
  double* X = mat_ptr(bt, md, kX);
  double* F = mat_ptr(bt, md, kF);
  double* T = mat_ptr(bt, md, kT);
  double* Ag = mat_ptr(bt, md, kA);
  double* Vg = mat_ptr(bt, md, kV);
  double* C = mat_ptr(bt, md, kC);
  double* Pm = mat_ptr(bt, md, kP);
  double* Wm = mat_ptr(bt, md, kW);
  double* Dm = mat_ptr(bt, md, kDm0);
  double* Qm = mat_ptr(bt, md, kQm0);
  double* eps = vec + mv.vl.eps;
  double* focc = vec + mv.vl.focc;
  double* xin = vec + mv.vl.xin;
  double* xout = vec + mv.vl.xout;
  const int mode = jacobi_mode(n, (size_t)bt.smem_bytes);
  // FP64 Jacobi storage: shared memory when it fits, else the A / V slots.
  double* JA = (mode <= 1) ? sh.jac : Ag;
  double* JV = (mode == 0) ? sh.jac + (long long)np * np : Vg;
  // FP32 storage (mixed): both matrices inside the FP64 A region (shared
  // memory up to mode 1). When the FP64 A does not fit (mode 2) but the FP32 A
  // does, the FP32 A goes to shared memory and the FP32 coefficient rows to the
  // A slot (which the finishing iterations overwrite only after copying them).
  const bool a32_shared =
      mode == 2 && scc_fixed_bytes(n) + sizeof(float) * (size_t)np * np <= (size_t)bt.smem_bytes;
  float* JA32 = a32_shared ? (float*)sh.jac : (float*)JA;
  float* JV32 = a32_shared ? (float*)Ag : (float*)JA + (long long)np * np;
  float* T32 = (float*)T;
  float* X32 = (float*)Wm;
  // Tensor-core context of the FP32 iterations (mixed mode): the staging buffer
  // of the operands goes after this molecule's part of shared memory when it
  // fits there, else (both FP64 Jacobi matrices in shared memory) into the
  // FP64 coefficient matrix, which the FP32 iterations leave unused. The
  // products have N = n columns: one MMA takes N <= 256 and the accumulator
  // holds kMmaTmemCols columns, so larger molecules keep the CUDA-core path.
  __shared__ uint32_t mma_tmem_slot;
  __shared__ __align__(8) uint64_t mma_bar;
  MmaCtx mctx;
  MmaCtx* mc = nullptr;
  if (MIXED && QCX_SCC_MMA && ((n + 15) & ~15) <= kMmaTmemCols) {
    const size_t jac_used = mode == 0 ? 2 * sizeof(double) * (size_t)np * np
                                      : mode == 1 ? sizeof(double) * (size_t)np * np
                                                  : (a32_shared ? sizeof(float) * (size_t)np * np : 0);
    const size_t need = (size_t)mma_stage_bytes((n + 15) & ~15);
    const size_t tail = (scc_fixed_bytes(n) + jac_used + 127) & ~(size_t)127;
    char* stage = nullptr;
    if (tail + need <= (size_t)bt.smem_bytes) stage = smem_raw + tail;
    else if (mode == 0 && sizeof(double) * (size_t)np * np >= need) stage = (char*)JV;
    if (stage) {
      mma_setup(mctx, &mma_tmem_slot, &mma_bar, stage);
      mc = &mctx;
    }
  }

  // --- per-AO maps -------------------------------------------------------
  const int* sh_atom = bt.sh_atom + md.sh_off;
  const int* sh_ao = bt.sh_ao + md.sh_off;
  const int* sh_k = bt.sh_k + md.sh_off;
  for (int s = threadIdx.x; s < nsh; s += blockDim.x) {
    int a = sh_atom[s] - md.atom_off;
    int l = P.sh_l[mv.Z[a]][sh_k[s]];
    for (int i = 0; i < 2 * l + 1; ++i) {
      sh.ao_sh[sh_ao[s] + i] = s;
      sh.ao_at[sh_ao[s] + i] = a;
    }
  }
  // --- geometry-dependent precomputation ------------------------------
  for (int i = threadIdx.x; i < nsh * nsh; i += blockDim.x) {
    int s = i / nsh, t = i % nsh;
    int a = sh_atom[s] - md.atom_off, b = sh_atom[t] - md.atom_off;
    double ea = P.hardness[mv.Z[a]][sh_k[s]], eb = P.hardness[mv.Z[b]][sh_k[t]];
    double eta = 0.5 * (ea + eb);
    double r2 = 0;
    for (int k = 0; k < 3; ++k) {
      double d = mv.xyz[3 * a + k] - mv.xyz[3 * b + k];
      r2 += d * d;
    }
    vec[mv.vl.gam + i] = 1.0 / sqrt(r2 + 1.0 / (eta * eta));
  }
  for (int i = threadIdx.x; i < nat * nat; i += blockDim.x) {
    int a = i / nat, b = i % nat;
    double gd = 0.0, f3 = 0.0, f5 = 0.0, d3r = 0, d3r0 = 0, d5r = 0, d5r0 = 0;
    if (a != b) {
      int za = mv.Z[a], zb = mv.Z[b];
      int ga = md.atom_off + a, gb = md.atom_off + b;
      double r2 = 0;
      for (int k = 0; k < 3; ++k) {
        double d = mv.xyz[3 * a + k] - mv.xyz[3 * b + k];
        r2 += d * d;
      }
      double r = sqrt(r2);
      double dg;
      bj_kernel(P, za, zb, r, gd, dg);
      double r0 = 0.5 * (bt.mrad[ga] + bt.mrad[gb]);
      mp_kernel(3, QCX_AES_A3, r, r0, f3, d3r, d3r0);
      mp_kernel(5, QCX_AES_A5, r, r0, f5, d5r, d5r0);
    }
    vec[mv.vl.gdisp + i] = gd;
    vec[mv.vl.f3 + i] = f3;
    vec[mv.vl.f5 + i] = f5;
    vec[mv.vl.d3r + i] = d3r;
    vec[mv.vl.d3r0 + i] = d3r0;
    vec[mv.vl.d5r + i] = d5r;
    vec[mv.vl.d5r0 + i] = d5r0;
  }
  double nel = md.nel;
  // --- Cholesky S = L L^T (L stored in T, lower) -------------------------
  for (long long i = threadIdx.x; i < nn; i += blockDim.x) T[i] = S[i];
  __syncthreads();
  int status = 0;
  for (int j = 0; j < n; ++j) {
    double djj = T[(long long)j * n + j];
    if (!(djj > 0.0)) {
      status |= kCholeskyFailed;
      break;
    }
    double ljj = sqrt(djj);
    for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x) T[(long long)i * n + j] /= ljj;
    __syncthreads();
    if (threadIdx.x == 0) T[(long long)j * n + j] = ljj;
    int m = n - j - 1;
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
      int i = j + 1 + e / m, k = j + 1 + e % m;
      if (k <= i) T[(long long)i * n + k] -= T[(long long)i * n + j] * T[(long long)k * n + j];
    }
    __syncthreads();
  }
  if (status) {
    if (threadIdx.x == 0) {
      bt.status[mol] = status;
      bt.iters[mol] = 0;
      if (bt.have_prev) bt.have_prev[mol] = 0;
    }
    if (mc) mma_teardown(mctx);
    return;
  }
  // X = L^-T: row j of X = column j of L^-1, one forward substitution per thread
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    X[(long long)j * n + j] = 1.0 / T[(long long)j * n + j];
    for (int i = 0; i < j; ++i) X[(long long)j * n + i] = 0.0;
    for (int i = j + 1; i < n; ++i) {
      double s = 0.0;
      for (int k = j; k < i; ++k) s -= T[(long long)i * n + k] * X[(long long)j * n + k];
      X[(long long)j * n + i] = s / T[(long long)i * n + i];
    }
  }
  __syncthreads();
  // FP32 copies of the fixed matrices for the FP32 iterations (conversions
  // from FP64 run at the FP64 rate, so they are done once here)
  float* S32 = (float*)mat_ptr(bt, md, kS32);
  float* H032 = S32 + nn;
  float* D32 = (float*)mat_ptr(bt, md, kD32);
  float* Q32 = (float*)mat_ptr(bt, md, kQ32);
  // double-float planes of the finishing iterations (mixed mode): V in the
  // coefficient storage, B in the A storage, F in the F slot, S as the FP32
  // copy plus a lo plane in the W slot (free until W is formed), scratch in
  // the T, C and X slots (X is only needed without an FP32 phase)
  DDMats dm;
  dm.V = (float2*)JV;
  dm.Vt = (float2*)Q32;  // the FP32 quadrupoles are not needed after the FP32 iterations
  dm.B = (float2*)JA;
  dm.F = (float2*)F;
  dm.S = (float2*)Wm;
  dm.T = (float2*)T;
  dm.M = (float2*)C;
  dm.Kf = (float*)X;
  dm.dV = dm.Kf + nn;
  if (MIXED) {
    for (long long e = threadIdx.x; e < nn; e += blockDim.x) {
      X32[e] = (float)X[e];
      S32[e] = (float)S[e];
      H032[e] = (float)H0[e];
#pragma unroll
      for (int c = 0; c < 3; ++c) D32[c * nn + e] = (float)Dm[c * nn + e];
#pragma unroll
      for (int c = 0; c < 6; ++c) Q32[c * nn + e] = (float)Qm[c * nn + e];
    }
  }
  // start from zero moments (the reference's fresh wavefunction), or, when the
  // caller asked for it, from the converged output moments of the previous
  // geometry of this trajectory (still in xout)
  const bool warm_guess = bt.guess == 1 && bt.have_prev != nullptr && (bt.have_prev[mol] & 1) != 0;
  // bit 1 of have_prev: the first-iteration FP32 eigenvectors of the previous SCC
  // of this molecule are kept (after the three FP32 dipole matrices in the kD32 slots)
  float* B32 = D32 + 3 * nn;
  // a resumed SCC seeds its first FP32 eigensolve with the eigenvectors it had
  // at the suspension (same geometry), and keeps its moment vector
  const bool basis_kept =
      MIXED && (resume ? cr.basis != 0 : (bt.have_prev != nullptr && (bt.have_prev[mol] & 2) != 0));
  bool basis_saved = false;
  if (!resume)
    for (int i = threadIdx.x; i < len; i += blockDim.x) xin[i] = warm_guess ? xout[i] : 0.0;
  __syncthreads();

  double en[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  double eprev = resume ? cr.eprev : 0.0, eel = 0.0, ets = 0.0, eband = 0.0, efermi = resume ? cr.efermi : 0.0;
  int it, converged = 0, eig_fail = resume ? cr.eig_fail : 0;
  bool fp32_phase = resume ? cr.phase32 != 0 : (MIXED != 0 && bt.max_iter > 8 && n >= bt.mixed_min_nao);
  bool have64 = false;  // JV holds an orthonormal FP64 basis from a previous iteration
  bool have32 = false;  // JV32 holds FP32 eigenvectors from a previous iteration
  int bro_it = resume ? cr.bro_it : 0;  // Broyden updates since the last (re)start of the mixer
  double best32 = resume ? cr.best32 : 1e300;  // best residual seen in the FP32 phase
  // mixer restart after QCX_BROYDEN_RESTART iterations without a 10 % better residual
  double rbest = resume ? cr.rbest : 1e300;
  int rsince = resume ? cr.rsince : 0;
  int stall32 = resume ? cr.stall32 : 0;
  int backoff32 = resume ? cr.backoff32 : 0;  // FP32 iterations left before the next refinement attempt
  int n64 = resume ? cr.n64 : 0;              // FP64 iterations done
  // iteration budget of this launch (0: none); suspension only between FP32
  // iterations in mixed mode, so that the double-float finishing iterations
  // always run in one launch
  const int it0 = resume ? cr.it + 1 : 1;
  int budget = 0;
  if (bt.scc_budget > 0 && bt.carry != nullptr) {
    const double r = (double)bt.budget_nao / (double)n;
    budget = (int)ceil((double)bt.scc_budget * r * r);
  }
  bool suspended = false;
  PHASE_BEGIN();
#ifdef QCX_SCC_PHASE_TIMING
  long long _t_start = clock64();
#endif
  for (it = it0; it <= bt.max_iter; ++it) {
    PHASE_MARK(15);
    // FP32 iterations take their potentials in FP32 straight into shared memory
    const bool pot32 = fp32_phase && potentials32(mv, xin, (float*)sh.mom, n);
    if (!pot32) potentials(mv, xin, en, sh.red);
    PHASE_MARK(0);
    // Fock matrix
    {
      const double* vsh = vec + mv.vl.vsh;
      const double* vdp = vec + mv.vl.vdp;
      const double* vqp = vec + mv.vl.vqp;
      if (fp32_phase) {
        // FP32 iterations: the Fock matrix only feeds FP32 products. The
        // potentials go to shared memory as FP32 (the moment scratch is free
        // until the moments are formed: nsh + 9 nat <= 10 n floats).
        float* vs32 = (float*)sh.mom;
        float* vd32 = vs32 + nsh;
        float* vq32 = vd32 + 3 * nat;
        float* r32 = vq32 + 6 * nat;  // atom positions (nsh + 12 nat <= 20 n floats)
        if (!pot32) {
          for (int i = threadIdx.x; i < nsh + 12 * nat; i += blockDim.x) {
            double v;
            if (i < nsh) v = vsh[i];
            else if (i < nsh + 3 * nat) v = vdp[i - nsh];
            else if (i < nsh + 9 * nat) v = vqp[i - nsh - 3 * nat];
            else v = mv.xyz[i - nsh - 9 * nat];
            vs32[i] = (float)v;
          }
          __syncthreads();
        }
        float* F32 = (float*)F;
        // The multipole operators are centred on the bra atom, so the (j,i)
        // elements follow from the (i,j) ones by shifting the centre by
        // d = R_A - R_B: D_ji = D_ij + d S_ij and, for the second moments,
        // M_ji = M_ij + d D_ij^T + D_ij d^T + d d^T S_ij (then made traceless).
        // This reads every matrix along rows only.
        for (long long e = threadIdx.x; e < nn; e += blockDim.x) {
          int i = (int)(e / n), j = (int)(e % n);
          int A = sh.ao_at[i], B = sh.ao_at[j];
          const float s = S32[e];
          float f = H032[e] - 0.5f * s * (vs32[sh.ao_sh[i]] + vs32[sh.ao_sh[j]]);
          float d[3], D[3];
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            d[c] = r32[3 * A + c] - r32[3 * B + c];
            D[c] = D32[c * nn + e];
            f -= 0.5f * (vd32[3 * A + c] * D[c] + vd32[3 * B + c] * (D[c] + d[c] * s));
          }
          const float dD = d[0] * D[0] + d[1] * D[1] + d[2] * D[2];
          const float dd = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            float q = Q32[c * nn + e];
            float qji = q + 3.f * d[c] * D[c] + 1.5f * d[c] * d[c] * s - dD - 0.5f * dd * s;
            f -= 0.5f * (vq32[6 * A + c] * q + vq32[6 * B + c] * qji);
          }
          // off-diagonal components xy, xz, yz
#pragma unroll
          for (int c = 3; c < 6; ++c) {
            const int a = c == 5 ? 1 : 0, b = c == 3 ? 1 : 2;
            float q = Q32[c * nn + e];
            float qji = q + 1.5f * (d[a] * D[b] + d[b] * D[a] + d[a] * d[b] * s);
            f -= 0.5f * (vq32[6 * A + c] * q + vq32[6 * B + c] * qji);
          }
          F32[e] = f;
        }
      } else {
        for (long long e = threadIdx.x; e < nn; e += blockDim.x) {
          int i = (int)(e / n), j = (int)(e % n);
          int A = sh.ao_at[i], B = sh.ao_at[j];
          long long ji = (long long)j * n + i;
          double f = H0[e] - 0.5 * S[e] * (vsh[sh.ao_sh[i]] + vsh[sh.ao_sh[j]]);
#pragma unroll
          for (int c = 0; c < 3; ++c) f -= 0.5 * (vdp[3 * A + c] * Dm[c * nn + e] + vdp[3 * B + c] * Dm[c * nn + ji]);
#pragma unroll
          for (int c = 0; c < 6; ++c) f -= 0.5 * (vqp[6 * A + c] * Qm[c * nn + e] + vqp[6 * B + c] * Qm[c * nn + ji]);
          if (MIXED && have32) {  // double-float finishing iterations
            float2 v;
            dd_split(f, v.x, v.y);
            dm.F[e] = v;
          }
          else F[e] = f;
        }
      }
    }
    __syncthreads();
    PHASE_MARK(1);
    int nocc = 0;
    // JV / JV32 hold C^T: row k is the AO coefficient vector of MO k
    // (S-orthonormal). After the first iteration the Fock matrix is expressed
    // in the previous MO basis, B = C^T F C, which is nearly diagonal, and the
    // Jacobi rotations update C^T in place.
    if (fp32_phase) {
      // ---- FP32 iteration ----
      // First FP32 iteration: start the eigensolve from the kept eigenvectors of
      // the previous geometry, re-orthonormalised in the new overlap (two
      // Newton-Schulz steps), when they are close to orthonormal there; the
      // sweeps then converge to the same tolerance as from scratch, in fewer sweeps.
      bool seeded = false;
      if (!have32 && basis_kept) {
        for (int e = threadIdx.x; e < np * np; e += blockDim.x) {
          int r = e / np, c = e - r * np;
          JV32[e] = (r < n && c < n) ? B32[r * n + c] : (r == c ? 1.f : 0.f);
        }
        __syncthreads();
        float* C32 = (float*)C;
        for (int st = 0; st < 2; ++st) {
          gemm_t<float>(mc, n, n, n, S32, n, false, JV32, np, true, T32, n);
          __syncthreads();
          gemm_t<float>(mc, n, n, n, JV32, np, false, T32, n, false, C32, n);
          __syncthreads();
          float em = 0.f;
          for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
            int i = e / n, j = e - i * n;
            float d = C32[e] - (i == j ? 1.f : 0.f);
            em = fmaxf(em, fabsf(d));
            C32[e] = (i == j ? 1.f : 0.f) - 0.5f * d;
          }
          const double emax = cta_max((double)em, sh.red);
          if (st == 0 && !(emax < 0.25)) break;  // too far from the new metric: start from scratch
          gemm_t<float>(mc, n, n, n, C32, n, false, JV32, np, false, T32, n);
          __syncthreads();
          for (int e = threadIdx.x; e < n * n; e += blockDim.x) JV32[(e / n) * np + (e % n)] = T32[e];
          __syncthreads();
          if (st == 1) seeded = true;
        }
      }
      if (!have32 && !seeded) {
        gemm_t<float>(mc, n, n, n, (const float*)F, n, false, X32, n, false, T32, n);
        __syncthreads();
        gemm_t<float>(mc, n, n, n, X32, n, true, T32, n, false, JA32, np);
        __syncthreads();
      } else {
        // B = V F V^T with V^T copied out first (the FP64 X slot is free in
        // the FP32 iterations), so that both products read along rows
        float* Vt32 = (float*)X;
        for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
          int k = e / n, j = e - k * n;
          Vt32[e] = JV32[j * np + k];
        }
        __syncthreads();
        gemm_t<float>(mc, n, n, n, (const float*)F, n, false, Vt32, n, false, T32, n);
        __syncthreads();
        gemm_t<float>(mc, n, n, n, JV32, np, false, T32, n, false, JA32, np);
        __syncthreads();
      }
      for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        int i = e / n, j = e % n;
        if (j < i) {
          float s = 0.5f * (JA32[i * np + j] + JA32[j * np + i]);
          JA32[i * np + j] = s;
          JA32[j * np + i] = s;
        }
      }
      __syncthreads();
      PHASE_MARK(2);
      // a failed refinement costs about a Jacobi sweep, so after a failure the
      // next QCX_REFINE32_BACKOFF iterations go straight to the sweep
      bool try32 = have32 && QCX_REFINE32_PASSES > 0 && backoff32 == 0;
      if (backoff32 > 0) --backoff32;
      bool ok32 = try32 &&
                  refine<float>(JA32, JV32, (const float*)F, S32, T32, (float*)C, eps, n, QCX_REFINE32_KFAIL, QCX_REFINE32_KTOL,
                                QCX_REFINE32_PASSES, 1e-3, sh, efermi, QCX_OCC_GAP_KT * md.kT + QCX_OCC_GAP_ABS, mc);
      PHASE_MARK(16);
      if (try32 && !ok32) backoff32 = QCX_REFINE32_BACKOFF;
      // the first (cold) solve only seeds the FP32 iterations: it stops at a
      // looser tolerance, the warm sweeps and refinements of later iterations
      // take the basis further
      if (!ok32)
        jacobi<float>(JA32, JV32, n, have32 || seeded, have32 ? 2e-6 : QCX_JAC32_COLD_TOL, sh,
                      have32 ? (n <= QCX_JAC32_WARM2_MAX_NAO ? QCX_JAC32_WARM_SWEEPS : 1) : 30);
#ifdef QCX_SCC_PHASE_TIMING
      if (threadIdx.x == 0) atomicAdd(&g_phase_cycles[ok32 ? 13 : 14], 1ull);
#endif
      PHASE_MARK(3);
      if (!have32) {
        if (!seeded) {
          // eigenvectors of X^T F X -> C^T = V X^T
          gemm_t<float>(mc, n, n, n, JV32, np, false, X32, n, true, T32, n);
          __syncthreads();
          for (int e = threadIdx.x; e < n * n; e += blockDim.x) JV32[(e / n) * np + (e % n)] = T32[e];
          __syncthreads();
        }
        // keep this first-iteration basis for the next geometry
        if (bt.have_prev) {
          for (int e = threadIdx.x; e < n * n; e += blockDim.x) B32[e] = JV32[(e / n) * np + (e % n)];
          basis_saved = true;
        }
        have32 = true;
      }
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        // a non-finite eigenvalue ranks as +inf, so that the ranks stay a permutation
        float di = JA32[i * np + i];
        if (!(di <= FLT_MAX)) di = INFINITY;
        int rank = 0;
        for (int j = 0; j < n; ++j) {
          float dj = JA32[j * np + j];
          if (!(dj <= FLT_MAX)) dj = INFINITY;
          rank += (dj < di || (dj == di && j < i)) ? 1 : 0;
        }
        sh.perm[rank] = i;
        eps[rank] = (double)di;
      }
      __syncthreads();
    } else if (MIXED && have32) {
      // ---- finishing iteration of mixed mode, in double-float ----
      double* lam = sh.mom;  // n eigenvalues (the moment scratch is free here)
      if (!have64) {
        // FP32 coefficients -> double-float rows, re-orthonormalised in the S
        // metric (the FP32 rows live in the lo plane of B, so this precedes B)
        for (long long e = threadIdx.x; e < (long long)np * np; e += blockDim.x) dm.V[e] = make_float2(JV32[e], 0.f);
        for (long long e = threadIdx.x; e < nn; e += blockDim.x)
          dm.S[e] = make_float2(S32[e], __double2float_rn(S[e] - (double)S32[e]));
        __syncthreads();
        dd_transpose(dm, n, np);
        dd_orthonormalize(dm, n, np, 2, sh);
      }
      dd_rotate_fock(dm, n, np);
      PHASE_MARK(4);
      bool refined = refine_dd(dm, n, lam, 0.2, 1e-4, 6, 1e-5, sh);
#ifdef QCX_SCC_PHASE_TIMING
      if (threadIdx.x == 0) atomicAdd(&g_counts[refined ? 0 : 1], 1ull);
#endif
      if (!refined) {
        // FP64 Jacobi on B in the current basis: planes -> FP64 through the T
        // and C slots, and the rotated rows back to double-float
        float2* tB = (float2*)T;
        float2* tV = (float2*)C;
        const long long np2 = (long long)np * np;
        for (long long e = threadIdx.x; e < np2; e += blockDim.x) {
          tB[e] = dm.B[e];
          tV[e] = dm.V[e];
        }
        __syncthreads();
        for (long long e = threadIdx.x; e < np2; e += blockDim.x) {
          JA[e] = (double)tB[e].x + (double)tB[e].y;
          JV[e] = (double)tV[e].x + (double)tV[e].y;
        }
        __syncthreads();
        for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
          int i = e / n, j = e % n;
          if (j < i) {
            double s = 0.5 * (JA[i * np + j] + JA[j * np + i]);
            JA[i * np + j] = s;
            JA[j * np + i] = s;
          }
        }
        __syncthreads();
        if (jacobi<double>(JA, JV, n, true, 1e-12, sh, 20) < 0) eig_fail = 1;
        for (int i = threadIdx.x; i < n; i += blockDim.x) lam[i] = JA[i * np + i];
        double* tD = C;
        for (long long e = threadIdx.x; e < np2; e += blockDim.x) tD[e] = JV[e];
        __syncthreads();
        for (long long e = threadIdx.x; e < np2; e += blockDim.x) {
          float2 v;
          dd_split(tD[e], v.x, v.y);
          dm.V[e] = v;
        }
        __syncthreads();
        dd_transpose(dm, n, np);
      }
      PHASE_MARK(5);
      have64 = true;
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double di = lam[i];
        if (!(di <= DBL_MAX)) di = INFINITY;
        int rank = 0;
        for (int j = 0; j < n; ++j) {
          double dj = lam[j];
          if (!(dj <= DBL_MAX)) dj = INFINITY;
          rank += (dj < di || (dj == di && j < i)) ? 1 : 0;
        }
        sh.perm[rank] = i;
        eps[rank] = di;
      }
      __syncthreads();
    } else {
      // ---- FP64 iteration ----
      bool cold = false;
      if (!have64) {
        if (MIXED && have32) {
          // FP32 coefficients -> FP64, re-orthonormalised in the S metric with
          // one Newton-Schulz step C^T <- (3I - C^T S C)/2 C^T. The FP32
          // matrices live inside the FP64 A storage, so this precedes any use of A.
          for (long long e = threadIdx.x; e < (long long)np * np; e += blockDim.x) JV[e] = (double)JV32[e];
          __syncthreads();
          cta_gemm<double, double, double, double>(n, n, n, S, n, false, JV, np, true, T, n);
          __syncthreads();
          cta_gemm<double, double, double, double>(n, n, n, JV, np, false, T, n, false, C, n);
          __syncthreads();
          for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
            int i = e / n, j = e % n;
            C[e] = (i == j ? 1.5 : 0.0) - 0.5 * C[e];
          }
          __syncthreads();
          cta_gemm<double, double, double, double>(n, n, n, C, n, false, JV, np, false, T, n);
          __syncthreads();
          for (int e = threadIdx.x; e < n * n; e += blockDim.x) JV[(e / n) * np + (e % n)] = T[e];
          __syncthreads();
        } else {
          cold = true;
        }
      }
      if (cold) {
        cta_gemm<double, double, double, double>(n, n, n, F, n, false, X, n, false, T, n);
        __syncthreads();
        cta_gemm<double, double, double, double>(n, n, n, X, n, true, T, n, false, JA, np);
        __syncthreads();
      } else {
        cta_gemm<double, double, double, double>(n, n, n, F, n, false, JV, np, true, T, n);
        __syncthreads();
        cta_gemm<double, double, double, double>(n, n, n, JV, np, false, T, n, false, JA, np);
        __syncthreads();
      }
      for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        int i = e / n, j = e % n;
        if (j < i) {
          double s = 0.5 * (JA[i * np + j] + JA[j * np + i]);
          JA[i * np + j] = s;
          JA[j * np + i] = s;
        }
      }
      __syncthreads();
      PHASE_MARK(4);
      // FP64 mode: eigenvectors to ~1e-14 every iteration (the oracle's path);
      // mixed mode: one pass suffices once max|K| < 1e-4 (error < 1e-8)
      bool refined = !cold && refine<double>(JA, JV, F, S, T, C, eps, n, 0.2, MIXED ? 1e-4 : 1e-7, 6, 1e-5, sh);
#ifdef QCX_SCC_PHASE_TIMING
      if (threadIdx.x == 0 && !cold) atomicAdd(&g_counts[refined ? 0 : 1], 1ull);
#endif
      if (!refined) {
        int sweeps = jacobi<double>(JA, JV, n, !cold, 1e-12, sh, cold ? 50 : 20);
        if (sweeps < 0) eig_fail = 1;
      }
      PHASE_MARK(5);
      if (cold) {
        cta_gemm<double, double, double, double>(n, n, n, JV, np, false, X, n, true, T, n);
        __syncthreads();
        for (int e = threadIdx.x; e < n * n; e += blockDim.x) JV[(e / n) * np + (e % n)] = T[e];
      }
      have64 = true;
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double di = JA[i * np + i];
        if (!(di <= DBL_MAX)) di = INFINITY;
        int rank = 0;
        for (int j = 0; j < n; ++j) {
          double dj = JA[j * np + j];
          if (!(dj <= DBL_MAX)) dj = INFINITY;
          rank += (dj < di || (dj == di && j < i)) ? 1 : 0;
        }
        sh.perm[rank] = i;
        eps[rank] = di;
      }
      __syncthreads();
    }
    PHASE_MARK(6);
    if (threadIdx.x < 32) {
      double ef;
      double ts = fp32_phase ? fermi_warp32(n, eps, nel, md.kT, focc, &ef, efermi, it > 1)
                             : fermi_warp(n, eps, nel, md.kT, focc, &ef, 1e-13, efermi, it > 1);
      // highest occupied orbital + 1 (occupations are >= 0, so focc > 0 is a
      // test on the bit pattern, not an FP64 compare); the warp has just written focc
      __syncwarp();
      int last = 0;
      for (int k = threadIdx.x; k < n; k += 32)
        if (__double_as_longlong(focc[k]) > 0) last = k + 1;
      for (int o = 16; o > 0; o >>= 1) last = max(last, __shfl_xor_sync(0xffffffffu, last, o));
      if (threadIdx.x == 0) {
        sh.scal[0] = ts;
        sh.scal[1] = ef;
        sh.scal[2] = (double)last;
      }
    }
    __syncthreads();
    ets = sh.scal[0];
    efermi = sh.scal[1];
    nocc = (int)sh.scal[2];
    PHASE_MARK(7);
    // P = C f C^T over the occupied (sorted) orbitals; the FP32 iterations keep
    // P as FP32 (in the P slot) for the FP32 moments
    if (fp32_phase) {
      float* f32 = (float*)sh.rc;  // np floats; the rotation scratch is free after the eigensolve
      for (int k = threadIdx.x; k < nocc; k += blockDim.x) f32[k] = (float)focc[k];
      __syncthreads();
      // P = G^T V_occ with G_k = f_k v_k (rows in occupation order, in the T and C slots)
      float* P32 = (float*)Pm;
      float* G32 = T32;
      float* Vo32 = (float*)C;
      for (int e = threadIdx.x; e < nocc * n; e += blockDim.x) {
        int k = e / n, j = e - k * n;
        float v = JV32[sh.perm[k] * np + j];
        G32[e] = f32[k] * v;
        Vo32[e] = v;
      }
      __syncthreads();
      gemm_t<float>(mc, n, n, nocc, G32, n, true, Vo32, n, false, P32, n);
    } else if (MIXED && have32) {
      dd_density(dm, n, nocc, sh.perm, focc, Pm, sh);
    } else {
      for (long long e = threadIdx.x; e < nn; e += blockDim.x) {
        int i = (int)(e / n), j = (int)(e % n);
        if (j < i) continue;
        double p = 0.0;
        for (int k = 0; k < nocc; ++k) {
          int c = sh.perm[k];
          p += focc[k] * JV[(long long)c * np + i] * JV[(long long)c * np + j];
        }
        Pm[(long long)i * n + j] = p;
        Pm[(long long)j * n + i] = p;
      }
    }
    __syncthreads();
    PHASE_MARK(8);
    // moments: per-AO rows (one warp per row)
    {
      int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
      for (int i = w; i < n; i += kWarps) {
        if (fp32_phase) {
          const float* P32 = (const float*)Pm;
          float acc[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
          for (int j = lane; j < n; j += 32) {
            long long e = (long long)i * n + j;
            float p = P32[e];
            acc[0] += p * S32[e];
#pragma unroll
            for (int c = 0; c < 3; ++c) acc[1 + c] += p * D32[c * nn + e];
#pragma unroll
            for (int c = 0; c < 6; ++c) acc[4 + c] += p * Q32[c * nn + e];
          }
#pragma unroll
          for (int c = 0; c < 10; ++c)
            for (int o = 16; o > 0; o >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
          if (lane == 0)
            for (int c = 0; c < 10; ++c) sh.mom[c * n + i] = (double)acc[c];
        } else {
          double acc[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
          for (int j = lane; j < n; j += 32) {
            long long e = (long long)i * n + j;
            double p = Pm[e];
            acc[0] += p * S[e];
#pragma unroll
            for (int c = 0; c < 3; ++c) acc[1 + c] += p * Dm[c * nn + e];
#pragma unroll
            for (int c = 0; c < 6; ++c) acc[4 + c] += p * Qm[c * nn + e];
          }
#pragma unroll
          for (int c = 0; c < 10; ++c) acc[c] = warp_sum(acc[c]);
          if (lane == 0)
            for (int c = 0; c < 10; ++c) sh.mom[c * n + i] = acc[c];
        }
      }
      __syncthreads();
      for (int s = threadIdx.x; s < nsh; s += blockDim.x) {
        int a = sh_atom[s] - md.atom_off;
        double q = P.refocc[mv.Z[a]][sh_k[s]];
        int l = P.sh_l[mv.Z[a]][sh_k[s]];
        for (int i = 0; i < 2 * l + 1; ++i) q -= sh.mom[sh_ao[s] + i];
        xout[s] = q;
      }
      for (int t = threadIdx.x; t < 9 * nat; t += blockDim.x) {
        int a = t / 9, c = t % 9;
        double v = 0.0;
        for (int i = 0; i < n; ++i)
          if (sh.ao_at[i] == a) v -= sh.mom[(1 + c) * n + i];
        if (c < 3) xout[nsh + 3 * a + c] = v;
        else xout[nsh + 3 * nat + 6 * a + (c - 3)] = v;
      }
      __syncthreads();
    }
    PHASE_MARK(9);
    // FP32 iterations only need the residual; the potentials of the output
    // moments (energy, and the gradient after the loop) are FP64-phase work
    if (!fp32_phase) potentials(mv, xout, en, sh.red);
    PHASE_MARK(10);
    bool stop = false;
    double res_it = 0.0;
    {
      double acc[2] = {0.0, 0.0};
      // the band energy only enters the FP64 convergence test
      if (!fp32_phase)
        for (long long e = threadIdx.x; e < nn; e += blockDim.x) acc[0] += Pm[e] * H0[e];
      for (int i = threadIdx.x; i < len; i += blockDim.x) {
        double d = xout[i] - xin[i];
        acc[1] += d * d;
      }
      cta_sum<2>(acc, sh.red);
      eband = acc[0];
      double res = sqrt(acc[1] / len);
      res_it = res;
      eel = eband + en[0] + en[1] + en[2] + en[3] + en[4] + ets;
      double de = fabs(eel - eprev);
#ifdef QCX_SCC_TRACE
      if (mol == 0 && threadIdx.x == 0 && it <= QCX_SCC_MAXITER) {
        g_trace[it][0] = res;
        g_trace[it][1] = de;
        g_trace[it][2] = eel;
        g_trace[it][3] = fp32_phase ? 1.0 : 0.0;
        g_trace[it][4] = efermi;
        g_trace[it][5] = (double)nocc;
      }
      if (mol == 0 && it <= QCX_SCC_MAXITER)
        for (int i = threadIdx.x; i < 128; i += blockDim.x) {
          g_trace_vec[it][0][i] = i < n ? eps[i] : 0.0;
          g_trace_vec[it][1][i] = i < n ? focc[i] : 0.0;
          g_trace_vec[it][2][i] = i < len ? xin[i] : 0.0;
          g_trace_vec[it][3][i] = i < len ? xout[i] : 0.0;
        }
#endif
      eprev = eel;
      if (fp32_phase) {
        // hand over to FP64 once the FP32 iterations reach their noise floor
        // (or once the FP32 residual has stopped improving below 1e-3); the
        // mixer keeps its history across the hand-over
        if (res < 0.9 * best32) {
          best32 = res;
          stall32 = 0;
        } else {
          ++stall32;
        }
        if ((it > 1 && res < kMixedSwitch) || (stall32 >= 4 && res < QCX_STALL_HANDOVER) || it >= QCX_FP32_MAXIT ||
            it >= bt.max_iter - 12)
          fp32_phase = false;
      } else {
        ++n64;
        // convergence needs two FP64 iterations so that dE compares FP64 energies
        if (it > 1 && (n64 >= 2 || !MIXED) && de < bt.econv && res < bt.pconv) {
          converged = 1;
          stop = true;
        }
      }
    }
    PHASE_MARK(11);
    if (stop || it == bt.max_iter) break;
    // charge sloshing between near-degenerate states can hold the Broyden
    // history at a residual of ~3e-2 for tens of iterations: restart it
    if (res_it < 0.9 * rbest) {
      rbest = res_it;
      rsince = 0;
    } else if (++rsince >= QCX_BROYDEN_RESTART) {
      bro_it = 0;
      rbest = res_it;
      rsince = 0;
    }
    broyden(mv, xin, xout, bro_it, bt.mix_alpha, sh);
    ++bro_it;
    PHASE_MARK(12);
    if (budget > 0 && it - it0 + 1 >= budget && (!MIXED || fp32_phase)) {
      suspended = true;
      break;
    }
  }
  if (it > bt.max_iter) it = bt.max_iter;
  if (suspended && !(mc && !mctx.ok)) {
    // keep the state for the next launch: the mixer's input moments (xin) and
    // history are in the vector block already; the FP32 eigenvectors go to
    // the B32 region (the FP64 path restarts its eigensolve cold)
    const bool keep_basis = MIXED && have32;
    if (keep_basis)
      for (int e = threadIdx.x; e < n * n; e += blockDim.x) B32[e] = JV32[(e / n) * np + (e % n)];
    if (threadIdx.x == 0) {
      SccCarry c{};
      c.it = it;
      c.bro_it = bro_it;
      c.phase32 = fp32_phase ? 1 : 0;
      c.stall32 = stall32;
      c.backoff32 = backoff32;
      c.n64 = n64;
      c.eig_fail = eig_fail;
      c.basis = keep_basis ? 1 : 0;
      c.best32 = best32;
      c.rbest = rbest;
      c.rsince = rsince;
      c.eprev = eprev;
      c.efermi = efermi;
      bt.carry[mol] = c;
      bt.status[mol] = kSccPending;
      bt.iters[mol] = it;
      if (bt.iter_sum) bt.iter_sum[mol] += it - it0 + 1;
      if (bt.have_prev) bt.have_prev[mol] = basis_saved ? 2 : 0;
    }
    if (mc) mma_teardown(mctx);
    return;
  }
#ifdef QCX_SCC_PHASE_TIMING
  if (threadIdx.x == 0 && mol < 4096) g_mol_cycles[mol] = (unsigned long long)(clock64() - _t_start);
#endif
  // energy-weighted density W = C f e C^T (coefficients of the last iteration)
  int nocc = 0;
  for (int k = 0; k < n; ++k)
    if (focc[k] > 0.0) nocc = k + 1;
  if (MIXED && have32) {
    double* w = sh.mom;
    for (int k = threadIdx.x; k < nocc; k += blockDim.x) w[k] = focc[k] * eps[k];
    __syncthreads();
    dd_density(dm, n, nocc, sh.perm, w, Wm, sh);
  } else {
    for (long long e = threadIdx.x; e < nn; e += blockDim.x) {
      int i = (int)(e / n), j = (int)(e % n);
      if (j < i) continue;
      double w = 0.0;
      for (int k = 0; k < nocc; ++k) {
        int c = sh.perm[k];
        w += focc[k] * eps[k] * JV[(long long)c * np + i] * JV[(long long)c * np + j];
      }
      Wm[(long long)i * n + j] = w;
      Wm[(long long)j * n + i] = w;
    }
  }
  // the orbitals of the last iteration for the MO populations of the spectrum
  // path: row k of the C slot = AO coefficients of the k-th orbital by energy
  if (!MIXED && bt.keep_mo) {
    for (long long e = threadIdx.x; e < nn; e += blockDim.x) {
      const int k = (int)(e / n), i = (int)(e - (long long)k * n);
      C[e] = JV[(long long)sh.perm[k] * np + i];
    }
  }
  // outputs
  for (int a = threadIdx.x; a < nat; a += blockDim.x) bt.qat[md.atom_off + a] = vec[mv.vl.qat + a];
  if (threadIdx.x == 0) {
    double* E = bt.energy + (long long)mol * kNumEnergy;
    E[kEBand] = eband;
    E[kEIes] = en[0];
    E[kE3] = en[1];
    E[kEAes] = en[2];
    E[kEAxc] = en[3];
    E[kEDisp] = en[4];
    E[kETs] = ets;
    E[kEFermi] = efermi;
    E[kIters64] = (double)(MIXED ? n64 : it);
    E[kETotal] = eel;  // electronic part; three-body and repulsion added by the gradient kernel
    int st = 0;
    if (!converged) st |= kSccNotConverged;
    if (eig_fail) st |= kEigenNotConverged;
    if (mc && !mctx.ok) st |= kEigenNotConverged | kNonFinite;  // a tensor-core wait ran out
    if (!isfinite(eel)) st |= kNonFinite;
    bt.status[mol] = st;
    if (bt.have_prev) bt.have_prev[mol] = (st == 0 ? 1 : 0) | (basis_saved ? 2 : 0);
    bt.iters[mol] = it;
    if (bt.iter_sum) bt.iter_sum[mol] += it - it0 + 1;
  }
  if (mc) mma_teardown(mctx);
}

#ifdef QCX_SCC_PHASE_TIMING
}  // namespace qcx
extern "C" int qcx_debug_refine32(unsigned long long* out, int reset) {
  if (cudaMemcpyFromSymbol(out, qcx::g_refine32, sizeof(unsigned long long) * 16) != cudaSuccess) return -1;
  if (reset) {
    unsigned long long z[16] = {0};
    cudaMemcpyToSymbol(qcx::g_refine32, z, sizeof(z));
  }
  return 0;
}
extern "C" int qcx_debug_counts(unsigned long long* out, int reset) {
  if (cudaMemcpyFromSymbol(out, qcx::g_counts, sizeof(unsigned long long) * 8) != cudaSuccess) return -1;
  if (reset) {
    unsigned long long z[8] = {0};
    cudaMemcpyToSymbol(qcx::g_counts, z, sizeof(z));
  }
  return 0;
}
extern "C" int qcx_debug_mol_cycles(unsigned long long* out, int n) {
  return cudaMemcpyFromSymbol(out, qcx::g_mol_cycles, sizeof(unsigned long long) * (n < 4096 ? n : 4096)) ==
                 cudaSuccess ? 0 : -1;
}
extern "C" int qcx_debug_phase_cycles(unsigned long long* out, int reset) {
  if (cudaMemcpyFromSymbol(out, qcx::g_phase_cycles, sizeof(unsigned long long) * 24) != cudaSuccess) return -1;
  if (reset) {
    unsigned long long z[24] = {0};
    cudaMemcpyToSymbol(qcx::g_phase_cycles, z, sizeof(z));
  }
  return 0;
}
namespace qcx {
#endif

// Self-check of the FP32 eigensolver through the C ABI: one CTA of the SCC
// kernel's shape diagonalises a symmetric host matrix with the cyclic parallel
// Jacobi of the FP32 iterations, in shared memory as in the SCC.
__global__ void __launch_bounds__(kSccThreads, 1) k_jacobi32_selftest(int n, const float* Ain, float* Aout,
                                                                       float* Vout, int warm, double reltol,
                                                                       int max_sweeps, int* sweeps, float* Ag,
                                                                       float* Vg) {
  extern __shared__ __align__(1024) char smem_raw[];
  const int np = n + (n & 1);
  // the matrices in shared memory when they fit (Ag == nullptr), else in the
  // global buffers, as the SCC kernel keeps them for large molecules
  const bool shared = Ag == nullptr;
  float* A = shared ? (float*)smem_raw : Ag;
  float* Vt = shared ? A + (size_t)np * np : Vg;
  double* red = (double*)(smem_raw + (shared ? sizeof(float) * 2 * (size_t)np * np : 0));
  int* rq = (int*)(red + 16 * kWarps);
  float* rc = (float*)(rq + 2 * 256);
  SccShared sh{};
  sh.red = red;
  sh.rp = rq;
  sh.rq = rq + 256;
  sh.rc = (double*)rc;
  for (int i = threadIdx.x; i < np * np; i += blockDim.x) {
    const int r = i / np, c = i % np;
    A[i] = (r < n && c < n) ? Ain[r * n + c] : 0.f;
    Vt[i] = (r < n && c < n) ? Vout[r * n + c] : (r == c ? 1.f : 0.f);
  }
  __syncthreads();
  const int sw = jacobi<float>(A, Vt, n, warm != 0, reltol, sh, max_sweeps);
  __syncthreads();
  for (int i = threadIdx.x; i < n * n; i += blockDim.x) {
    const int r = i / n, c = i % n;
    Aout[i] = A[r * np + c];
    Vout[i] = Vt[r * np + c];
  }
  if (threadIdx.x == 0) *sweeps = sw;
}

#ifdef QCX_SCC_TRACE
}  // namespace qcx
extern "C" int qcx_debug_trace(double* out) {
  return cudaMemcpyFromSymbol(out, qcx::g_trace, sizeof(double) * (QCX_SCC_MAXITER + 1) * 6) == cudaSuccess ? 0 : -1;
}
extern "C" int qcx_debug_trace_vec(double* out) {
  return cudaMemcpyFromSymbol(out, qcx::g_trace_vec, sizeof(double) * (QCX_SCC_MAXITER + 1) * 4 * 128) == cudaSuccess
             ? 0 : -1;
}
namespace qcx {
#endif

void launch_scc(const DevBatch& bt, int precision, cudaStream_t st) {
  // The shared-memory limit is a per-device attribute of each kernel: set it
  // once on every device this process launches on (one bit per device index;
  // two threads racing to set it both set the same value).
  static std::atomic<unsigned long long> configured{0};
  int dev = 0;
  cudaGetDevice(&dev);
  const unsigned long long bit = 1ull << (dev & 63);
  if (!(configured.load(std::memory_order_acquire) & bit)) {
    cudaFuncSetAttribute(k_scc<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemCap);
    cudaFuncSetAttribute(k_scc<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemCap);
    configured.fetch_or(bit, std::memory_order_release);
  }
  if (precision == 1)
    k_scc<1><<<bt.nmol, kSccThreads, bt.smem_bytes, st>>>(bt);
  else
    k_scc<0><<<bt.nmol, kSccThreads, bt.smem_bytes, st>>>(bt);
}

}  // namespace qcx

extern "C" int qcx_jacobi32_selftest(int n, const float* A, float* Aout, float* V, int warm, double reltol,
                                     int max_sweeps, int* sweeps) {
  using namespace qcx;
  if (n < 1 || n > 256 || !A || !Aout || !V || !sweeps || max_sweeps < 1 || !(reltol > 0.0)) {
    set_last_error("qcx_jacobi32_selftest: 1 <= n <= 256, max_sweeps >= 1, reltol > 0");
    return -1;
  }
  const int np = n + (n & 1);
  const size_t mats = sizeof(float) * 2 * (size_t)np * np;
  const size_t rest = sizeof(double) * 16 * kWarps + sizeof(int) * 512 + sizeof(float) * 512;
  const bool in_shared = mats + rest <= 200 * 1024;
  const size_t smem = (in_shared ? mats : 0) + rest;
  float *dA = nullptr, *dAo = nullptr, *dV = nullptr, *dAg = nullptr, *dVg = nullptr;
  int* dsw = nullptr;
  const size_t nb = sizeof(float) * (size_t)n * n;
  cudaError_t e = cudaSuccess;
  if (!in_shared) {
    e = cudaMalloc(&dAg, sizeof(float) * (size_t)np * np);
    if (e == cudaSuccess) e = cudaMalloc(&dVg, sizeof(float) * (size_t)np * np);
  }
  if (e == cudaSuccess) e = cudaMalloc(&dA, nb);
  if (e == cudaSuccess) e = cudaMalloc(&dAo, nb);
  if (e == cudaSuccess) e = cudaMalloc(&dV, nb);
  if (e == cudaSuccess) e = cudaMalloc(&dsw, sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpy(dA, A, nb, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dV, V, nb, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_jacobi32_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) {
    k_jacobi32_selftest<<<1, kSccThreads, smem>>>(n, dA, dAo, dV, warm, reltol, max_sweeps, dsw, dAg, dVg);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(Aout, dAo, nb, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(V, dV, nb, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(sweeps, dsw, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(dA);
  cudaFree(dAo);
  cudaFree(dV);
  cudaFree(dsw);
  cudaFree(dAg);
  cudaFree(dVg);
  if (e != cudaSuccess) {
    set_last_error(std::string("qcx_jacobi32_selftest: ") + cudaGetErrorString(e));
    return -1;
  }
  return 0;
}
