// Device layout of a batch of independent trajectories (one molecule each).
//
// All molecules of a batch live in flat pools; a MolDesc gives each
// molecule's offsets. Per-molecule dense matrices are n x n row-major blocks
// (n = number of atomic orbitals); indices inside a molecule are local.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "qcx_device.cuh"

namespace qcx {

// matrix slots inside a molecule's matrix block (each np*np doubles).
// kS32 holds FP32 copies of S (first n*n floats) and H0 (next n*n floats);
// kD32 the three dipole and kQ32 the six quadrupole matrices in FP32 (n*n
// floats each, spanning the slots that follow them). The FP32 SCC iterations
// read these instead of converting the FP64 matrices element by element.
enum MatSlot {
  kS = 0, kH0, kX, kF, kT, kA, kV, kC, kP, kW,
  kDm0, kDm1, kDm2,
  kQm0, kQm1, kQm2, kQm3, kQm4, kQm5,
  kS32, kD32, kD32b, kQ32, kQ32b, kQ32c,
  kNumMat
};

// per-molecule energy terms
enum EnergySlot {
  kEBand = 0, kEIes, kE3, kEAes, kEAxc, kEDisp, kEAtm, kERep, kETs, kETotal, kEFermi, kIters64, kNumEnergy
};

// per-molecule status bits
enum Status : int {
  kOk = 0,
  kSccNotConverged = 1,
  kNonFinite = 2,
  kCholeskyFailed = 4,
  kEigenNotConverged = 8,
  // checkqc (src/iniqm.f90:684-715) rejected the result
  kCheckqcFailed = 16,
  // the SCC used up its iteration budget of one launch (qcx_batch_set_scc_budget)
  // before converging: the next launch resumes it at the same geometry, and
  // until then the trajectory neither moves nor counts a step
  kSccPending = 32,
};
// evaluations that end a trajectory whatever checkqc says
constexpr int kFailedEval = kSccNotConverged | kNonFinite | kCholeskyFailed;

// SCC state kept between the launches of a suspended SCC (kSccPending); the
// moment vector and the Broyden history stay in the molecule's vector block
struct SccCarry {
  int it;         // iterations done
  int bro_it;     // Broyden updates since the mixer's last restart
  int phase32;    // mixed mode: still in the FP32 iterations
  int stall32, backoff32, n64, eig_fail;
  int basis;      // mixed mode: the FP32 eigenvectors were saved (B32 region of the kD32 slots)
  int rsince;     // iterations since the residual last improved by 10 % (mixer restart)
  double best32, eprev, efermi, rbest;
};

struct MolDesc {
  int nat, nsh, nao, len;      // len = nsh + 9 nat (mixed moment vector)
  int atom_off, sh_off;        // offsets into atom / shell arrays
  int nmem;                    // Broyden history capacity
  int pad_;
  long long mat_off;           // offset (doubles) of the matrix block
  long long vec_off;           // offset (doubles) of the vector block
  double nel, kT, charge, pad2_;
};

// offsets inside a molecule's vector block
struct VecLayout {
  // gdisp: BJ kernel g_AB of every atom pair; wq, dwq, zq: per atom and D4
  // reference, gw zeta(q), gw dzeta/dq and zeta(q) at the last potentials' charges
  long long eps, focc, xin, xout, vsh, vdp, vqp, qat, vat, gam, gdisp, f3, f5, d3r, d3r0, d5r, d5r0, wq, dwq, zq,
      bdf, bu, ba, bxl, bfl, bc, bm, total;
  __host__ __device__ static VecLayout make(int nat, int nsh, int nao, int len, int nmem) {
    VecLayout v;
    long long o = 0;
    auto take = [&o](long long n) {
      long long r = o;
      o += (n + 3) & ~3LL;  // keep 32-byte alignment
      return r;
    };
    v.eps = take(nao);
    v.focc = take(nao);
    v.xin = take(len);
    v.xout = take(len);
    v.vsh = take(nsh);
    v.vdp = take(3LL * nat);
    v.vqp = take(6LL * nat);
    v.qat = take(nat);
    v.vat = take(nat);
    v.gam = take((long long)nsh * nsh);
    v.gdisp = take((long long)nat * nat);
    v.f3 = take((long long)nat * nat);
    v.f5 = take((long long)nat * nat);
    v.d3r = take((long long)nat * nat);
    v.d3r0 = take((long long)nat * nat);
    v.d5r = take((long long)nat * nat);
    v.d5r0 = take((long long)nat * nat);
    v.wq = take((long long)kMaxRef * nat);
    v.dwq = take((long long)kMaxRef * nat);
    v.zq = take((long long)kMaxRef * nat);
    v.bdf = take((long long)nmem * len);
    v.bu = take((long long)nmem * len);
    v.ba = take((long long)nmem * nmem);
    v.bxl = take(len);
    v.bfl = take(len);
    v.bc = take(nmem);
    v.bm = take((long long)nmem * nmem + nmem);
    v.total = o;
    return v;
  }
};

struct ShellPair {
  int s, t;  // global shell indices (same molecule)
};

// Pointers handed to every kernel of a batch (by value).
struct DevBatch {
  int nmol, natom, nshell, npair;
  const Params* prm;
  const MolDesc* mol;
  // atoms (global index)
  const int* Z;
  const int* atom_mol;
  double* xyz;     // [natom][3]
  double* grad;    // [natom][3]
  double* vel;     // [natom][3]
  const double* mass;
  double* cn;
  double* cnd;
  double* dedcn;
  double* dedcnd;
  double* mrad;
  double* dmrad;
  double* w4;      // [natom][kMaxRef] D4 reference weights at the covalent CN
  double* dw4;     // [natom][kMaxRef] their CN derivatives
  double* qat;     // output atomic charges
  // shells (global index)
  const int* sh_atom;  // global atom index
  const int* sh_k;     // shell index within the element
  const int* sh_ao;    // local AO offset within the molecule
  // shell pairs (ordered, both directions, same molecule)
  const ShellPair* pairs;  // grouped by angular-momentum class l_a*3 + l_b
  int pair_off[10];        // class c occupies pairs[pair_off[c] .. pair_off[c+1])
  // pools
  double* mats;
  double* vecs;
  double* energy;  // [nmol][kNumEnergy]
  int* status;     // [nmol]
  int* iters;      // [nmol]
  double* ekin;    // [nmol]
  int* active;     // [nmol] 1 while the trajectory runs; 0 after a failed evaluation
  long long* steps_done;  // [nmol] successful energy+gradient evaluations
  int* have_prev;    // [nmol] 1 when the moment vector of a converged SCC at an earlier geometry is kept
  int guess;         // SCC start: 0 = zero moments (a fresh wavefunction every call), 1 = the kept moments
  int checkqc;       // 1: apply checkqc after every evaluation, as egrad does (src/iniqm.f90:650)
  int keep_mo;       // 1: the FP64 SCC leaves its last orbitals, by energy, as the rows of the kC slot
  // per-launch SCC budget: 0 = every SCC runs to convergence (or max_iter) in
  // one launch; b > 0 = a molecule of budget_nao AOs stops after b iterations,
  // a molecule of n AOs after ceil(b (budget_nao / n)^2), and resumes in the
  // next launch (kSccPending)
  int scc_budget, budget_nao;
  SccCarry* carry;   // [nmol] (allocated with the first nonzero budget)
  long long* iter_sum;  // [nmol] SCC iterations run so far (all launches)
  // atom-level kernels of one molecule group: the group's atoms (nullptr: all natom atoms)
  const int* atom_list;
  int natom_list;
  const int* order;  // [nmol] molecules by decreasing size: CTA b of a per-molecule kernel takes order[b]
  int max_nao;
  int smem_bytes;  // dynamic shared memory granted to the SCC kernel
  // SCC controls
  int max_iter;
  int mixed_min_nao;  // mixed mode: molecules with fewer AOs run FP64 iterations only
  double econv, pconv, mix_alpha;
};

// every matrix slot holds np*np doubles, np = nao rounded up to even, so the
// padded Jacobi matrices fit in a slot; S, H0, ... use leading dimension nao.
__host__ __device__ inline long long slot_size(int nao) {
  long long np = nao + (nao & 1);
  return np * np;
}

__host__ __device__ inline bool scc_pending(const DevBatch& b, int mol) {
  return (b.status[mol] & kSccPending) != 0;
}

__host__ __device__ inline double* mat_ptr(const DevBatch& b, const MolDesc& m, int slot) {
  return b.mats + m.mat_off + (long long)slot * slot_size(m.nao);
}

}  // namespace qcx
