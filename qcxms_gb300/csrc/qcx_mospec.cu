// MO populations of the spectrum path: get_xtb_egrad(spec_calc=.true.)
// (src/tblite.f90:153-166) passes the overlap, the AO-to-atom map and the
// orbitals of the converged SCC to write_qmo (src/mo_energ.f90:7-80), which
// forms per orbital k and atom a
//   qmo(k,a) = sum_{j on a} sum_l (C(j,k) C(l,k)) S(j,l) + 1e-10
// (j and l ascending) and divides each orbital's row by its sum over the
// atoms (atoms ascending). One CTA per molecule; a thread per (orbital,
// atom) pair keeps the reference's summation order, with explicit roundings.
#include "qcx_batch.cuh"
#include "qcx_device.cuh"
#include "qcx_kernels.h"

namespace qcx {

namespace {

constexpr int kPopThreads = 256;

// qmo [nao][nat] of molecule mol; the kC slot holds the orbitals by energy
// (row k = the AO coefficients of orbital k), kS the overlap
__global__ void __launch_bounds__(kPopThreads) k_mo_pops(const DevBatch bt, int mol, double* qmo) {
  extern __shared__ int ao_at[];
  const MolDesc md = bt.mol[mol];
  const int n = md.nao, nat = md.nat;
  const Params& P = *bt.prm;
  const double* S = mat_ptr(bt, md, kS);
  const double* C = mat_ptr(bt, md, kC);
  for (int s = threadIdx.x; s < md.nsh; s += blockDim.x) {
    const int a = bt.sh_atom[md.sh_off + s] - md.atom_off;
    const int l = P.sh_l[bt.Z[md.atom_off + a]][bt.sh_k[md.sh_off + s]];
    for (int i = 0; i < 2 * l + 1; ++i) ao_at[bt.sh_ao[md.sh_off + s] + i] = a;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < n * nat; e += blockDim.x) {
    const int k = e / nat, a = e - k * nat;
    const double* ck = C + (long long)k * n;
    double sum = 0.0;
    for (int j = 0; j < n; ++j) {
      if (ao_at[j] != a) continue;
      const double cj = ck[j];
      const double* sj = S + (long long)j * n;
      for (int l = 0; l < n; ++l) sum = __dadd_rn(sum, __dmul_rn(__dmul_rn(cj, ck[l]), sj[l]));
    }
    qmo[e] = __dadd_rn(sum, 1e-10);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    double* row = qmo + (long long)k * nat;
    double sum = 0.0;
    for (int a = 0; a < nat; ++a) sum = __dadd_rn(sum, row[a]);
    for (int a = 0; a < nat; ++a) row[a] = __ddiv_rn(row[a], sum);
  }
}

}  // namespace

void launch_mo_pops(const DevBatch& bt, int mol, int nao, double* qmo, cudaStream_t st) {
  k_mo_pops<<<1, kPopThreads, sizeof(int) * (size_t)nao, st>>>(bt, mol, qmo);
}

}  // namespace qcx
