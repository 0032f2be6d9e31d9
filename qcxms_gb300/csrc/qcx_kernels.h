// Kernel launchers shared between the translation units of libqcxgpu.
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "qcx_batch.cuh"

struct qcx_batch;  // the batch handle of the C ABI (include/qcxgpu.h)

namespace qcx {

void launch_cn(const DevBatch& bt, cudaStream_t st);
// The shell-pair kernels launch one specialised kernel per angular-momentum
// class; they return the number of kernels launched.
int launch_integrals(const DevBatch& bt, cudaStream_t st);
void launch_scc(const DevBatch& bt, int precision, cudaStream_t st);
int launch_grad_pairs(const DevBatch& bt, cudaStream_t st);
void launch_grad_atoms(const DevBatch& bt, cudaStream_t st);
void launch_leapfrog(const DevBatch& bt, double tstep, cudaStream_t st);
void launch_zero_grad(const DevBatch& bt, cudaStream_t st);
// checkqc (src/iniqm.f90:684-715) of one result in device memory: *code = 0
// accepted, 1 |E| < 1e-8, 2 gradient norm, 3 charges; *e set to 0 for 2 and 3
void launch_checkqc(int nat, const double* grad, const double* qat, double charge, double* e, int* code,
                    cudaStream_t st);
// normalised Mulliken populations of every orbital of molecule mol on every
// atom (qmo [nao][nat], write_qmo, src/mo_energ.f90:7-80), from the orbitals a
// keep_mo SCC left in the kC slot
void launch_mo_pops(const DevBatch& bt, int mol, int nao, double* qmo, cudaStream_t st);
// fragment numbers of every molecule's atoms (frag[natom]) and fragment counts (nfrag[nmol])
// skip_last = 1: the last atom of every molecule is left out (fragment 0)
void launch_fragments(const DevBatch& bt, int max_nat, const double* rad, double rcut, int at1, int at2, int* frag,
                      int* nfrag, cudaStream_t st, int skip_last = 0);

// Per-trajectory state of the MD bookkeeping and exit rules (src/md.f90:285-682)
struct MdState {
  int nstep, nfrag, fconst, morestep, fragstate, mdok, done, heat_failed;
  int nadd, kdump;  // kdump: steps in the current window of the averaged structure (src/md.f90:352-362)
  double tav, epav, ekav, edum, eerror, ttime, dtime;
  double eimp, fadd, ekinstart;  // heating of the first nadd steps (impactscale)
  double fragT[10];
  double etemp;  // electronic temperature (K) of the next evaluation when the per-step etemp is on
};
struct MdRules {
  int nfragexit, more, max_steps;
  int max_nat;  // largest molecule (per-warp scratch of the heating)
  double tstep;
  // per-step electronic temperature (setetemp, src/utility.f90:69-86, called by
  // src/md.f90:443-446 after every step): on, ax and ieetemp of the input
  int etemp_on;
  double ax, ieetemp;
};
// setetemp (src/utility.f90:69-86): 5000 + 20000 ax, plus eimp * ieetemp while
// eimp > 0 and the molecule is one fragment (5000. and 20000. are
// default-real literals, exact in FP32)
__host__ __device__ inline double setetemp(int nfrag, double eimp, double ax, double ieetemp) {
  double etemp = 5000.0 + 20000.0 * ax;
  if (eimp > 0.0 && nfrag <= 1) etemp = etemp + (eimp > 0.0 ? eimp : 0.0) * ieetemp;
  return etemp;
}
// heat [nmol][3] = (eimp, fadd, nadd) or nullptr (no heating); velof [natom] or nullptr
// avxyz [natom][3]: running sum of the coordinates over the current window of avdump = 50 steps
// etemp0 [nmol] (or nullptr): the electronic temperature of the start (set by qcx_batch_set_md_etemp)
void launch_md_begin(const DevBatch& bt, MdState* st, const double* heat, double* avxyz, const double* etemp0,
                     cudaStream_t stream);
void launch_md_rules(const DevBatch& bt, MdState* st, const int* frag, const int* nfrag, const double* velof,
                     double* avxyz, const MdRules& r, cudaStream_t stream);

// Per-trajectory state of the collision MD stop rules (src/cid.f90:739-1052);
// the last atom of every molecule is the collision gas atom
struct CidState {
  int nstep, m, step_counter, collided, fragmented, total_steps, nfrag, done, failed, distance_dump;
  double ttime, tav, avgT, lowest, highest, new_temp, ecom, summass;
  double old_cm[3];
  // averaged structures (src/cid.f90:743-746, 802-909): the window counter of
  // avxyz, the count of avxyz2, whether the fragments' structure is averaged,
  // the fragment count that started it and the fragments' atom counts then
  int xyzavg_dump, cnt, count_average, check_fragmented;
  int save_natf[10];
};
struct CidRules {
  double tinit, tstep;
  int ntot;
};
// cav [natom][9]: per ion atom avxyz (3), avxyz2 (3) and store_avxyz (3)
void launch_cid_begin(const DevBatch& bt, CidState* st, double* cav, const CidRules& r, cudaStream_t stream);
void launch_cid_rules(const DevBatch& bt, CidState* st, const int* frag, const int* nfrag, double* cav,
                      const CidRules& r, cudaStream_t stream);

// sets the text qcx_last_error() returns
void set_last_error(const std::string& s);
// the same from a C string, without allocating
void set_last_error_text(const char* s);
// mixed mode: molecules with fewer atomic orbitals run FP64 SCC iterations only
// (0 by default; set before the batch's first evaluation)
void batch_set_mixed_min_nao(::qcx_batch* b, int n);
// 0: results are not put through checkqc (the fragment single points of
// analyse go through eqm, which does not call it); 1 (default): egrad's checks
void batch_set_checkqc(::qcx_batch* b, int on);

// dynamic shared memory the SCC kernel asks for, given the largest molecule
size_t scc_smem_bytes(int max_nao, int precision);

}  // namespace qcx
