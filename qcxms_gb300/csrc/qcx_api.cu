// Host side of libqcxgpu: batch construction, launch sequencing, CUDA graph
// capture of one MD step, and the C ABI declared in include/qcxgpu.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/qcxgpu.h"
#include "qcx_batch.cuh"
#include "qcx_d4host.h"
#include "qcx_kernels.h"

using namespace qcx;

// number of molecule groups whose SCC and gradient kernels run on separate streams
#ifndef QCX_MOL_GROUPS
#define QCX_MOL_GROUPS 8
#endif

namespace {

// Text of the last failure of the calling thread: a fixed buffer, so that
// setting it allocates nothing (qcx_egrad_noalloc sets it too).
constexpr size_t kErrLen = 512;
thread_local char g_last_error[kErrLen] = {0};

void set_error_text(const char* s) { std::snprintf(g_last_error, kErrLen, "%s", s ? s : ""); }
void set_error(const std::string& s) { set_error_text(s.c_str()); }

#define CK(call)                                                                   \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess) {                                                       \
      set_error(std::string(#call) + ": " + cudaGetErrorString(e_));              \
      return -1;                                                                   \
    }                                                                              \
  } while (0)

double prim_norm(double a, int l) { return std::pow(2.0 * a / QCX_PI, 0.75) * std::pow(4.0 * a, 0.5 * l); }

void fill_params(Params& p) {
  std::memset(&p, 0, sizeof(p));
  for (int z = 0; z <= kMaxZ; ++z) {
    p.nsh[z] = qcx_nsh[z];
    for (int k = 0; k < kMaxSh; ++k) {
      p.sh_l[z][k] = qcx_sh_l[z][k];
      p.sh_nprim[z][k] = qcx_sh_nprim[z][k];
      p.zeta[z][k] = qcx_sh_zeta[z][k];
      p.refocc[z][k] = qcx_sh_refocc[z][k];
      p.selfenergy[z][k] = qcx_sh_selfenergy[z][k];
      p.kcn[z][k] = qcx_sh_kcn[z][k];
      p.kpoly[z][k] = qcx_sh_kpoly[z][k];
      p.hardness[z][k] = qcx_sh_hardness[z][k];
      p.gamma3[z][k] = qcx_sh_gamma3[z][k];
      for (int i = 0; i < kMaxPrim; ++i) {
        p.alpha[z][k][i] = qcx_prim_alpha[z][k][i];
        p.cnorm[z][k][i] = (i < qcx_sh_nprim[z][k] && z > 0 && k < qcx_nsh[z])
                               ? qcx_prim_coeff[z][k][i] * prim_norm(qcx_prim_alpha[z][k][i], qcx_sh_l[z][k])
                               : 0.0;
      }
    }
    p.en[z] = qcx_en[z];
    p.rcov[z] = qcx_rcov[z];
    p.rep_alpha[z] = qcx_rep_alpha[z];
    p.rep_zeff[z] = qcx_rep_zeff[z];
    p.aes_dk[z] = qcx_aes_dkernel[z];
    p.aes_qk[z] = qcx_aes_qkernel[z];
    p.aes_rad0[z] = qcx_aes_rad0[z];
    p.aes_valcn[z] = qcx_aes_valcn[z];
  }
  fill_d4_params(p);
}

template <typename T>
int dalloc(T** p, size_t n) {
  if (n == 0) n = 1;
  CK(cudaMalloc((void**)p, sizeof(T) * n));
  return 0;
}

// Timing events of one call, destroyed on every return path.
struct CallEvents {
  std::vector<cudaEvent_t> ev;
  explicit CallEvents(size_t n) : ev(n, nullptr) {}
  ~CallEvents() {
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
  }
  cudaError_t create() {
    for (cudaEvent_t& e : ev) {
      const cudaError_t r = cudaEventCreate(&e);
      if (r != cudaSuccess) {
        e = nullptr;
        return r;
      }
    }
    return cudaSuccess;
  }
  cudaEvent_t operator[](size_t i) const { return ev[i]; }
};

}  // namespace

struct qcx_batch {
  int nmol = 0, natom = 0, nshell = 0, npair = 0, max_nao = 0;
  std::vector<MolDesc> mol;
  std::vector<int> Z;
  cudaStream_t stream = nullptr;
  DevBatch dev{};
  // device allocations
  Params* d_prm = nullptr;
  MolDesc* d_mol = nullptr;
  int *d_Z = nullptr, *d_atom_mol = nullptr, *d_sh_atom = nullptr, *d_sh_k = nullptr, *d_sh_ao = nullptr;
  ShellPair* d_pairs = nullptr;
  double *d_xyz = nullptr, *d_grad = nullptr, *d_vel = nullptr, *d_mass = nullptr;
  double *d_cn = nullptr, *d_cnd = nullptr, *d_dedcn = nullptr, *d_dedcnd = nullptr, *d_mrad = nullptr,
         *d_dmrad = nullptr, *d_w4 = nullptr, *d_dw4 = nullptr, *d_qat = nullptr;
  double *d_mats = nullptr, *d_vecs = nullptr, *d_energy = nullptr, *d_ekin = nullptr;
  int *d_status = nullptr, *d_iters = nullptr, *d_active = nullptr, *d_order = nullptr, *d_have_prev = nullptr;
  int *d_frag = nullptr, *d_nfrag = nullptr;  // fragment numbers [natom], counts [nmol]
  double* d_frad = nullptr;                   // QCxMS fragment radii (Bohr) by atomic number
  int min_nat = 0, max_nat = 0;
  long long* d_steps = nullptr;
  // MD bookkeeping and exit rules on the device (qcx_batch_set_md_rules)
  MdState* d_md = nullptr;
  double* d_md_heat = nullptr;  // [nmol][3] eimp, fadd, nadd (qcx_batch_set_md_heating)
  double* d_velof = nullptr;    // [natom] velocity scaling weights of the heating
  SccCarry* d_carry = nullptr;  // [nmol] state of suspended SCCs (qcx_batch_set_scc_budget)
  long long* d_iter_sum = nullptr;  // [nmol] SCC iterations run
  // Size-bucketed stepping (qcx_batch_step_groups / _paced): one step graph per
  // molecule group, replayed on the group's own stream as often as the group's
  // step count asks; the group's atoms for its atom-level kernels.
  int* d_gatoms = nullptr;
  std::vector<int> g_atom_start, g_atom_count;
  std::vector<cudaGraph_t> gg_graph;
  std::vector<cudaGraphExec_t> gg_exec;
  double gg_tstep = 0.0;
  std::vector<int> gg_kernels;           // kernels in each group's step graph
  std::vector<cudaEvent_t> gg_end;       // per group: end of its steps in the last paced call
  cudaEvent_t gg_start = nullptr;
  std::vector<int> gg_n;                 // steps of each group in the last paced call
  std::vector<double> gg_ms_per_step;    // measured per-step time of each group (0: unknown)
  bool gg_pending_times = false;         // the last paced call's events are not read yet
  double* d_avxyz = nullptr;    // [natom][3] coordinate sums of the averaged structure
  bool md_heat = false;
  std::vector<double> h_eimp;   // eimp of every trajectory (qcx_batch_set_md_heating)
  // per-step electronic temperature (qcx_batch_set_md_etemp)
  bool md_etemp = false;
  double* d_etemp0 = nullptr;   // [nmol] the start's electronic temperature (K)
  bool md_on = false;
  // collision MD stop rules on the device (qcx_batch_set_cid_rules)
  CidState* d_cid = nullptr;
  double* d_cav = nullptr;  // [natom][9] the collision loop's averaged-structure sums
  bool cid_on = false;
  CidRules cid_rules{};
  MdRules md_rules{};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  double graph_tstep = 0.0;
  long long launches = 0;
  size_t bytes = 0;
  int precision = 0;
  int step_launches = 0;
  // Molecule groups: contiguous chunks of the size order (largest first).
  // After the batch-wide coordination numbers, each group runs its integral,
  // SCC and gradient kernels on its own stream, so that the group of the
  // largest molecules starts its SCC after its own integrals and the gradients
  // of groups that converge early overlap the SCC of the slowest molecules.
  int ngroup = 1;
  std::vector<int> g_start, g_count;      // range of each group in the size order
  std::vector<int> g_smem;                // SCC shared memory of each group (its largest molecule's)
  std::vector<int> g_max_nao;             // AOs of each group's largest molecule
  // grouped steps: the SCC budget scales with each group's largest molecule
  // (else with the batch's largest)
  bool budget_per_group = true;
  std::vector<int> g_pair_start;          // first pair of each group in d_gpairs
  std::vector<std::array<int, 10>> g_pair_off;  // class offsets inside the group
  ShellPair* d_gpairs = nullptr;          // shell pairs ordered by group, then class
  std::vector<cudaStream_t> g_stream;     // g_stream[0] is the batch stream
  std::vector<cudaEvent_t> g_join;
  cudaEvent_t g_fork = nullptr;
  // Timing marks recorded inside the captured step (qcx_batch_set_timing):
  // t_ev[0] at the start of the step, per group g four marks (integrals start,
  // SCC start, SCC end, gradient end) at t_ev[1 + 4 g + k], the end of the step last.
  bool timing = false;
  std::vector<cudaEvent_t> t_ev;
};

namespace {

// the batch restricted to molecule group g (SCC and gradient kernels)
DevBatch group_dev(const qcx_batch* b, int g) {
  DevBatch d = b->dev;
  d.nmol = b->g_count[g];
  d.order = b->dev.order + b->g_start[g];
  d.pairs = b->d_gpairs + b->g_pair_start[g];
  for (int c = 0; c < 10; ++c) d.pair_off[c] = b->g_pair_off[g][c];
  d.npair = d.pair_off[9];
  d.atom_list = b->d_gatoms + b->g_atom_start[g];
  d.natom_list = b->g_atom_count[g];
  // shared memory for the group's largest molecule only: groups of small
  // molecules leave room for more CTAs per SM
  d.smem_bytes = b->g_smem[g];
  // the per-step SCC budget of a group's step scales with the group's own
  // largest molecule (by default): every group's step is then bounded by about
  // the same number of iterations of its largest molecule, and an outlier among
  // small molecules (an SCC that needs several times the usual count) waits for
  // the next step instead of holding its group back. Measured on the
  // 256-trajectory workload (paced, budget 20): 5685 trajectory-steps/s against
  // 3512 with the batch's largest molecule as the scale; on the collision
  // workload (4096 ions of 18-281 AOs, groups of 512) the batch-wide scale was
  // faster (budget 10: 817 against 595), which the autotuner finds.
  if (b->budget_per_group) d.budget_nao = b->g_max_nao[g];
  return d;
}

// Records timing mark k into the step graph being captured (an event record
// node; a plain cudaEventRecord during capture only orders streams).
int mark(qcx_batch* b, bool marks, int k, cudaStream_t st) {
  if (!marks) return 0;
  return cudaEventRecordWithFlags(b->t_ev[k], st, cudaEventRecordExternal) == cudaSuccess ? 0 : -1;
}

// Enqueues one energy + gradient evaluation; returns the number of kernels
// launched, or -1 on an error in the stream bookkeeping. marks: record the
// per-group timing marks (only while capturing the step graph). budget: the
// SCCs may stop at the per-launch budget (the step graph); without it every
// SCC, a suspended one included, runs to its end (qcx_batch_egrad).
int enqueue_egrad(qcx_batch* b, bool marks = false, bool budget = false) {
  DevBatch d = b->dev;
  if (!budget) d.scc_budget = 0;
  int n = 0;
  launch_cn(d, b->stream);
  launch_zero_grad(d, b->stream);
  n += 2;
  if (b->ngroup == 1) {
    if (mark(b, marks, 1, b->stream)) return -1;
    n += launch_integrals(d, b->stream);
    if (mark(b, marks, 2, b->stream)) return -1;
    launch_scc(d, b->precision, b->stream);
    if (mark(b, marks, 3, b->stream)) return -1;
    n += 1 + launch_grad_pairs(d, b->stream);
    launch_grad_atoms(d, b->stream);
    if (mark(b, marks, 4, b->stream)) return -1;
    return n + 1;
  }
  if (cudaEventRecord(b->g_fork, b->stream) != cudaSuccess) return -1;
  for (int g = 0; g < b->ngroup; ++g) {
    cudaStream_t st = b->g_stream[g];
    if (g > 0 && cudaStreamWaitEvent(st, b->g_fork, 0) != cudaSuccess) return -1;
    DevBatch gd = group_dev(b, g);
    if (!budget) gd.scc_budget = 0;
    if (mark(b, marks, 1 + 4 * g, st)) return -1;
    n += launch_integrals(gd, st);  // the group's shell pairs only
    if (mark(b, marks, 2 + 4 * g, st)) return -1;
    launch_scc(gd, b->precision, st);
    if (mark(b, marks, 3 + 4 * g, st)) return -1;
    n += 1 + launch_grad_pairs(gd, st);
    launch_grad_atoms(gd, st);
    if (mark(b, marks, 4 + 4 * g, st)) return -1;
    ++n;
    if (g > 0) {
      if (cudaEventRecord(b->g_join[g], st) != cudaSuccess) return -1;
      if (cudaStreamWaitEvent(b->stream, b->g_join[g], 0) != cudaSuccess) return -1;
    }
  }
  return n;
}
constexpr int kEgradPhases = 6;

void free_batch(qcx_batch* b) {
  if (!b) return;
  if (b->graph_exec) cudaGraphExecDestroy(b->graph_exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  void* ptrs[] = {b->d_prm, b->d_mol, b->d_Z, b->d_atom_mol, b->d_sh_atom, b->d_sh_k, b->d_sh_ao, b->d_pairs,
                  b->d_xyz, b->d_grad, b->d_vel, b->d_mass, b->d_cn, b->d_cnd, b->d_dedcn, b->d_dedcnd,
                  b->d_mrad, b->d_dmrad, b->d_w4, b->d_dw4, b->d_qat, b->d_mats, b->d_vecs, b->d_energy,
                  b->d_ekin, b->d_status, b->d_iters, b->d_active, b->d_steps, b->d_order, b->d_have_prev,
                  b->d_frag, b->d_nfrag, b->d_frad};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (b->d_gpairs) cudaFree(b->d_gpairs);
  if (b->d_md) cudaFree(b->d_md);
  if (b->d_md_heat) cudaFree(b->d_md_heat);
  if (b->d_etemp0) cudaFree(b->d_etemp0);
  if (b->d_avxyz) cudaFree(b->d_avxyz);
  if (b->d_cid) cudaFree(b->d_cid);
  if (b->d_cav) cudaFree(b->d_cav);
  if (b->d_velof) cudaFree(b->d_velof);
  if (b->d_carry) cudaFree(b->d_carry);
  if (b->d_iter_sum) cudaFree(b->d_iter_sum);
  if (b->d_gatoms) cudaFree(b->d_gatoms);
  for (cudaGraphExec_t e : b->gg_exec)
    if (e) cudaGraphExecDestroy(e);
  for (cudaGraph_t g : b->gg_graph)
    if (g) cudaGraphDestroy(g);
  for (cudaEvent_t e : b->gg_end)
    if (e) cudaEventDestroy(e);
  if (b->gg_start) cudaEventDestroy(b->gg_start);
  for (size_t g = 1; g < b->g_stream.size(); ++g)
    if (b->g_stream[g]) cudaStreamDestroy(b->g_stream[g]);
  for (cudaEvent_t e : b->g_join)
    if (e) cudaEventDestroy(e);
  if (b->g_fork) cudaEventDestroy(b->g_fork);
  for (cudaEvent_t e : b->t_ev)
    if (e) cudaEventDestroy(e);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

// the step graph is captured again at the next qcx_batch_step
static void drop_graph(qcx_batch* b) {
  if (b->graph_exec) cudaGraphExecDestroy(b->graph_exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->graph_exec = nullptr;
  b->graph = nullptr;
  for (cudaGraphExec_t& e : b->gg_exec) {
    if (e) cudaGraphExecDestroy(e);
    e = nullptr;
  }
  for (cudaGraph_t& g : b->gg_graph) {
    if (g) cudaGraphDestroy(g);
    g = nullptr;
  }
}

int build_batch(qcx_batch* b, int nmol, const int32_t* nat, const int32_t* num, const double* charge,
                const double* etemp) {
  b->nmol = nmol;
  std::vector<int> atom_mol, sh_atom, sh_k, sh_ao;
  std::vector<ShellPair> pairs;
  long long mat_off = 0, vec_off = 0;
  int aoff = 0;
  for (int m = 0; m < nmol; ++m) {
    if (nat[m] < 1) {
      set_error("molecule with no atoms");
      return -1;
    }
    MolDesc md{};
    md.nat = nat[m];
    md.atom_off = aoff;
    md.sh_off = (int)sh_atom.size();
    int nao = 0;
    double nel = -charge[m];
    for (int a = 0; a < nat[m]; ++a) {
      int z = num[aoff + a];
      if (z < 1 || z > kMaxZ) {
        set_error("atomic number outside the parameterised range 1..18");
        return -1;
      }
      b->Z.push_back(z);
      atom_mol.push_back(m);
      for (int k = 0; k < qcx_nsh[z]; ++k) {
        sh_atom.push_back(aoff + a);
        sh_k.push_back(k);
        sh_ao.push_back(nao);
        nao += 2 * qcx_sh_l[z][k] + 1;
        nel += qcx_sh_refocc[z][k];
      }
    }
    md.nsh = (int)sh_atom.size() - md.sh_off;
    md.nao = nao;
    md.len = md.nsh + 9 * md.nat;
    md.nmem = QCX_BROYDEN_WINDOW;
    md.nel = nel;
    md.kT = etemp[m] * QCX_KTOAU;
    md.charge = charge[m];
    md.mat_off = mat_off;
    mat_off += (long long)kNumMat * slot_size(nao);
    md.vec_off = vec_off;
    vec_off += VecLayout::make(md.nat, md.nsh, nao, md.len, md.nmem).total;
    b->mol.push_back(md);
    b->max_nao = nao > b->max_nao ? nao : b->max_nao;
    aoff += nat[m];
  }
  b->natom = aoff;
  b->nshell = (int)sh_atom.size();
  // ordered shell pairs of every molecule, grouped by angular-momentum class
  int pair_off[10] = {0};
  {
    std::vector<int> sh_l(sh_atom.size());
    for (size_t s = 0; s < sh_atom.size(); ++s) sh_l[s] = qcx_sh_l[b->Z[sh_atom[s]]][sh_k[s]];
    for (int c = 0; c < 9; ++c) {
      pair_off[c] = (int)pairs.size();
      for (const MolDesc& md : b->mol)
        for (int s = md.sh_off; s < md.sh_off + md.nsh; ++s)
          for (int t = md.sh_off; t < md.sh_off + md.nsh; ++t)
            if (sh_l[s] * 3 + sh_l[t] == c) pairs.push_back({s, t});
    }
    pair_off[9] = (int)pairs.size();
  }
  b->npair = (int)pairs.size();
  CK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  std::unique_ptr<Params> hp(new Params);  // ~230 KB: not on the stack
  fill_params(*hp);
  int na = b->natom;
  if (dalloc(&b->d_prm, 1) || dalloc(&b->d_mol, nmol) || dalloc(&b->d_Z, na) || dalloc(&b->d_atom_mol, na) ||
      dalloc(&b->d_sh_atom, b->nshell) || dalloc(&b->d_sh_k, b->nshell) || dalloc(&b->d_sh_ao, b->nshell) ||
      dalloc(&b->d_pairs, b->npair) || dalloc(&b->d_xyz, 3 * na) || dalloc(&b->d_grad, 3 * na) ||
      dalloc(&b->d_vel, 3 * na) || dalloc(&b->d_mass, na) || dalloc(&b->d_cn, na) || dalloc(&b->d_cnd, na) ||
      dalloc(&b->d_dedcn, na) || dalloc(&b->d_dedcnd, na) || dalloc(&b->d_mrad, na) || dalloc(&b->d_dmrad, na) ||
      dalloc(&b->d_w4, (size_t)na * kMaxRef) || dalloc(&b->d_dw4, (size_t)na * kMaxRef) || dalloc(&b->d_qat, na) ||
      dalloc(&b->d_mats, (size_t)mat_off) || dalloc(&b->d_vecs, (size_t)vec_off) ||
      dalloc(&b->d_energy, (size_t)nmol * kNumEnergy) || dalloc(&b->d_ekin, nmol) || dalloc(&b->d_status, nmol) ||
      dalloc(&b->d_iters, nmol) || dalloc(&b->d_active, nmol) || dalloc(&b->d_steps, nmol) ||
      dalloc(&b->d_order, nmol) || dalloc(&b->d_have_prev, nmol) || dalloc(&b->d_frag, na) ||
      dalloc(&b->d_nfrag, nmol) || dalloc(&b->d_frad, kMaxZ + 1) || dalloc(&b->d_iter_sum, nmol))
    return -1;
  {
    // launch order of the per-molecule kernels: decreasing nao^3 (work of the SCC)
    std::vector<int> order(nmol);
    for (int m = 0; m < nmol; ++m) order[m] = m;
    std::stable_sort(order.begin(), order.end(), [b](int x, int y) { return b->mol[x].nao > b->mol[y].nao; });
    CK(cudaMemcpy(b->d_order, order.data(), sizeof(int) * nmol, cudaMemcpyHostToDevice));
    // molecule groups (contiguous in the size order) and their shell pairs,
    // ordered by group and then by angular-momentum class
    const int G = nmol < QCX_MOL_GROUPS ? nmol : QCX_MOL_GROUPS;
    b->ngroup = G;
    std::vector<int> sh_l(sh_atom.size());
    for (size_t sh = 0; sh < sh_atom.size(); ++sh) sh_l[sh] = qcx_sh_l[b->Z[sh_atom[sh]]][sh_k[sh]];
    std::vector<ShellPair> gp;
    gp.reserve(pairs.size());
    for (int g = 0; g < G; ++g) {
      const int k0 = (int)((long long)g * nmol / G), k1 = (int)((long long)(g + 1) * nmol / G);
      b->g_start.push_back(k0);
      b->g_count.push_back(k1 - k0);
      b->g_smem.push_back((int)scc_smem_bytes(b->mol[order[k0]].nao, 0));
      b->g_max_nao.push_back(b->mol[order[k0]].nao);
      b->g_pair_start.push_back((int)gp.size());
      std::array<int, 10> off{};
      for (int c = 0; c < 9; ++c) {
        off[c] = (int)gp.size() - b->g_pair_start[g];
        for (int k = k0; k < k1; ++k) {
          const MolDesc& md = b->mol[order[k]];
          for (int s = md.sh_off; s < md.sh_off + md.nsh; ++s)
            for (int t = md.sh_off; t < md.sh_off + md.nsh; ++t)
              if (sh_l[s] * 3 + sh_l[t] == c) gp.push_back({s, t});
        }
      }
      off[9] = (int)gp.size() - b->g_pair_start[g];
      b->g_pair_off.push_back(off);
    }
    // every group's atoms, for the atom-level kernels of its own step graph
    std::vector<int> gatoms;
    for (int g = 0; g < G; ++g) {
      b->g_atom_start.push_back((int)gatoms.size());
      for (int k = b->g_start[g]; k < b->g_start[g] + b->g_count[g]; ++k) {
        const MolDesc& md = b->mol[order[k]];
        for (int a = 0; a < md.nat; ++a) gatoms.push_back(md.atom_off + a);
      }
      b->g_atom_count.push_back((int)gatoms.size() - b->g_atom_start[g]);
    }
    if (dalloc(&b->d_gatoms, gatoms.size())) return -1;
    CK(cudaMemcpy(b->d_gatoms, gatoms.data(), sizeof(int) * gatoms.size(), cudaMemcpyHostToDevice));
    b->gg_graph.assign(G, nullptr);
    b->gg_exec.assign(G, nullptr);
    b->gg_end.assign(G, nullptr);
    b->gg_n.assign(G, 0);
    b->gg_kernels.assign(G, 0);
    b->gg_ms_per_step.assign(G, 0.0);
    for (int g = 0; g < G; ++g) CK(cudaEventCreate(&b->gg_end[g]));
    CK(cudaEventCreate(&b->gg_start));
    if (dalloc(&b->d_gpairs, gp.size())) return -1;
    CK(cudaMemcpy(b->d_gpairs, gp.data(), sizeof(ShellPair) * gp.size(), cudaMemcpyHostToDevice));
    b->g_stream.assign(G, nullptr);
    b->g_join.assign(G, nullptr);
    b->g_stream[0] = b->stream;
    for (int g = 1; g < G; ++g) {
      CK(cudaStreamCreateWithFlags(&b->g_stream[g], cudaStreamNonBlocking));
      CK(cudaEventCreateWithFlags(&b->g_join[g], cudaEventDisableTiming));
    }
    CK(cudaEventCreateWithFlags(&b->g_fork, cudaEventDisableTiming));
  }
  b->bytes = sizeof(double) * ((size_t)mat_off + (size_t)vec_off);
  CK(cudaMemcpy(b->d_prm, hp.get(), sizeof(Params), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b->d_mol, b->mol.data(), sizeof(MolDesc) * nmol, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b->d_Z, b->Z.data(), sizeof(int) * na, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b->d_atom_mol, atom_mol.data(), sizeof(int) * na, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b->d_sh_atom, sh_atom.data(), sizeof(int) * b->nshell, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b->d_sh_k, sh_k.data(), sizeof(int) * b->nshell, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b->d_sh_ao, sh_ao.data(), sizeof(int) * b->nshell, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b->d_pairs, pairs.data(), sizeof(ShellPair) * b->npair, cudaMemcpyHostToDevice));
  CK(cudaMemset(b->d_vel, 0, sizeof(double) * 3 * na));
  CK(cudaMemset(b->d_grad, 0, sizeof(double) * 3 * na));
  CK(cudaMemset(b->d_xyz, 0, sizeof(double) * 3 * na));
  CK(cudaMemset(b->d_status, 0, sizeof(int) * nmol));
  CK(cudaMemset(b->d_energy, 0, sizeof(double) * nmol * kNumEnergy));
  CK(cudaMemset(b->d_ekin, 0, sizeof(double) * nmol));
  CK(cudaMemset(b->d_steps, 0, sizeof(long long) * nmol));
  CK(cudaMemset(b->d_iter_sum, 0, sizeof(long long) * nmol));
  CK(cudaMemset(b->d_have_prev, 0, sizeof(int) * nmol));
  {
    // radii of the fragment test: src/covalent_radii.f90:89 (Rad, Angstrom) times
    // aatoau = 1/0.52917726 (src/xtb_mctc_convert.f90:24-25), elements 1-18
    static const double rad_aa[19] = {0.0,  0.32, 0.37, 1.30, 0.99, 0.84, 0.75, 0.71, 0.64, 0.60,
                                      0.62, 1.60, 1.40, 1.24, 1.14, 1.09, 1.04, 1.00, 1.01};
    static_assert(kMaxZ == 18, "fragment radii cover elements 1-18");
    const double aatoau = 1.0 / 0.52917726;
    double rad[kMaxZ + 1];
    for (int z = 0; z <= kMaxZ; ++z) rad[z] = aatoau * rad_aa[z];
    CK(cudaMemcpy(b->d_frad, rad, sizeof(rad), cudaMemcpyHostToDevice));
    b->min_nat = nat[0];
    b->max_nat = nat[0];
    for (int m = 1; m < nmol; ++m) {
      b->min_nat = nat[m] < b->min_nat ? nat[m] : b->min_nat;
      b->max_nat = nat[m] > b->max_nat ? nat[m] : b->max_nat;
    }
  }
  {
    std::vector<int> on(nmol, 1);
    CK(cudaMemcpy(b->d_active, on.data(), sizeof(int) * nmol, cudaMemcpyHostToDevice));
  }
  {
    std::vector<double> m(na, 1.0);
    CK(cudaMemcpy(b->d_mass, m.data(), sizeof(double) * na, cudaMemcpyHostToDevice));
  }
  DevBatch& d = b->dev;
  d.nmol = nmol;
  d.natom = na;
  d.nshell = b->nshell;
  d.npair = b->npair;
  for (int c = 0; c < 10; ++c) d.pair_off[c] = pair_off[c];
  d.prm = b->d_prm;
  d.mol = b->d_mol;
  d.Z = b->d_Z;
  d.atom_mol = b->d_atom_mol;
  d.xyz = b->d_xyz;
  d.grad = b->d_grad;
  d.vel = b->d_vel;
  d.mass = b->d_mass;
  d.cn = b->d_cn;
  d.cnd = b->d_cnd;
  d.dedcn = b->d_dedcn;
  d.dedcnd = b->d_dedcnd;
  d.mrad = b->d_mrad;
  d.dmrad = b->d_dmrad;
  d.w4 = b->d_w4;
  d.dw4 = b->d_dw4;
  d.qat = b->d_qat;
  d.sh_atom = b->d_sh_atom;
  d.sh_k = b->d_sh_k;
  d.sh_ao = b->d_sh_ao;
  d.pairs = b->d_pairs;
  d.mats = b->d_mats;
  d.vecs = b->d_vecs;
  d.energy = b->d_energy;
  d.status = b->d_status;
  d.iters = b->d_iters;
  d.ekin = b->d_ekin;
  d.active = b->d_active;
  d.steps_done = b->d_steps;
  d.iter_sum = b->d_iter_sum;
  d.atom_list = nullptr;
  d.natom_list = 0;
  d.have_prev = b->d_have_prev;
  d.guess = 0;
  d.checkqc = 1;
  d.order = b->d_order;
  d.max_nao = b->max_nao;
  d.smem_bytes = (int)scc_smem_bytes(b->max_nao, 0);
  d.max_iter = QCX_SCC_MAXITER;
  d.mixed_min_nao = 0;
  d.econv = QCX_SCC_ECONV;
  d.pconv = QCX_SCC_PCONV;
  d.mix_alpha = QCX_BROYDEN_ALPHA;
  return 0;
}

int check_launch() {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(std::string("kernel launch: ") + cudaGetErrorString(e));
    return -1;
  }
  return 0;
}

}  // namespace

namespace qcx {
// error text for qcx_last_error, set by the other translation units
void set_last_error(const std::string& s) { set_error(s); }
void set_last_error_text(const char* s) { set_error_text(s); }
void batch_set_mixed_min_nao(qcx_batch* b, int n) { b->dev.mixed_min_nao = n; }
void batch_set_checkqc(qcx_batch* b, int on) {
  if (b->dev.checkqc != on) drop_graph(b);
  b->dev.checkqc = on;
}
}  // namespace qcx

extern "C" {

int qcx_version(void) { return 100; }

const char* qcx_last_error(void) { return g_last_error; }

qcx_batch* qcx_batch_create(int nmol, const int32_t* nat, const int32_t* num, const double* charge,
                            const double* etemp) {
  if (nmol < 1 || !nat || !num || !charge || !etemp) {
    set_error("qcx_batch_create: invalid arguments");
    return nullptr;
  }
  qcx_batch* b = new qcx_batch();
  if (build_batch(b, nmol, nat, num, charge, etemp)) {
    free_batch(b);
    return nullptr;
  }
  return b;
}

void qcx_batch_destroy(qcx_batch* b) { free_batch(b); }

int qcx_batch_set_scc(qcx_batch* b, int max_iter, double econv, double pconv, double mixing) {
  if (!b || max_iter < 1 || max_iter > QCX_SCC_MAXITER || !(econv > 0) || !(pconv > 0) || !(mixing > 0)) {
    set_error("qcx_batch_set_scc: invalid arguments");
    return -1;
  }
  b->dev.max_iter = max_iter;
  b->dev.econv = econv;
  b->dev.pconv = pconv;
  b->dev.mix_alpha = mixing;
  // the step graphs hold the SCC settings as kernel arguments: the whole-batch
  // graph and the molecule groups' graphs are captured again
  drop_graph(b);
  return 0;
}

int qcx_batch_fragments(qcx_batch* b, double rcut, int at1, int at2, int32_t* frag, int32_t* nfrag) {
  if (!b || !(rcut > 0.0) || at1 < 0 || at2 < 0 || at1 > b->min_nat || at2 > b->min_nat ||
      (at1 == 0 && at2 != 0)) {
    set_error("qcx_batch_fragments: invalid arguments (rcut > 0, 0 <= at1, at2 <= atoms of the smallest molecule, "
              "at1 = 0 only with at2 = 0)");
    return -1;
  }
  launch_fragments(b->dev, b->max_nat, b->d_frad, rcut, at1, at2, b->d_frag, b->d_nfrag, b->stream);
  if (check_launch()) return -1;
  if (frag) CK(cudaMemcpyAsync(frag, b->d_frag, sizeof(int) * b->natom, cudaMemcpyDeviceToHost, b->stream));
  if (nfrag) CK(cudaMemcpyAsync(nfrag, b->d_nfrag, sizeof(int) * b->nmol, cudaMemcpyDeviceToHost, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  return 0;
}
int qcx_batch_set_md_rules(qcx_batch* b, int nfragexit, int more, int max_steps) {
  if (!b || nfragexit < 1 || more < 0 || max_steps < 1) {
    set_error("qcx_batch_set_md_rules: nfragexit >= 1, more >= 0, max_steps >= 1");
    return -1;
  }
  if (!b->d_md && dalloc(&b->d_md, b->nmol)) return -1;
  if (!b->d_avxyz && dalloc(&b->d_avxyz, 3 * (size_t)b->natom)) return -1;
  CK(cudaMemsetAsync(b->d_avxyz, 0, sizeof(double) * 3 * b->natom, b->stream));
  b->md_rules.nfragexit = nfragexit;
  b->md_rules.more = more;
  b->md_rules.max_steps = max_steps;
  b->md_rules.etemp_on = b->md_etemp ? 1 : 0;
  launch_md_begin(b->dev, b->d_md, b->md_heat ? b->d_md_heat : nullptr, b->d_avxyz,
                  b->md_etemp ? b->d_etemp0 : nullptr, b->stream);
  if (check_launch()) return -1;
  CK(cudaStreamSynchronize(b->stream));
  drop_graph(b);  // the rules are kernel arguments of the captured step graphs
  b->md_on = true;
  b->cid_on = false;
  return 0;
}

int qcx_batch_get_md_avg_xyz(qcx_batch* b, double* axyz) {
  if (!b || !b->d_md || !b->d_avxyz || !axyz) {
    set_error("qcx_batch_get_md_avg_xyz: no MD rules set up (qcx_batch_set_md_rules)");
    return -1;
  }
  std::vector<MdState> st(b->nmol);
  CK(cudaMemcpyAsync(st.data(), b->d_md, sizeof(MdState) * b->nmol, cudaMemcpyDeviceToHost, b->stream));
  CK(cudaMemcpyAsync(axyz, b->d_avxyz, sizeof(double) * 3 * b->natom, cudaMemcpyDeviceToHost, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  // axyz = avxyz / kdump (src/md.f90:695)
  for (int m = 0; m < b->nmol; ++m) {
    const MolDesc& md = b->mol[m];
    for (int k = 0; k < 3 * md.nat; ++k) axyz[3LL * md.atom_off + k] /= (double)st[m].kdump;
  }
  return 0;
}

int qcx_batch_set_cid_rules(qcx_batch* b, double tinit, int ntot) {
  if (!b || ntot < 1 || b->min_nat < 2) {
    set_error("qcx_batch_set_cid_rules: ntot >= 1 and molecules of the ion plus one gas atom");
    return -1;
  }
  if (!b->d_cid && dalloc(&b->d_cid, b->nmol)) return -1;
  if (!b->d_cav && dalloc(&b->d_cav, 9 * (size_t)b->natom)) return -1;
  b->cid_rules.tinit = tinit;
  b->cid_rules.ntot = ntot;
  launch_cid_begin(b->dev, b->d_cid, b->d_cav, b->cid_rules, b->stream);
  if (check_launch()) return -1;
  CK(cudaStreamSynchronize(b->stream));
  drop_graph(b);
  b->cid_on = true;
  b->md_on = false;
  return 0;
}

int qcx_batch_get_cid_avg_xyz(qcx_batch* b, double* axyz) {
  if (!b || !b->d_cid || !axyz) {
    set_error("qcx_batch_get_cid_avg_xyz: no collision rules set");
    return -1;
  }
  std::vector<CidState> st(b->nmol);
  std::vector<double> av(9 * (size_t)b->natom);
  CK(cudaMemcpyAsync(st.data(), b->d_cid, sizeof(CidState) * b->nmol, cudaMemcpyDeviceToHost, b->stream));
  CK(cudaMemcpyAsync(av.data(), b->d_cav, sizeof(double) * av.size(), cudaMemcpyDeviceToHost, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  // src/cid.f90:1095-1101: the fragments' average when the ion fell apart,
  // else the current window's sum over its steps
  for (int m = 0; m < b->nmol; ++m) {
    const MolDesc& md = b->mol[m];
    for (int i = 0; i < md.nat; ++i)
      for (int d = 0; d < 3; ++d) {
        const size_t a = (size_t)(md.atom_off + i);
        double v = 0.0;
        if (i < md.nat - 1)
          v = st[m].check_fragmented > 1 ? av[9 * a + 6 + d] : av[9 * a + d] / (double)st[m].xyzavg_dump;
        axyz[3 * a + d] = v;
      }
  }
  return 0;
}

int qcx_batch_get_cid_state(qcx_batch* b, int32_t* nstep, int32_t* nfrag, int32_t* collided, int32_t* fragmented,
                            int32_t* total_steps, int32_t* done, int32_t* failed, double* avg_temp,
                            double* ecom_ev) {
  if (!b || !b->d_cid) {
    set_error("qcx_batch_get_cid_state: no collision rules set up (qcx_batch_set_cid_rules)");
    return -1;
  }
  std::vector<CidState> st(b->nmol);
  CK(cudaMemcpyAsync(st.data(), b->d_cid, sizeof(CidState) * b->nmol, cudaMemcpyDeviceToHost, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  for (int m = 0; m < b->nmol; ++m) {
    if (nstep) nstep[m] = st[m].nstep;
    if (nfrag) nfrag[m] = st[m].nfrag;
    if (collided) collided[m] = st[m].collided;
    if (fragmented) fragmented[m] = st[m].fragmented;
    if (total_steps) total_steps[m] = st[m].total_steps;
    if (done) done[m] = st[m].done;
    if (failed) failed[m] = st[m].failed;
    if (avg_temp) avg_temp[m] = st[m].avgT;
    if (ecom_ev) ecom_ev[m] = st[m].ecom;
  }
  return 0;
}

int qcx_batch_set_md_heating(qcx_batch* b, const double* eimp, const double* tadd, const double* velof,
                             double tstep) {
  if (!b || !eimp || !tadd || !(tstep > 0.0)) {
    set_error("qcx_batch_set_md_heating: eimp[nmol], tadd[nmol] and tstep > 0 are required");
    return -1;
  }
  std::vector<double> h(3 * (size_t)b->nmol);
  for (int m = 0; m < b->nmol; ++m) {
    if (!(eimp[m] >= 0.0) || !(tadd[m] >= 0.0) || !(tadd[m] / tstep < 1.0e9)) {
      set_error("qcx_batch_set_md_heating: eimp and tadd must be >= 0 and tadd below 1e9 steps");
      return -1;
    }
    // src/md.f90:265-266: nadd = (tadd + tstep) / tstep - 1 (truncated), fadd = tstep / (tadd + tstep)
    h[3 * m] = eimp[m];
    h[3 * m + 1] = tstep / (tadd[m] + tstep);
    h[3 * m + 2] = (double)(int)((tadd[m] + tstep) / tstep - 1.0);
  }
  std::vector<double> vf(b->natom, 1.0);
  if (velof)
    for (int a = 0; a < b->natom; ++a) vf[a] = velof[a];
  if (!b->d_md_heat && dalloc(&b->d_md_heat, 3 * (size_t)b->nmol)) return -1;
  if (!b->d_velof && dalloc(&b->d_velof, (size_t)b->natom)) return -1;
  CK(cudaMemcpy(b->d_md_heat, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b->d_velof, vf.data(), sizeof(double) * vf.size(), cudaMemcpyHostToDevice));
  if (!b->md_heat) drop_graph(b);  // the graphs pass the heating factors only when it is on
  b->md_heat = true;
  b->h_eimp.assign(eimp, eimp + b->nmol);
  return 0;
}

int qcx_batch_set_md_etemp(qcx_batch* b, double ax, double ieetemp) {
  if (!b || !std::isfinite(ax) || !std::isfinite(ieetemp)) {
    set_error("qcx_batch_set_md_etemp: invalid arguments");
    return -1;
  }
  // the start (src/md.f90:167-168): setetemp(nfrag = 1, eimp, etemp)
  std::vector<double> et(b->nmol);
  std::vector<MolDesc> md = b->mol;
  for (int m = 0; m < b->nmol; ++m) {
    const double eimp = b->md_heat ? b->h_eimp[m] : 0.0;
    et[m] = setetemp(1, eimp, ax, ieetemp);
    md[m].kT = et[m] * QCX_KTOAU;
  }
  if (!b->d_etemp0 && dalloc(&b->d_etemp0, (size_t)b->nmol)) return -1;
  CK(cudaMemcpyAsync(b->d_etemp0, et.data(), sizeof(double) * b->nmol, cudaMemcpyHostToDevice, b->stream));
  CK(cudaMemcpyAsync(b->d_mol, md.data(), sizeof(MolDesc) * b->nmol, cudaMemcpyHostToDevice, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  b->md_rules.ax = ax;
  b->md_rules.ieetemp = ieetemp;
  b->md_etemp = true;
  drop_graph(b);
  return 0;
}

int qcx_batch_get_md_etemp(qcx_batch* b, double* etemp) {
  if (!b || !b->d_md || !etemp) {
    set_error("qcx_batch_get_md_etemp: no MD rules set up (qcx_batch_set_md_rules)");
    return -1;
  }
  std::vector<MdState> st(b->nmol);
  CK(cudaMemcpyAsync(st.data(), b->d_md, sizeof(MdState) * b->nmol, cudaMemcpyDeviceToHost, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  for (int m = 0; m < b->nmol; ++m) etemp[m] = st[m].etemp;
  return 0;
}

int qcx_batch_get_md_state(qcx_batch* b, int32_t* nstep, int32_t* nfrag, int32_t* fragstate, int32_t* mdok,
                           int32_t* done, double* tav, double* eerror, double* fragT) {
  if (!b || !b->d_md) {
    set_error("qcx_batch_get_md_state: no MD rules set up (qcx_batch_set_md_rules)");
    return -1;
  }
  std::vector<MdState> st(b->nmol);
  CK(cudaMemcpyAsync(st.data(), b->d_md, sizeof(MdState) * b->nmol, cudaMemcpyDeviceToHost, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  for (int m = 0; m < b->nmol; ++m) {
    if (nstep) nstep[m] = st[m].nstep;
    if (nfrag) nfrag[m] = st[m].nfrag;
    if (fragstate) fragstate[m] = st[m].fragstate;
    if (mdok) mdok[m] = st[m].mdok;
    if (done) done[m] = st[m].done;
    if (tav) tav[m] = st[m].tav;
    if (eerror) eerror[m] = st[m].eerror;
    if (fragT)
      for (int j = 0; j < 10; ++j) fragT[10 * m + j] = st[m].fragT[j];
  }
  return 0;
}

int qcx_batch_set_guess(qcx_batch* b, int guess) {
  if (!b || (guess != QCX_GUESS_ZERO && guess != QCX_GUESS_PREVIOUS)) {
    set_error("qcx_batch_set_guess: guess must be 0 (zero moments) or 1 (previous converged moments)");
    return -1;
  }
  if (guess != b->dev.guess) drop_graph(b);
  b->dev.guess = guess;
  return 0;
}
int qcx_batch_set_precision(qcx_batch* b, int precision) {
  if (!b || (precision != 0 && precision != 1)) {
    set_error("qcx_batch_set_precision: precision must be 0 (FP64) or 1 (mixed)");
    return -1;
  }
  if (precision != b->precision) drop_graph(b);
  b->precision = precision;
  return 0;
}

int qcx_batch_set_state(qcx_batch* b, const double* xyz, const double* vel, const double* mass) {
  if (!b) return -1;
  size_t n3 = sizeof(double) * 3 * b->natom;
  if (xyz) {
    if (b->md_on || b->cid_on || b->md_etemp) {
      // new coordinates start new runs: the MD or collision rules must be set up
      // again, and the electronic temperatures return to the batch's
      b->md_on = false;
      b->cid_on = false;
      if (b->md_etemp)
        CK(cudaMemcpyAsync(b->d_mol, b->mol.data(), sizeof(MolDesc) * b->nmol, cudaMemcpyHostToDevice, b->stream));
      b->md_etemp = false;
      drop_graph(b);
    }
    CK(cudaMemcpyAsync(b->d_xyz, xyz, n3, cudaMemcpyHostToDevice, b->stream));
    // new coordinates start every trajectory afresh (and end suspended SCCs)
    CK(cudaMemsetAsync(b->d_status, 0, sizeof(int) * b->nmol, b->stream));
    std::vector<int> on(b->nmol, 1);
    CK(cudaMemcpyAsync(b->d_active, on.data(), sizeof(int) * b->nmol, cudaMemcpyHostToDevice, b->stream));
    CK(cudaStreamSynchronize(b->stream));
  }
  if (vel) CK(cudaMemcpyAsync(b->d_vel, vel, n3, cudaMemcpyHostToDevice, b->stream));
  if (mass) CK(cudaMemcpyAsync(b->d_mass, mass, sizeof(double) * b->natom, cudaMemcpyHostToDevice, b->stream));
  return 0;
}

int qcx_batch_load_state(qcx_batch* b, const double* xyz, const double* vel) {
  if (!b) return -1;
  const size_t n3 = sizeof(double) * 3 * b->natom;
  if (xyz) CK(cudaMemcpyAsync(b->d_xyz, xyz, n3, cudaMemcpyHostToDevice, b->stream));
  if (vel) CK(cudaMemcpyAsync(b->d_vel, vel, n3, cudaMemcpyHostToDevice, b->stream));
  return 0;
}

int qcx_batch_egrad(qcx_batch* b) {
  if (!b) return -1;
  int n = enqueue_egrad(b);
  if (n < 0) {
    set_error("qcx_batch_egrad: stream synchronisation failed");
    return -1;
  }
  b->launches = n;
  return check_launch();
}

int qcx_batch_step(qcx_batch* b, int nsteps, double tstep) {
  if (!b || nsteps < 0) return -1;
  if (!b->graph_exec || b->graph_tstep != tstep) {
    if (b->graph_exec) {
      cudaGraphExecDestroy(b->graph_exec);
      cudaGraphDestroy(b->graph);
      b->graph_exec = nullptr;
      b->graph = nullptr;
    }
    CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    const bool marks = b->timing;
    int n = mark(b, marks, 0, b->stream);
    launch_leapfrog(b->dev, tstep, b->stream);
    if (n >= 0) n = enqueue_egrad(b, marks, true);
    if (n >= 0 && b->md_on) {
      // fragment_structure(nuc, iat, xyz, 3.0, 1, 0, list) of src/md.f90:450, then the rules
      launch_fragments(b->dev, b->max_nat, b->d_frad, 3.0, 1, 0, b->d_frag, b->d_nfrag, b->stream);
      MdRules r = b->md_rules;
      r.tstep = tstep;
      r.max_nat = b->max_nat;
      launch_md_rules(b->dev, b->d_md, b->d_frag, b->d_nfrag, b->md_heat ? b->d_velof : nullptr, b->d_avxyz, r,
                      b->stream);
      n += 2;
    }
    if (n >= 0 && b->cid_on) {
      // fragment_structure over the ion's atoms (src/cid.f90:800), then the stop rules
      launch_fragments(b->dev, b->max_nat, b->d_frad, 3.0, 1, 0, b->d_frag, b->d_nfrag, b->stream, 1);
      CidRules r = b->cid_rules;
      r.tstep = tstep;
      launch_cid_rules(b->dev, b->d_cid, b->d_frag, b->d_nfrag, b->d_cav, r, b->stream);
      n += 2;
    }
    if (n >= 0 && mark(b, marks, 1 + 4 * b->ngroup, b->stream)) n = -1;
    cudaError_t ce = cudaStreamEndCapture(b->stream, &b->graph);
    if (n < 0 || ce != cudaSuccess) {
      if (ce == cudaSuccess && b->graph) cudaGraphDestroy(b->graph);
      b->graph = nullptr;
      set_error(std::string("qcx_batch_step: graph capture failed: ") + cudaGetErrorString(ce));
      return -1;
    }
    b->step_launches = 1 + n;
    CK(cudaGraphInstantiate(&b->graph_exec, b->graph, 0));
    b->graph_tstep = tstep;
  }
  for (int s = 0; s < nsteps; ++s) CK(cudaGraphLaunch(b->graph_exec, b->stream));
  b->launches = (long long)nsteps * b->step_launches;
  return check_launch();
}

}  // extern "C"

namespace {
// Captures the step graph of molecule group g on the group's stream: leapfrog,
// coordination numbers, integrals, SCC and gradient of the group's molecules,
// then the device loop rules when they are on. Returns its kernel count or -1.
int capture_group(qcx_batch* b, int g, double tstep) {
  cudaStream_t st = b->g_stream[g];
  const DevBatch gd = group_dev(b, g);
  CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  int n = 3;
  launch_leapfrog(gd, tstep, st);
  launch_cn(gd, st);
  launch_zero_grad(gd, st);
  n += launch_integrals(gd, st);
  launch_scc(gd, b->precision, st);
  n += 2 + launch_grad_pairs(gd, st);
  launch_grad_atoms(gd, st);
  if (b->md_on) {
    launch_fragments(gd, b->max_nat, b->d_frad, 3.0, 1, 0, b->d_frag, b->d_nfrag, st);
    MdRules r = b->md_rules;
    r.tstep = tstep;
    r.max_nat = b->max_nat;
    launch_md_rules(gd, b->d_md, b->d_frag, b->d_nfrag, b->md_heat ? b->d_velof : nullptr, b->d_avxyz, r, st);
    n += 2;
  }
  if (b->cid_on) {
    launch_fragments(gd, b->max_nat, b->d_frad, 3.0, 1, 0, b->d_frag, b->d_nfrag, st, 1);
    CidRules r = b->cid_rules;
    r.tstep = tstep;
    launch_cid_rules(gd, b->d_cid, b->d_frag, b->d_nfrag, b->d_cav, r, st);
    n += 2;
  }
  cudaGraph_t graph = nullptr;
  cudaError_t ce = cudaStreamEndCapture(st, &graph);
  if (ce != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    set_error(std::string("group step graph capture failed: ") + cudaGetErrorString(ce));
    return -1;
  }
  b->gg_graph[g] = graph;
  CK(cudaGraphInstantiate(&b->gg_exec[g], graph, 0));
  return n;
}
}  // namespace

extern "C" {

int qcx_batch_step_groups(qcx_batch* b, const int32_t* nsteps, double tstep) {
  if (!b || !nsteps) {
    set_error("qcx_batch_step_groups: invalid arguments");
    return -1;
  }
  const int G = b->ngroup;
  for (int g = 0; g < G; ++g)
    if (nsteps[g] < 0) {
      set_error("qcx_batch_step_groups: negative step count");
      return -1;
    }
  if (b->gg_tstep != tstep || !b->gg_exec[0]) {
    for (int g = 0; g < G; ++g) {
      if (b->gg_exec[g]) cudaGraphExecDestroy(b->gg_exec[g]);
      if (b->gg_graph[g]) cudaGraphDestroy(b->gg_graph[g]);
      b->gg_exec[g] = nullptr;
      b->gg_graph[g] = nullptr;
    }
    for (int g = 0; g < G; ++g) {
      const int n = capture_group(b, g, tstep);
      if (n < 0) {
        drop_graph(b);  // no partial set of group graphs survives a failed capture
        return -1;
      }
      b->gg_kernels[g] = n;
    }
    b->gg_tstep = tstep;
  }
  // every group starts after the work queued so far on the batch stream and
  // the batch stream continues after every group's last step
  CK(cudaEventRecord(b->gg_start, b->stream));
  long long launches = 0;
  for (int g = 0; g < G; ++g) {
    cudaStream_t st = b->g_stream[g];
    if (g > 0) CK(cudaStreamWaitEvent(st, b->gg_start, 0));
    for (int s = 0; s < nsteps[g]; ++s) CK(cudaGraphLaunch(b->gg_exec[g], st));
    CK(cudaEventRecord(b->gg_end[g], st));
    b->gg_n[g] = nsteps[g];
    launches += (long long)nsteps[g] * b->gg_kernels[g];
  }
  for (int g = 1; g < G; ++g) CK(cudaStreamWaitEvent(b->stream, b->gg_end[g], 0));
  b->gg_pending_times = true;
  b->launches = launches;
  return check_launch();
}

int qcx_batch_step_paced(qcx_batch* b, int nsteps, double tstep) {
  if (!b || nsteps < 0) {
    set_error("qcx_batch_step_paced: invalid arguments");
    return -1;
  }
  const int G = b->ngroup;
  // per-step time of every group from the previous call (when its work is done)
  if (b->gg_pending_times) {
    bool done = true;
    for (int g = 0; g < G; ++g) done = done && cudaEventQuery(b->gg_end[g]) == cudaSuccess;
    if (done) {
      for (int g = 0; g < G; ++g) {
        float ms = 0.f;
        if (b->gg_n[g] > 0 && cudaEventElapsedTime(&ms, b->gg_start, b->gg_end[g]) == cudaSuccess) {
          const double per = ms / b->gg_n[g];
          double& t = b->gg_ms_per_step[g];
          t = t > 0.0 ? 0.5 * (t + per) : per;
        }
      }
      b->gg_pending_times = false;
    }
    cudaGetLastError();  // a query of unfinished work is not an error
  }
  // group 0 (the largest molecules) takes nsteps steps; every other group as
  // many as fit into the same time, at least one and at most 16 per step of
  // group 0 (a group whose trajectories have mostly stopped steps in almost
  // no time and would otherwise take hundreds of steps per call)
  std::vector<int32_t> n(G, nsteps);
  const double T = b->gg_ms_per_step[0] * nsteps;
  for (int g = 1; g < G; ++g) {
    const double t = b->gg_ms_per_step[g];
    if (nsteps > 0 && T > 0.0 && t > 0.0) {
      const double k = std::floor(T / t);
      n[g] = (int32_t)std::max(1.0, std::min(k, 16.0 * nsteps));
    }
  }
  return qcx_batch_step_groups(b, n.data(), tstep);
}

int qcx_batch_autotune_budget(qcx_batch* b, double tstep, const int32_t* cand, int ncand, int calls,
                              double* rates) {
  return qcx_batch_autotune_paced(b, tstep, 1, cand, ncand, calls, rates);
}

int qcx_batch_autotune_paced(qcx_batch* b, double tstep, int steps_per_call, const int32_t* cand, int ncand,
                             int calls, double* rates) {
  if (!b || !cand || ncand < 1 || calls < 1 || steps_per_call < 1) {
    set_error("qcx_batch_autotune_paced: invalid arguments");
    return -1;
  }
  for (int c = 0; c < ncand; ++c)
    if (cand[c] < 0) {
      set_error("qcx_batch_autotune_paced: negative budget");
      return -1;
    }
  // Completed trajectory-steps per second of paced steps under every candidate
  // budget and both budget scales (each group's largest molecule, the batch's
  // largest), measured on the batch's own trajectories (the steps are real MD
  // steps: every candidate continues the run where the previous one left it).
  // One untimed call per candidate lets the pacing settle to it. The batch
  // ages over the calls (trajectories fragment and stop, small molecules run
  // ahead), so the configurations are measured twice, the second pass in
  // reverse order, and each rate is taken over both of its measurements.
  CallEvents ev(2);
  CK(ev.create());
  const cudaEvent_t e0 = ev[0], e1 = ev[1];
  std::vector<long long> s0(b->nmol), s1(b->nmol);
  const int ncfg = 2 * ncand;
  std::vector<double> done_sum(ncfg, 0.0), ms_sum(ncfg, 0.0);
  int rc = 0;
  for (int q = 0; q < 2 * ncfg && rc == 0; ++q) {
    const int c = q < ncfg ? q : 2 * ncfg - 1 - q;
    rc = qcx_batch_set_scc_budget(b, cand[c % ncand]);
    if (!rc) rc = qcx_batch_set_scc_budget_scale(b, c < ncand ? 1 : 0);
    if (!rc) rc = qcx_batch_step_paced(b, steps_per_call, tstep);
    if (!rc && cudaMemcpyAsync(s0.data(), b->d_steps, sizeof(long long) * b->nmol, cudaMemcpyDeviceToHost,
                               b->stream) != cudaSuccess) rc = -1;
    if (!rc && cudaEventRecord(e0, b->stream) != cudaSuccess) rc = -1;
    for (int k = 0; k < calls && !rc; ++k) rc = qcx_batch_step_paced(b, steps_per_call, tstep);
    if (!rc && cudaEventRecord(e1, b->stream) != cudaSuccess) rc = -1;
    if (!rc && cudaMemcpyAsync(s1.data(), b->d_steps, sizeof(long long) * b->nmol, cudaMemcpyDeviceToHost,
                               b->stream) != cudaSuccess) rc = -1;
    if (!rc && cudaStreamSynchronize(b->stream) != cudaSuccess) rc = -1;
    float ms = 0.f;
    if (!rc && cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) rc = -1;
    if (rc) break;
    long long done = 0;
    for (int m = 0; m < b->nmol; ++m) done += s1[m] - s0[m];
    done_sum[c] += (double)done;
    ms_sum[c] += (double)ms;
  }
  int best = 0;
  double best_rate = -1.0;
  for (int c = 0; c < ncfg && rc == 0; ++c) {
    const double rate = ms_sum[c] > 0.0 ? 1e3 * done_sum[c] / ms_sum[c] : 0.0;
    if (rates) rates[c] = rate;
    if (rate > best_rate) {
      best_rate = rate;
      best = c;
    }
  }
  if (rc) {
    set_error("qcx_batch_autotune_paced: a timed step failed");
    return -1;
  }
  if (qcx_batch_set_scc_budget(b, cand[best % ncand]) || qcx_batch_set_scc_budget_scale(b, best < ncand ? 1 : 0))
    return -1;
  return cand[best % ncand];
}

int qcx_batch_group_info(qcx_batch* b, int32_t* group_of_mol, int32_t* nsteps_last, double* ms_per_step) {
  if (!b) return -1;
  std::vector<int> order(b->nmol);
  CK(cudaMemcpy(order.data(), b->d_order, sizeof(int) * b->nmol, cudaMemcpyDeviceToHost));
  for (int g = 0; g < b->ngroup; ++g) {
    for (int k = b->g_start[g]; k < b->g_start[g] + b->g_count[g]; ++k)
      if (group_of_mol) group_of_mol[order[k]] = g;
    if (nsteps_last) nsteps_last[g] = b->gg_n[g];
    if (ms_per_step) ms_per_step[g] = b->gg_ms_per_step[g];
  }
  return b->ngroup;
}

int qcx_batch_get_iterations(qcx_batch* b, int64_t* iter_sum) {
  if (!b || !iter_sum) return -1;
  CK(cudaMemcpyAsync(iter_sum, b->d_iter_sum, sizeof(long long) * b->nmol, cudaMemcpyDeviceToHost, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  return 0;
}

int qcx_batch_get(qcx_batch* b, double* xyz, double* vel, double* grad, double* energy, double* qat, double* ekin,
                  int32_t* status, int32_t* iters) {
  if (!b) return -1;
  size_t n3 = sizeof(double) * 3 * b->natom;
  if (xyz) CK(cudaMemcpyAsync(xyz, b->d_xyz, n3, cudaMemcpyDeviceToHost, b->stream));
  if (vel) CK(cudaMemcpyAsync(vel, b->d_vel, n3, cudaMemcpyDeviceToHost, b->stream));
  if (grad) CK(cudaMemcpyAsync(grad, b->d_grad, n3, cudaMemcpyDeviceToHost, b->stream));
  if (qat) CK(cudaMemcpyAsync(qat, b->d_qat, sizeof(double) * b->natom, cudaMemcpyDeviceToHost, b->stream));
  if (ekin) CK(cudaMemcpyAsync(ekin, b->d_ekin, sizeof(double) * b->nmol, cudaMemcpyDeviceToHost, b->stream));
  if (status) CK(cudaMemcpyAsync(status, b->d_status, sizeof(int) * b->nmol, cudaMemcpyDeviceToHost, b->stream));
  if (iters) CK(cudaMemcpyAsync(iters, b->d_iters, sizeof(int) * b->nmol, cudaMemcpyDeviceToHost, b->stream));
  if (energy) {
    std::vector<double> e((size_t)b->nmol * kNumEnergy);
    CK(cudaMemcpyAsync(e.data(), b->d_energy, sizeof(double) * e.size(), cudaMemcpyDeviceToHost, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    for (int m = 0; m < b->nmol; ++m) energy[m] = e[(size_t)m * kNumEnergy + kETotal];
  }
  CK(cudaStreamSynchronize(b->stream));
  return 0;
}

int qcx_batch_get_energy_terms(qcx_batch* b, int i, double* terms) {
  if (!b || i < 0 || i >= b->nmol || !terms) return -1;
  CK(cudaMemcpyAsync(terms, b->d_energy + (size_t)i * kNumEnergy, sizeof(double) * kNumEnergy,
                     cudaMemcpyDeviceToHost, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  return 0;
}

int qcx_batch_get_matrix(qcx_batch* b, int i, int which, double* out) {
  if (!b || i < 0 || i >= b->nmol || which < 0 || which >= kNumMat || !out) return -1;
  const MolDesc& md = b->mol[i];
  const double* src = b->d_mats + md.mat_off + (long long)which * slot_size(md.nao);
  CK(cudaMemcpyAsync(out, src, sizeof(double) * md.nao * md.nao, cudaMemcpyDeviceToHost, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  return md.nao;
}

long long qcx_batch_kernel_launches(qcx_batch* b) { return b ? b->launches : -1; }

int qcx_batch_get_progress(qcx_batch* b, int32_t* active, int64_t* steps_done) {
  if (!b) return -1;
  if (active) CK(cudaMemcpyAsync(active, b->d_active, sizeof(int) * b->nmol, cudaMemcpyDeviceToHost, b->stream));
  if (steps_done)
    CK(cudaMemcpyAsync(steps_done, b->d_steps, sizeof(long long) * b->nmol, cudaMemcpyDeviceToHost, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  return 0;
}

int qcx_batch_sync(qcx_batch* b) {
  if (!b) return -1;
  CK(cudaStreamSynchronize(b->stream));
  return 0;
}

void* qcx_batch_stream(qcx_batch* b) { return b ? (void*)b->stream : nullptr; }

int qcx_batch_profile_egrad(qcx_batch* b, float* ms) {
  if (!b || !ms) return -1;
  CallEvents ev(kEgradPhases + 1);
  CK(ev.create());
  const DevBatch& d = b->dev;
  CK(cudaEventRecord(ev[0], b->stream));
  launch_cn(d, b->stream);
  CK(cudaEventRecord(ev[1], b->stream));
  int nl = 3 + launch_integrals(d, b->stream);
  CK(cudaEventRecord(ev[2], b->stream));
  launch_scc(d, b->precision, b->stream);
  CK(cudaEventRecord(ev[3], b->stream));
  launch_zero_grad(d, b->stream);
  CK(cudaEventRecord(ev[4], b->stream));
  nl += launch_grad_pairs(d, b->stream);
  CK(cudaEventRecord(ev[5], b->stream));
  launch_grad_atoms(d, b->stream);
  CK(cudaEventRecord(ev[6], b->stream));
  CK(cudaEventSynchronize(ev[6]));
  for (int i = 0; i < kEgradPhases; ++i) CK(cudaEventElapsedTime(&ms[i], ev[i], ev[i + 1]));
  b->launches = nl;
  return check_launch();
}

int qcx_batch_set_timing(qcx_batch* b, int on) {
  if (!b || (on != 0 && on != 1)) {
    set_error("qcx_batch_set_timing: on must be 0 or 1");
    return -1;
  }
  if (on && b->t_ev.empty()) {
    CallEvents ev(2 + 4 * (size_t)b->ngroup);
    CK(ev.create());
    b->t_ev.swap(ev.ev);  // the batch owns them from here (destroyed with it)
  }
  if ((on != 0) != b->timing) drop_graph(b);
  b->timing = on != 0;
  return 0;
}

int qcx_batch_get_timing(qcx_batch* b, float* ms, int n) {
  if (!b || !ms || !b->timing || n < 2 + 4 * b->ngroup) {
    set_error("qcx_batch_get_timing: timing marks are off (qcx_batch_set_timing) or the output is too small");
    return -1;
  }
  const int m = 2 + 4 * b->ngroup;
  CK(cudaEventSynchronize(b->t_ev[m - 1]));
  ms[0] = 0.0f;
  for (int k = 1; k < m; ++k) CK(cudaEventElapsedTime(&ms[k], b->t_ev[0], b->t_ev[k]));
  return b->ngroup;
}

int qcx_batch_get_sizes(qcx_batch* b, int32_t* nao, int32_t* nat) {
  if (!b) return -1;
  for (int m = 0; m < b->nmol; ++m) {
    if (nao) nao[m] = b->mol[m].nao;
    if (nat) nat[m] = b->mol[m].nat;
  }
  return 0;
}

int qcx_checkqc(int nat, const double* grad, const double* qat, int charge, double* energy) {
  if (nat < 1 || !grad || !qat || !energy) {
    set_error("qcx_checkqc: invalid arguments");
    return -1;
  }
  double* d = nullptr;
  const size_t nd = 4 * (size_t)nat + 1;
  CK(cudaMalloc((void**)&d, sizeof(double) * nd + sizeof(int)));
  int* dcode = (int*)(d + nd);
  int code = -1;
  cudaError_t e = cudaMemcpy(d, grad, sizeof(double) * 3 * nat, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d + 3 * nat, qat, sizeof(double) * nat, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d + 4 * nat, energy, sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    launch_checkqc(nat, d, d + 3 * nat, (double)charge, d + 4 * nat, dcode, 0);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(energy, d + 4 * nat, sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&code, dcode, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) {
    set_error(std::string("qcx_checkqc: ") + cudaGetErrorString(e));
    return -1;
  }
  return code;
}

// ---------------------------------------------------------------------------
// single-structure drop-in with a per-process cache of the device state
// ---------------------------------------------------------------------------
int qcx_egrad(int method, int nat, const int32_t* num, const double* xyz, int charge, int multiplicity,
              double etemp, double* energy, double* grad, double* qat) {
  // one cached device state per GPU (the calling thread's current device)
  struct Cache {
    qcx_batch* b = nullptr;
    std::vector<int> num;
    double charge = 0.0, etemp = -1.0;
  };
  constexpr int kMaxDevices = 64;
  static std::mutex mtx;
  static Cache caches[kMaxDevices];
  (void)multiplicity;
  if (method != QCX_METHOD_GFN2) {
    set_error("only the GFN2-xTB Hamiltonian is implemented");
    return 5;
  }
  if (nat < 1 || !num || !xyz || !energy || !grad || !qat) {
    set_error("qcx_egrad: invalid arguments");
    return -1;
  }
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("qcx_egrad: device index out of range");
    return -1;
  }
  std::lock_guard<std::mutex> lock(mtx);
  Cache& c = caches[dev];
  std::vector<int> key(num, num + nat);
  if (!c.b || key != c.num || c.charge != (double)charge || c.etemp != etemp) {
    if (c.b) free_batch(c.b);
    int32_t n1 = nat;
    double ch = charge, et = etemp;
    c.b = qcx_batch_create(1, &n1, num, &ch, &et);
    if (!c.b) return -1;
    c.num = key;
    c.charge = charge;
    c.etemp = etemp;
  }
  qcx_batch* cached = c.b;
  if (qcx_batch_set_state(cached, xyz, nullptr, nullptr)) return -1;
  if (qcx_batch_egrad(cached)) return -1;
  int32_t st = 0;
  if (qcx_batch_get(cached, nullptr, nullptr, grad, energy, qat, nullptr, &st, nullptr)) return -1;
  if (st != 0) {
    char buf[128];
    if (st == QCX_STATUS_CHECKQC)
      std::snprintf(buf, sizeof(buf), "result rejected by checkqc (energy, gradient norm or charges out of range)");
    else
      std::snprintf(buf, sizeof(buf), "calculation failed, status bits 0x%x", st);
    set_error(buf);
    return -1;
  }
  return 0;
}

int qcx_batch_set_scc_budget(qcx_batch* b, int iters) {
  if (!b || iters < 0) {
    set_error("qcx_batch_set_scc_budget: iters must be >= 0");
    return -1;
  }
  if (iters > 0 && !b->d_carry) {
    CK(cudaMalloc((void**)&b->d_carry, sizeof(SccCarry) * b->nmol));
    CK(cudaMemset(b->d_carry, 0, sizeof(SccCarry) * b->nmol));
    b->dev.carry = b->d_carry;
  }
  if (iters != b->dev.scc_budget) drop_graph(b);
  b->dev.scc_budget = iters;
  b->dev.budget_nao = b->max_nao;
  return 0;
}

int qcx_batch_set_scc_budget_scale(qcx_batch* b, int per_group) {
  if (!b || (per_group != 0 && per_group != 1)) {
    set_error("qcx_batch_set_scc_budget_scale: per_group must be 0 or 1");
    return -1;
  }
  if ((per_group != 0) != b->budget_per_group) drop_graph(b);
  b->budget_per_group = per_group != 0;
  return 0;
}

int qcx_batch_get_scc_budget(qcx_batch* b, int32_t* iters, int32_t* per_group) {
  if (!b) return -1;
  if (iters) *iters = b->dev.scc_budget;
  if (per_group) *per_group = b->budget_per_group ? 1 : 0;
  return 0;
}

int qcx_batch_set_keep_mo(qcx_batch* b, int on) {
  if (!b || (on != 0 && on != 1)) {
    set_error("qcx_batch_set_keep_mo: on must be 0 or 1");
    return -1;
  }
  if (b->dev.keep_mo != on) drop_graph(b);
  b->dev.keep_mo = on;
  return 0;
}

int qcx_batch_mo_populations(qcx_batch* b, int mol, double* emo, double* focc, double* qmo, int32_t* ihomo) {
  if (!b || mol < 0 || mol >= b->nmol) {
    set_error("qcx_batch_mo_populations: invalid batch or molecule index");
    return -1;
  }
  if (!b->dev.keep_mo || b->precision != 0) {
    set_error("qcx_batch_mo_populations: needs qcx_batch_set_keep_mo(b, 1) and FP64 precision before qcx_batch_egrad");
    return -1;
  }
  const MolDesc& md = b->mol[mol];
  const VecLayout vl = VecLayout::make(md.nat, md.nsh, md.nao, md.len, md.nmem);
  const double* vec = b->d_vecs + md.vec_off;
  if (emo) CK(cudaMemcpyAsync(emo, vec + vl.eps, sizeof(double) * md.nao, cudaMemcpyDeviceToHost, b->stream));
  if (focc) CK(cudaMemcpyAsync(focc, vec + vl.focc, sizeof(double) * md.nao, cudaMemcpyDeviceToHost, b->stream));
  if (qmo) {
    double* d = nullptr;
    const size_t bytes = sizeof(double) * (size_t)md.nao * md.nat;
    CK(cudaMallocAsync((void**)&d, bytes, b->stream));
    qcx::launch_mo_pops(b->dev, mol, md.nao, d, b->stream);
    if (check_launch()) {
      cudaFreeAsync(d, b->stream);
      return -1;
    }
    cudaError_t e = cudaMemcpyAsync(qmo, d, bytes, cudaMemcpyDeviceToHost, b->stream);
    cudaFreeAsync(d, b->stream);
    if (e != cudaSuccess) {
      set_error(std::string("qcx_batch_mo_populations: ") + cudaGetErrorString(e));
      return -1;
    }
  }
  // ihomo = max(homo, 1) (src/tblite.f90:161): the aufbau count of one spin
  // channel of the spin-restricted wavefunction, floor(nel / 2)
  if (ihomo) {
    const int homo = (int)std::floor(0.5 * md.nel);
    *ihomo = homo > 1 ? homo : 1;
  }
  CK(cudaStreamSynchronize(b->stream));
  return md.nao;
}

int qcx_mo_spectrum(int method, int nat, const int32_t* num, const double* xyz, int charge, int multiplicity,
                    double etemp, double* energy, int32_t* nao, int32_t* ihomo, double* emo, double* focc,
                    double* qmo, int max_nao) {
  (void)multiplicity;
  if (method != QCX_METHOD_GFN2) {
    set_error("only the GFN2-xTB Hamiltonian is implemented");
    return 5;
  }
  if (nat < 1 || !num || !xyz || !energy || !nao || !ihomo || !emo || !focc || !qmo) {
    set_error("qcx_mo_spectrum: invalid arguments");
    return -1;
  }
  int32_t n1 = nat;
  double ch = charge, et = etemp;
  qcx_batch* b = qcx_batch_create(1, &n1, num, &ch, &et);
  if (!b) return -1;
  int32_t na = 0, nt = 0;
  qcx_batch_get_sizes(b, &na, &nt);
  *nao = na;
  if (na > max_nao) {
    set_error("qcx_mo_spectrum: the structure has more atomic orbitals than max_nao");
    free_batch(b);
    return -1;
  }
  // the spectrum call of eqm has no checkqc (src/mo_spec.f90:74, src/iniqm.f90:393-421)
  qcx::batch_set_checkqc(b, 0);
  int32_t st = 0;
  int rc = qcx_batch_set_keep_mo(b, 1);
  if (!rc) rc = qcx_batch_set_state(b, xyz, nullptr, nullptr);
  if (!rc) rc = qcx_batch_egrad(b);
  if (!rc) rc = qcx_batch_get(b, nullptr, nullptr, nullptr, energy, nullptr, nullptr, &st, nullptr);
  if (!rc && st != 0) {
    char buf[96];
    std::snprintf(buf, sizeof(buf), "qcx_mo_spectrum: calculation failed, status bits 0x%x", st);
    set_error(buf);
    rc = -1;
  }
  if (!rc && qcx_batch_mo_populations(b, 0, emo, focc, qmo, ihomo) < 0) rc = -1;
  free_batch(b);
  return rc;
}

}  // extern "C"
