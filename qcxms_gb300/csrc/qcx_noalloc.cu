// Allocation-free single-structure energy + gradient.
//
// Some callers cannot call cudaMalloc: a host program whose device memory is
// owned by another runtime's pool and capped at start-up, or a code path that
// must not trigger the implicit device synchronisation and address-space
// changes that an allocation causes. qcx_egrad_noalloc serves them: it runs the
// same kernels as qcx_egrad, but every piece of device scratch (the molecule
// description, the shell-pair list, the matrix and vector pools, the
// per-atom arrays) is carved out of one file-scope __device__ array of fixed
// size. Nothing is allocated on the device or the heap: host-side bookkeeping
// uses file-scope host buffers, inputs and outputs are plain host pointers.
//
// Limits: at most QCX_NOALLOC_MAX_ATOMS atoms and QCX_NOALLOC_MAX_NAO atomic
// orbitals (64 and 160; about 6 MB of device memory). After cudaDeviceReset the
// next call finds the array without its parameters (a marker word is checked
// on every call) and copies them in again.
// The array is held by every GPU that loads the library until the process
// exits. All calls share it: calls that overlap on the GPU race on it (within
// one process the host side serialises calls with a mutex, so only work the
// caller itself overlaps with can race).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/qcxgpu.h"
#include "qcx_batch.cuh"
#include "qcx_d4host.h"
#include "qcx_kernels.h"

namespace qcx {

constexpr int kStaticMaxAtoms = QCX_NOALLOC_MAX_ATOMS;
constexpr int kStaticMaxNao = QCX_NOALLOC_MAX_NAO;
constexpr int kStaticMaxShells = kMaxSh * kStaticMaxAtoms;
constexpr int kStaticMaxPairs = kStaticMaxShells * kStaticMaxShells;
constexpr int kStaticNmem = QCX_BROYDEN_WINDOW;

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// byte offsets of every region inside the static array
struct StaticLayout {
  size_t magic, prm, mol, Z, atom_mol, sh_atom, sh_k, sh_ao, pairs, xyz, grad, vel, mass, cn, cnd, dedcn, dedcnd, mrad,
      dmrad, w4, dw4, qat, mats, vecs, energy, ekin, status, iters, active, steps, total;
};

constexpr StaticLayout make_layout() {
  StaticLayout L{};
  size_t o = 0;
  const size_t na = kStaticMaxAtoms;
  const long long np = kStaticMaxNao + (kStaticMaxNao & 1);
  const int len = kStaticMaxShells + 9 * kStaticMaxAtoms;
  // vector block of the largest molecule (same formula as VecLayout::make)
  auto r4 = [](long long n) { return (n + 3) & ~3LL; };
  const long long vec_doubles = r4(kStaticMaxNao) * 2 + r4(len) * 2 + r4(kStaticMaxShells) + r4(3 * na) +
                                r4(6 * na) + r4(na) * 2 + r4((long long)kStaticMaxShells * kStaticMaxShells) +
                                r4((long long)na * na) * 7 + r4((long long)kMaxRef * na) * 3 +
                                r4((long long)kStaticNmem * len) * 2 +
                                r4((long long)kStaticNmem * kStaticNmem) + r4(len) * 2 + r4(kStaticNmem) +
                                r4((long long)kStaticNmem * kStaticNmem + kStaticNmem);
  L.magic = o; o = align256(o + sizeof(unsigned long long));
  L.prm = o; o = align256(o + sizeof(Params));
  L.mol = o; o = align256(o + sizeof(MolDesc));
  L.Z = o; o = align256(o + sizeof(int) * na);
  L.atom_mol = o; o = align256(o + sizeof(int) * na);
  L.sh_atom = o; o = align256(o + sizeof(int) * kStaticMaxShells);
  L.sh_k = o; o = align256(o + sizeof(int) * kStaticMaxShells);
  L.sh_ao = o; o = align256(o + sizeof(int) * kStaticMaxShells);
  L.pairs = o; o = align256(o + sizeof(ShellPair) * kStaticMaxPairs);
  L.xyz = o; o = align256(o + sizeof(double) * 3 * na);
  L.grad = o; o = align256(o + sizeof(double) * 3 * na);
  L.vel = o; o = align256(o + sizeof(double) * 3 * na);
  L.mass = o; o = align256(o + sizeof(double) * na);
  L.cn = o; o = align256(o + sizeof(double) * na);
  L.cnd = o; o = align256(o + sizeof(double) * na);
  L.dedcn = o; o = align256(o + sizeof(double) * na);
  L.dedcnd = o; o = align256(o + sizeof(double) * na);
  L.mrad = o; o = align256(o + sizeof(double) * na);
  L.dmrad = o; o = align256(o + sizeof(double) * na);
  L.w4 = o; o = align256(o + sizeof(double) * na * kMaxRef);
  L.dw4 = o; o = align256(o + sizeof(double) * na * kMaxRef);
  L.qat = o; o = align256(o + sizeof(double) * na);
  L.mats = o; o = align256(o + sizeof(double) * (size_t)kNumMat * np * np);
  L.vecs = o; o = align256(o + sizeof(double) * (size_t)vec_doubles);
  L.energy = o; o = align256(o + sizeof(double) * kNumEnergy);
  L.ekin = o; o = align256(o + sizeof(double));
  L.status = o; o = align256(o + sizeof(int));
  L.iters = o; o = align256(o + sizeof(int));
  L.active = o; o = align256(o + sizeof(int));
  L.steps = o; o = align256(o + sizeof(long long));
  L.total = o;
  return L;
}

constexpr StaticLayout kLayout = make_layout();

// the scratch of qcx_egrad_noalloc (device memory held for the process lifetime)
static __device__ __align__(256) unsigned char g_static_scratch[kLayout.total];

}  // namespace qcx

using namespace qcx;

namespace {

std::mutex g_static_mutex;
constexpr int kMaxDevices = 64;
unsigned char* g_static_base[kMaxDevices] = {nullptr};

// host-side bookkeeping buffers (file scope: no heap allocation per call)
MolDesc h_mol;
int h_Z[kStaticMaxAtoms], h_atom_mol[kStaticMaxAtoms];
int h_sh_atom[kStaticMaxShells], h_sh_k[kStaticMaxShells], h_sh_ao[kStaticMaxShells];
ShellPair h_pairs[kStaticMaxPairs];
int h_one[1] = {1};
int h_zero_i[2] = {0, 0};
long long h_zero_ll[1] = {0};
double h_energy[kNumEnergy];
Params h_params;

// Failures are reported by the return value -1, on stderr, and in the text
// qcx_last_error() returns (a fixed per-thread buffer; formatting goes into
// stack buffers, so reporting allocates nothing).
int fail(const char* what) {
  std::fprintf(stderr, "%s\n", what);
  qcx::set_last_error_text(what);
  return -1;
}

double prim_norm_host(double a, int l) { return std::pow(2.0 * a / QCX_PI, 0.75) * std::pow(4.0 * a, 0.5 * l); }

void fill_params_static(Params& p) {
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
                               ? qcx_prim_coeff[z][k][i] * prim_norm_host(qcx_prim_alpha[z][k][i], qcx_sh_l[z][k])
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

#define SCK(call, what)                                                 \
  do {                                                                  \
    cudaError_t e_ = (call);                                            \
    if (e_ != cudaSuccess) {                                            \
      char m_[192];                                                     \
      std::snprintf(m_, sizeof(m_), "%s: %s", what, cudaGetErrorString(e_)); \
      return fail(m_);                                                  \
    }                                                                   \
  } while (0)

// Written after the parameter block once it is in place; a device reset (or a
// context created anew) leaves the array zeroed, which the next call sees here.
constexpr unsigned long long kParamsMagic = 0x51435847505531ull;
unsigned long long h_magic = kParamsMagic;

// With the device current: find the array's device address (every call, it is
// a cheap lookup) and, on the first call on this device or when the array no
// longer holds the parameters (after cudaDeviceReset), copy them in.
int static_setup(int dev, unsigned char** base) {
  if (dev < 0 || dev >= kMaxDevices) return fail("qcx_egrad_noalloc: device index out of range");
  void* ptr = nullptr;
  SCK(cudaGetSymbolAddress(&ptr, g_static_scratch), "qcx_egrad_noalloc: cudaGetSymbolAddress");
  unsigned char* b = (unsigned char*)ptr;
  if (g_static_base[dev] == b) {
    unsigned long long magic = 0;
    SCK(cudaMemcpy(&magic, b + kLayout.magic, sizeof(magic), cudaMemcpyDeviceToHost),
        "qcx_egrad_noalloc: parameter check");
    if (magic == kParamsMagic) {
      *base = b;
      return 0;
    }
  }
  fill_params_static(h_params);
  SCK(cudaMemcpy(b + kLayout.prm, &h_params, sizeof(Params), cudaMemcpyHostToDevice),
      "qcx_egrad_noalloc: parameter upload");
  SCK(cudaMemcpy(b + kLayout.magic, &h_magic, sizeof(h_magic), cudaMemcpyHostToDevice),
      "qcx_egrad_noalloc: parameter upload");
  g_static_base[dev] = b;
  *base = b;
  return 0;
}

}  // namespace

extern "C" int qcx_egrad_noalloc(int method, int nat, const int32_t* num, const double* xyz, int charge,
                                 int multiplicity, double etemp, double* energy, double* grad, double* qat) {
  (void)multiplicity;
  if (method != QCX_METHOD_GFN2) return 5;  // only the GFN2-xTB Hamiltonian is implemented
  if (nat < 1 || !num || !xyz || !energy || !grad || !qat) return fail("qcx_egrad_noalloc: invalid arguments");
  if (nat > kStaticMaxAtoms) {
    char msg[160];
    std::snprintf(msg, sizeof(msg), "qcx_egrad_noalloc: %d atoms exceed the static scratch limit of %d atoms", nat,
                  kStaticMaxAtoms);
    return fail(msg);
  }
  std::lock_guard<std::mutex> lock(g_static_mutex);
  // molecule description (host buffers at file scope)
  int nsh = 0, nao = 0;
  double nel = -(double)charge;
  for (int a = 0; a < nat; ++a) {
    int z = num[a];
    if (z < 1 || z > kMaxZ) return fail("qcx_egrad_noalloc: atomic number outside the parameterised range 1..18");
    h_Z[a] = z;
    h_atom_mol[a] = 0;
    for (int k = 0; k < qcx_nsh[z]; ++k) {
      h_sh_atom[nsh] = a;
      h_sh_k[nsh] = k;
      h_sh_ao[nsh] = nao;
      nao += 2 * qcx_sh_l[z][k] + 1;
      nel += qcx_sh_refocc[z][k];
      ++nsh;
    }
  }
  if (nao > kStaticMaxNao) {
    char msg[160];
    std::snprintf(msg, sizeof(msg),
                  "qcx_egrad_noalloc: %d atomic orbitals exceed the static scratch limit of %d orbitals", nao,
                  kStaticMaxNao);
    return fail(msg);
  }
  // ordered shell pairs grouped by angular-momentum class
  int npair = 0;
  int pair_off[10];
  for (int c = 0; c < 9; ++c) {
    pair_off[c] = npair;
    for (int s = 0; s < nsh; ++s)
      for (int t = 0; t < nsh; ++t)
        if (qcx_sh_l[h_Z[h_sh_atom[s]]][h_sh_k[s]] * 3 + qcx_sh_l[h_Z[h_sh_atom[t]]][h_sh_k[t]] == c)
          h_pairs[npair++] = ShellPair{s, t};
  }
  pair_off[9] = npair;
  std::memset(&h_mol, 0, sizeof(h_mol));
  h_mol.nat = nat;
  h_mol.nsh = nsh;
  h_mol.nao = nao;
  h_mol.len = nsh + 9 * nat;
  h_mol.atom_off = 0;
  h_mol.sh_off = 0;
  h_mol.nmem = kStaticNmem;
  h_mol.mat_off = 0;
  h_mol.vec_off = 0;
  h_mol.nel = nel;
  h_mol.kT = etemp * QCX_KTOAU;
  h_mol.charge = charge;

  // The regions above were sized from the largest molecule the limits allow;
  // check this molecule's real layout against them before any launch.
  {
    const long long vec_need = VecLayout::make(nat, nsh, nao, nsh + 9 * nat, kStaticNmem).total;
    const long long np_ = nao + (nao & 1);
    if ((size_t)vec_need * sizeof(double) > kLayout.energy - kLayout.vecs ||
        (size_t)kNumMat * np_ * np_ * sizeof(double) > kLayout.vecs - kLayout.mats ||
        (size_t)npair * sizeof(ShellPair) > kLayout.xyz - kLayout.pairs)
      return fail("qcx_egrad_noalloc: internal error: the static scratch layout is too small for this molecule");
  }
  int dev = 0;
  SCK(cudaGetDevice(&dev), "qcx_egrad_noalloc: cudaGetDevice");
  unsigned char* base = nullptr;
  if (static_setup(dev, &base)) return -1;
  const StaticLayout& L = kLayout;
  cudaMemcpyKind h2d = cudaMemcpyHostToDevice;
  SCK(cudaMemcpy(base + L.mol, &h_mol, sizeof(MolDesc), h2d), "qcx_egrad_noalloc: upload");
  SCK(cudaMemcpy(base + L.Z, h_Z, sizeof(int) * nat, h2d), "qcx_egrad_noalloc: upload");
  SCK(cudaMemcpy(base + L.atom_mol, h_atom_mol, sizeof(int) * nat, h2d), "qcx_egrad_noalloc: upload");
  SCK(cudaMemcpy(base + L.sh_atom, h_sh_atom, sizeof(int) * nsh, h2d), "qcx_egrad_noalloc: upload");
  SCK(cudaMemcpy(base + L.sh_k, h_sh_k, sizeof(int) * nsh, h2d), "qcx_egrad_noalloc: upload");
  SCK(cudaMemcpy(base + L.sh_ao, h_sh_ao, sizeof(int) * nsh, h2d), "qcx_egrad_noalloc: upload");
  SCK(cudaMemcpy(base + L.pairs, h_pairs, sizeof(ShellPair) * npair, h2d), "qcx_egrad_noalloc: upload");
  SCK(cudaMemcpy(base + L.xyz, xyz, sizeof(double) * 3 * nat, h2d), "qcx_egrad_noalloc: upload");
  // state that must start fresh on every call (the array keeps the last call's contents)
  SCK(cudaMemcpy(base + L.active, h_one, sizeof(int), h2d), "qcx_egrad_noalloc: upload");
  SCK(cudaMemcpy(base + L.status, h_zero_i, sizeof(int), h2d), "qcx_egrad_noalloc: upload");
  SCK(cudaMemcpy(base + L.steps, h_zero_ll, sizeof(long long), h2d), "qcx_egrad_noalloc: upload");

  DevBatch d{};
  d.nmol = 1;
  d.natom = nat;
  d.nshell = nsh;
  d.npair = npair;
  for (int c = 0; c < 10; ++c) d.pair_off[c] = pair_off[c];
  d.prm = (const Params*)(base + L.prm);
  d.mol = (const MolDesc*)(base + L.mol);
  d.Z = (const int*)(base + L.Z);
  d.atom_mol = (const int*)(base + L.atom_mol);
  d.xyz = (double*)(base + L.xyz);
  d.grad = (double*)(base + L.grad);
  d.vel = (double*)(base + L.vel);
  d.mass = (const double*)(base + L.mass);
  d.cn = (double*)(base + L.cn);
  d.cnd = (double*)(base + L.cnd);
  d.dedcn = (double*)(base + L.dedcn);
  d.dedcnd = (double*)(base + L.dedcnd);
  d.mrad = (double*)(base + L.mrad);
  d.dmrad = (double*)(base + L.dmrad);
  d.w4 = (double*)(base + L.w4);
  d.dw4 = (double*)(base + L.dw4);
  d.qat = (double*)(base + L.qat);
  d.sh_atom = (const int*)(base + L.sh_atom);
  d.sh_k = (const int*)(base + L.sh_k);
  d.sh_ao = (const int*)(base + L.sh_ao);
  d.pairs = (const ShellPair*)(base + L.pairs);
  d.mats = (double*)(base + L.mats);
  d.vecs = (double*)(base + L.vecs);
  d.energy = (double*)(base + L.energy);
  d.status = (int*)(base + L.status);
  d.iters = (int*)(base + L.iters);
  d.ekin = (double*)(base + L.ekin);
  d.active = (int*)(base + L.active);
  d.steps_done = (long long*)(base + L.steps);
  d.max_nao = nao;
  d.smem_bytes = (int)scc_smem_bytes(nao, 0);
  d.max_iter = QCX_SCC_MAXITER;
  d.mixed_min_nao = 0;
  d.checkqc = 1;
  d.econv = QCX_SCC_ECONV;
  d.pconv = QCX_SCC_PCONV;
  d.mix_alpha = QCX_BROYDEN_ALPHA;

  cudaStream_t st = 0;  // legacy default stream: no stream object is created
  launch_cn(d, st);
  launch_integrals(d, st);
  launch_scc(d, 0, st);
  launch_zero_grad(d, st);
  launch_grad_pairs(d, st);
  launch_grad_atoms(d, st);
  SCK(cudaGetLastError(), "qcx_egrad_noalloc: kernel launch");
  cudaMemcpyKind d2h = cudaMemcpyDeviceToHost;
  int status = 0;
  SCK(cudaMemcpy(h_energy, base + L.energy, sizeof(double) * kNumEnergy, d2h), "qcx_egrad_noalloc: download");
  SCK(cudaMemcpy(&status, base + L.status, sizeof(int), d2h), "qcx_egrad_noalloc: download");
  SCK(cudaMemcpy(grad, base + L.grad, sizeof(double) * 3 * nat, d2h), "qcx_egrad_noalloc: download");
  SCK(cudaMemcpy(qat, base + L.qat, sizeof(double) * nat, d2h), "qcx_egrad_noalloc: download");
  *energy = h_energy[kETotal];
  if (status != 0) {
    char msg[128];
    if (status == QCX_STATUS_CHECKQC)
      std::snprintf(msg, sizeof(msg), "qcx_egrad_noalloc: result rejected by checkqc");
    else
      std::snprintf(msg, sizeof(msg), "qcx_egrad_noalloc: calculation failed, status bits 0x%x", status);
    return fail(msg);
  }
  return 0;
}
