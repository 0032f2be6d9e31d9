// Atom-level kernels: coordination numbers, the pairwise/three-body gradient
// terms with the coordination-number chain rule, and the leapfrog update.
#include "qcx_batch.cuh"
#include "qcx_kernels.h"

namespace qcx {

// ---------------------------------------------------------------------------
// coordination numbers, multipole radii and dispersion reference weights
// ---------------------------------------------------------------------------
// thread t of an atom-level kernel: atom t of the batch, or of the group's list
__device__ inline int atom_of_thread(const DevBatch& bt, int t) {
  if (bt.atom_list) return t < bt.natom_list ? bt.atom_list[t] : -1;
  return t < bt.natom ? t : -1;
}
inline int atom_threads(const DevBatch& bt) { return bt.atom_list ? bt.natom_list : bt.natom; }

__global__ void k_cn(DevBatch bt) {
  const int a = atom_of_thread(bt, blockIdx.x * blockDim.x + threadIdx.x);
  if (a < 0) return;
  if (!bt.active[bt.atom_mol[a]]) return;
  const Params& P = *bt.prm;
  const MolDesc md = bt.mol[bt.atom_mol[a]];
  int za = bt.Z[a];
  double xa = bt.xyz[3 * a], ya = bt.xyz[3 * a + 1], zz = bt.xyz[3 * a + 2];
  double cn = 0.0, cnd = 0.0;  // the H0 / multipole CN and the D4 covalent CN
  for (int b = md.atom_off; b < md.atom_off + md.nat; ++b) {
    if (b == a) continue;
    double dx = xa - bt.xyz[3 * b], dy = ya - bt.xyz[3 * b + 1], dz = zz - bt.xyz[3 * b + 2];
    double r2 = dx * dx + dy * dy + dz * dz;
    double r = sqrt(r2);
    double rc = P.rcov[za] + P.rcov[bt.Z[b]], f, df;
    cn_exp_pair(r, rc, f, df);
    cn += f;
    d4_cn_pair(P, za, bt.Z[b], r2, f, df);
    cnd += f;
  }
  bt.cn[a] = cn;
  bt.cnd[a] = cnd;
  double r, dr;
  mpole_radius(P, za, cn, r, dr);
  bt.mrad[a] = r;
  bt.dmrad[a] = dr;
  d4_weights(P, za, cnd, bt.w4 + (long long)a * kMaxRef, bt.dw4 + (long long)a * kMaxRef);
}

void launch_cn(const DevBatch& bt, cudaStream_t st) {
  int threads = 128;
  k_cn<<<(atom_threads(bt) + threads - 1) / threads, threads, 0, st>>>(bt);
}

__global__ void k_zero_grad(DevBatch bt) {
  const int a = atom_of_thread(bt, blockIdx.x * blockDim.x + threadIdx.x);
  if (a < 0) return;
  if (!bt.active[bt.atom_mol[a]]) return;
  bt.grad[3 * a] = 0.0;
  bt.grad[3 * a + 1] = 0.0;
  bt.grad[3 * a + 2] = 0.0;
  bt.dedcn[a] = 0.0;
  bt.dedcnd[a] = 0.0;
}

void launch_zero_grad(const DevBatch& bt, cudaStream_t st) {
  int threads = 128;
  k_zero_grad<<<(atom_threads(bt) + threads - 1) / threads, threads, 0, st>>>(bt);
}

// ---------------------------------------------------------------------------
// per-molecule gradient assembly (one CTA per molecule)
// ---------------------------------------------------------------------------
constexpr int kAtomThreads = 256;

__device__ inline double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  for (int i = 0; i < kAtomThreads / 32; ++i) s += red[i];
  __syncthreads();
  return s;
}

// gnorm (src/iniqm.f90:719-732): the reference sums grad(1,i)**2 and
// grad(2,i)**2 twice (no z term) in atom order; kept as written, with explicit
// roundings, because it decides which results checkqc accepts.
__device__ double gnorm(int nat, const double* g) {
  double gn = 0.0;
  for (int a = 0; a < nat; ++a) {
    const double x = g[3 * a], y = g[3 * a + 1];
    gn = __dadd_rn(__dadd_rn(__dadd_rn(gn, __dmul_rn(x, x)), __dmul_rn(y, y)), __dmul_rn(y, y));
  }
  return __dsqrt_rn(gn);
}

// checkqc (src/iniqm.f90:684-715), which egrad applies to every GFN2 result
// (src/iniqm.f90:650). Returns 0 when the result is accepted, else the failed
// test: 1 |E| < 1e-8 (energy left as it is), 2 gnorm outside [1e-8, 20],
// 3 a cation (mchrg > 0) with max(qat) below 1e-5 in magnitude; 2 and 3 set
// e = 0 as the reference does. 20.0 is a default-real literal, exact in FP32.
__device__ int checkqc(int nat, const double* grad, const double* qat, double charge, double& e) {
  if (fabs(e) < 1.0e-8) return 1;
  const double gn = gnorm(nat, grad);
  if (gn < 1.0e-8 || gn > (double)20.0f) {
    e = 0.0;
    return 2;
  }
  if (charge > 0.0) {
    double mx = qat[0];
    for (int a = 1; a < nat; ++a) mx = qat[a] > mx ? qat[a] : mx;
    if (fabs(mx) < 1.0e-5) {
      e = 0.0;
      return 3;
    }
  }
  return 0;
}

__global__ void __launch_bounds__(kAtomThreads) k_grad_atoms(DevBatch bt) {
  extern __shared__ __align__(16) double sm[];
  const int mol = bt.order ? bt.order[blockIdx.x] : blockIdx.x;
  const MolDesc md = bt.mol[mol];
  if (!bt.active[mol] || scc_pending(bt, mol)) return;  // no result yet: nothing to add
  if (bt.status[mol] & kCholeskyFailed) {
    if (threadIdx.x == 0) bt.active[mol] = 0;
    return;
  }
  const Params& P = *bt.prm;
  const int nat = md.nat, nsh = md.nsh, n = md.nao;
  const int off = md.atom_off;
  VecLayout vl = VecLayout::make(nat, nsh, n, md.len, md.nmem);
  const double* vec = bt.vecs + md.vec_off;
  const double* xout = vec + vl.xout;
  const double* qsh = xout;
  const double* dp = xout + nsh;
  const double* qp = xout + nsh + 3 * nat;
  const double* qa = vec + vl.qat;
  const double* wq = vec + vl.wq;  // gw zeta(q) per atom and reference, at the final charges
  const double* zq = vec + vl.zq;  // zeta(q)
  const double* gam = vec + vl.gam;
  double* g = sm;                // [3 nat]
  double* dcn = sm + 3 * nat;    // [nat]
  double* dcnd = sm + 4 * nat;   // [nat]
  double* red = sm + 5 * nat;    // [32]
  // zero-charge reference weights of the three-body term (gw zeta(0), dgw zeta(0)), FP32
  float* w0 = (float*)(sm + 6 * nat + 32);  // [nat][kMaxRef], after the int scratch below
  float* dw0 = w0 + kMaxRef * nat;
  const double* xyz = bt.xyz + 3LL * off;
  const int* Z = bt.Z + off;
  const int* sh_atom = bt.sh_atom + md.sh_off;
  const int* sh_k = bt.sh_k + md.sh_off;
  const int* sh_ao = bt.sh_ao + md.sh_off;
  const double* Pm = mat_ptr(bt, md, kP);
  for (int a = threadIdx.x; a < nat; a += blockDim.x) {
    g[3 * a] = 0.0;
    g[3 * a + 1] = 0.0;
    g[3 * a + 2] = 0.0;
    // on-site self-energy CN dependence
    double d = 0.0;
    for (int s = 0; s < nsh; ++s) {
      if (sh_atom[s] - off != a) continue;
      int l = P.sh_l[Z[a]][sh_k[s]];
      for (int i = 0; i < 2 * l + 1; ++i) {
        int mu = sh_ao[s] + i;
        d += P.kcn[Z[a]][sh_k[s]] * Pm[(long long)mu * n + mu];
      }
    }
    dcn[a] = d;
    dcnd[a] = 0.0;
    const int z = Z[a];
    for (int i = 0; i < kMaxRef; ++i) {
      double zt = 0.0, dzt;
      if (i < P.d4_refn[z]) d4_zeta(P, z, i, 0.0, zt, dzt);
      w0[kMaxRef * a + i] = (float)(bt.w4[(long long)(off + a) * kMaxRef + i] * zt);
      dw0[kMaxRef * a + i] = (float)(bt.dw4[(long long)(off + a) * kMaxRef + i] * zt);
    }
  }
  __syncthreads();
  // (a) pair terms over all ordered atom pairs (b-major, so that consecutive
  // threads add into different atoms); each pair is visited from both ends
  int* at_sh0 = (int*)(red + 32);  // [nat] first shell of each atom
  int* at_nsh = at_sh0 + nat;      // [nat] shell count
  for (int s = threadIdx.x; s < nsh; s += blockDim.x) {
    int at = sh_atom[s] - off;
    if (s == 0 || sh_atom[s - 1] - off != at) at_sh0[at] = s;
    if (s == nsh - 1 || sh_atom[s + 1] - off != at) at_nsh[at] = s + 1;  // one past the last, fixed below
  }
  __syncthreads();
  for (int x = threadIdx.x; x < nat; x += blockDim.x) at_nsh[x] -= at_sh0[x];
  __syncthreads();
  double erep = 0.0;
  for (int idx = threadIdx.x; idx < nat * nat; idx += blockDim.x) {
    int b = idx / nat, a = idx - b * nat;
    if (b == a) continue;
    double ga[3] = {0, 0, 0}, dca = 0.0, dcda = 0.0;
    int za = Z[a];
    const double* ma = dp + 3 * a;
    const double* ta = qp + 6 * a;
    {
      int zb = Z[b];
      double r[3] = {xyz[3 * a] - xyz[3 * b], xyz[3 * a + 1] - xyz[3 * b + 1], xyz[3 * a + 2] - xyz[3 * b + 2]};
      double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
      double R = sqrt(r2);
      double dEdR = 0.0;
      // isotropic electrostatics
      for (int s = at_sh0[a]; s < at_sh0[a] + at_nsh[a]; ++s)
        for (int t = at_sh0[b]; t < at_sh0[b] + at_nsh[b]; ++t) {
          double gm = gam[s * nsh + t];
          dEdR += qsh[s] * qsh[t] * (-R * gm * gm * gm);
        }
      // dispersion (two-body) at the converged charges, as dispgrad
      // (src/dftd4.f90:1198-1262): E_ab = -C6_ab(q) g_ab with
      // C6_ab(q) = sum_ij (gw zeta(q))_ai (gw zeta(q))_bj C6_ij; the CN derivative
      // goes through the weights of atom a
      double gd, dgd;
      bj_kernel(P, za, zb, R, gd, dgd);
      const double* wqa = wq + (long long)kMaxRef * a;
      const double* wqb = wq + (long long)kMaxRef * b;
      const double* zqa = zq + (long long)kMaxRef * a;
      const double* dgwa = bt.dw4 + (long long)(off + a) * kMaxRef;
      double dwa[kMaxRef];
      for (int i = 0; i < kMaxRef; ++i) dwa[i] = dgwa[i] * zqa[i];
      double c6ab, dc6a;
      d4_c6_pair(P, za, wqa, dwa, zb, wqb, c6ab, dc6a);
      dEdR += -c6ab * dgd;
      dcda += -gd * dc6a;
      // repulsion
      {
        double al = sqrt(P.rep_alpha[za] * P.rep_alpha[zb]);
        double rk = pow(R, QCX_REP_KEXP);
        double v = P.rep_zeff[za] * P.rep_zeff[zb] / R * exp(-al * rk);
        erep += 0.5 * v;
        dEdR += v * (-1.0 / R - QCX_REP_KEXP * al * rk / R);
      }
      // anisotropic electrostatics
      long long ab = (long long)a * nat + b;
      double f3 = vec[vl.f3 + ab], f5 = vec[vl.f5 + ab];
      double d3r = vec[vl.d3r + ab], d3r0 = vec[vl.d3r0 + ab], d5r = vec[vl.d5r + ab], d5r0 = vec[vl.d5r0 + ab];
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
      double s1 = qa[a] * mbr - qa[b] * mar;
      double s2 = qa[a] * rtb + qa[b] * rta + mab * r2 - 3.0 * mar * mbr;
      double tar[3], tbr[3];
      tar[0] = ta[0] * r[0] + ta[3] * r[1] + ta[4] * r[2];
      tar[1] = ta[3] * r[0] + ta[1] * r[1] + ta[5] * r[2];
      tar[2] = ta[4] * r[0] + ta[5] * r[1] + ta[2] * r[2];
      tbr[0] = tb[0] * r[0] + tb[3] * r[1] + tb[4] * r[2];
      tbr[1] = tb[3] * r[0] + tb[1] * r[1] + tb[5] * r[2];
      tbr[2] = tb[4] * r[0] + tb[5] * r[1] + tb[2] * r[2];
      for (int k = 0; k < 3; ++k) {
        double ds2 = 2.0 * qa[a] * tbr[k] + 2.0 * qa[b] * tar[k] + 2.0 * mab * r[k] - 3.0 * (mbr * ma[k] + mar * mb[k]);
        ga[k] += (d3r * s1 + d5r * s2 + dEdR) * r[k] / R + f3 * (qa[a] * mb[k] - qa[b] * ma[k]) + f5 * ds2;
      }
      dca += (d3r0 * s1 + d5r0 * s2) * 0.5 * bt.dmrad[off + a];
    }
    atomicAdd(&g[3 * a], ga[0]);
    atomicAdd(&g[3 * a + 1], ga[1]);
    atomicAdd(&g[3 * a + 2], ga[2]);
    atomicAdd(&dcn[a], dca);
    atomicAdd(&dcnd[a], dcda);
  }
  __syncthreads();
  // (b) three-body dispersion, one thread per ordered triple a > b > c. The term is
  // small (~1e-3 Eh); it is evaluated in FP32 (relative error ~1e-7) and summed in FP64.
  double eatm = 0.0;
  long long ntrip = (long long)nat * nat * nat;
  for (long long t = threadIdx.x; t < ntrip; t += blockDim.x) {
    int a = (int)(t / ((long long)nat * nat)), b = (int)((t / nat) % nat), c = (int)(t % nat);
    if (!(a > b && b > c)) continue;
    int za = Z[a], zb = Z[b], zc = Z[c];
    float rab[3], rbc[3], rca[3], x = 0, y = 0, z = 0;
    for (int k = 0; k < 3; ++k) {
      rab[k] = (float)(xyz[3 * a + k] - xyz[3 * b + k]);
      rbc[k] = (float)(xyz[3 * b + k] - xyz[3 * c + k]);
      rca[k] = (float)(xyz[3 * c + k] - xyz[3 * a + k]);
      x += rab[k] * rab[k];
      y += rbc[k] * rbc[k];
      z += rca[k] * rca[k];
    }
    const int at3[3] = {a, b, c};
    int zs[3] = {za, zb, zc};
    // zero-charge C6 of the three pairs and their CN derivatives: pair (i,j) for (0,1),(1,2),(2,0)
    float c6p[3], dc6[3][2];
    const int pi[3] = {0, 1, 2}, pj[3] = {1, 2, 0};
    for (int pr = 0; pr < 3; ++pr) {
      const int i0 = pi[pr], j0 = pj[pr];
      const float* wi = w0 + kMaxRef * at3[i0];
      const float* wj = w0 + kMaxRef * at3[j0];
      c6p[pr] = d4_c6(P, zs[i0], wi, zs[j0], wj);
      dc6[pr][0] = d4_c6(P, zs[i0], dw0 + kMaxRef * at3[i0], zs[j0], wj);
      dc6[pr][1] = d4_c6(P, zs[j0], dw0 + kMaxRef * at3[j0], zs[i0], wi);
    }
    // C9 = s9 sqrt(C6_ab C6_bc C6_ca); damping 1/(1 + 6 (R0/rbar)^alp) with the
    // geometric means R0, rbar of the three BJ radii and distances (apprabc,
    // src/dftd4.f90:1339-1400)
    float c9 = (float)QCX_D4_S9 * sqrtf(c6p[0] * c6p[1] * c6p[2]);
    float r0 = cbrtf((float)(bj_radius(P, za, zb) * bj_radius(P, zb, zc) * bj_radius(P, zc, za)));
    float rrr = sqrtf(x) * sqrtf(y) * sqrtf(z);
    float rbar = cbrtf(rrr);
    const float alp3 = (float)QCX_ATM_ALP;
    float tt = 6.0f * powf(r0 / rbar, alp3);
    float fd = 1.0f / (1.0f + tt);
    float u1 = x + z - y, u2 = x + y - z, u3 = y + z - x;
    float num = u1 * u2 * u3;
    float den = 8.0f * x * y * z;
    float ang = 3.0f * num / den + 1.0f;
    float r3 = rrr * rrr * rrr;
    float h = fd / r3;
    float en = c9 * ang * h;
    eatm += (double)en;
    float dnx = u2 * u3 + u1 * u3 - u1 * u2;
    float dny = -u2 * u3 + u1 * u3 + u1 * u2;
    float dnz = u2 * u3 - u1 * u3 + u1 * u2;
    float dlnh = fd * tt * alp3 - 9.0f;
    float ex = c9 * (3.0f * (dnx / den - num / (den * x)) * h + ang * h * dlnh / (6.0f * x));
    float ey = c9 * (3.0f * (dny / den - num / (den * y)) * h + ang * h * dlnh / (6.0f * y));
    float ez = c9 * (3.0f * (dnz / den - num / (den * z)) * h + ang * h * dlnh / (6.0f * z));
    for (int k = 0; k < 3; ++k) {
      float gx = 2.0f * ex * rab[k], gy = 2.0f * ey * rbc[k], gz = 2.0f * ez * rca[k];
      atomicAdd(&g[3 * a + k], (double)(gx - gz));
      atomicAdd(&g[3 * b + k], (double)(-gx + gy));
      atomicAdd(&g[3 * c + k], (double)(-gy + gz));
    }
    // d ln C9 / d CN'_p = 1/2 sum over the two pairs containing p of dC6/C6
    float da = 0.5f * (dc6[0][0] / c6p[0] + dc6[2][1] / c6p[2]);
    float db = 0.5f * (dc6[0][1] / c6p[0] + dc6[1][0] / c6p[1]);
    float dc = 0.5f * (dc6[1][1] / c6p[1] + dc6[2][0] / c6p[2]);
    atomicAdd(&dcnd[a], (double)(en * da));
    atomicAdd(&dcnd[b], (double)(en * db));
    atomicAdd(&dcnd[c], (double)(en * dc));
  }
  __syncthreads();
  // dedcn from the shell-pair kernel
  for (int a = threadIdx.x; a < nat; a += blockDim.x) dcn[a] += bt.dedcn[off + a];
  __syncthreads();
  // (c) coordination-number chain rule, over ordered pairs into the smem gradient
  for (int idx = threadIdx.x; idx < nat * nat; idx += blockDim.x) {
    int b = idx / nat, a = idx - b * nat;
    if (b == a) continue;
    double r[3] = {xyz[3 * a] - xyz[3 * b], xyz[3 * a + 1] - xyz[3 * b + 1], xyz[3 * a + 2] - xyz[3 * b + 2]};
    double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    double R = sqrt(r2);
    double rc = P.rcov[Z[a]] + P.rcov[Z[b]], f, df1, df2;
    cn_exp_pair(R, rc, f, df1);
    d4_cn_pair(P, Z[a], Z[b], r2, f, df2);
    double s = (dcn[a] + dcn[b]) * df1 + (dcnd[a] + dcnd[b]) * df2;
    for (int k = 0; k < 3; ++k) atomicAdd(&g[3 * a + k], s * r[k] / R);
  }
  __syncthreads();
  for (int a = threadIdx.x; a < nat; a += blockDim.x)
    for (int k = 0; k < 3; ++k) bt.grad[3LL * (off + a) + k] += g[3 * a + k];
  erep = block_sum(erep, red);
  eatm = block_sum(eatm, red);
  __syncthreads();  // the gradient rows written above are read by checkqc
  if (threadIdx.x == 0) {
    double* E = bt.energy + (long long)mol * kNumEnergy;
    E[kEAtm] = eatm;
    E[kERep] = erep;
    E[kETotal] += eatm + erep;
    if (!isfinite(E[kETotal])) bt.status[mol] |= kNonFinite;
    if (bt.checkqc && !(bt.status[mol] & kFailedEval)) {
      double e = E[kETotal];
      if (checkqc(nat, bt.grad + 3LL * off, bt.qat + off, md.charge, e)) bt.status[mol] |= kCheckqcFailed;
      E[kETotal] = e;
    }
    // A failed evaluation ends the trajectory, as QCxMS ends an MD run whose
    // energy call failed (src/md.f90:317-344). checkqc's rejections zero the
    // energy, and md.f90:317 ends the run on Epot == 0; a tiny energy
    // (|E| < 1e-8) is reported but keeps its value, and that run goes on.
    if ((bt.status[mol] & kFailedEval) || E[kETotal] == 0.0) bt.active[mol] = 0;
    else bt.steps_done[mol] += 1;
  }
}

// checkqc of one result held in device memory (qcx_checkqc): the same device
// function the gradient kernel applies to every evaluation
__global__ void k_checkqc(int nat, const double* grad, const double* qat, double charge, double* e, int* code) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double v = *e;
    *code = checkqc(nat, grad, qat, charge, v);
    *e = v;
  }
}

void launch_checkqc(int nat, const double* grad, const double* qat, double charge, double* e, int* code,
                    cudaStream_t st) {
  k_checkqc<<<1, 32, 0, st>>>(nat, grad, qat, charge, e, code);
}

void launch_grad_atoms(const DevBatch& bt, cudaStream_t st) {
  // largest molecule bounds the shared memory (nat <= nao): 5 nat + 32 doubles,
  // 2 nat ints, 2 kMaxRef nat floats
  size_t smem = sizeof(double) * ((6 + kMaxRef) * (size_t)bt.max_nao + 64);
  k_grad_atoms<<<bt.nmol, kAtomThreads, smem, st>>>(bt);
}

// ---------------------------------------------------------------------------
// leapfrog step (src/md.f90:749-773) and kinetic energy, one CTA per molecule
// ---------------------------------------------------------------------------
__global__ void k_leapfrog(DevBatch bt, double tstep) {
  __shared__ double red[32];
  const int mol = bt.order ? bt.order[blockIdx.x] : blockIdx.x;
  const MolDesc md = bt.mol[mol];
  // a trajectory whose SCC is pending has moved already and waits for its gradient
  if (!bt.active[mol] || scc_pending(bt, mol)) return;
  double ke = 0.0;
  for (int i = threadIdx.x; i < 3 * md.nat; i += blockDim.x) {
    long long e = 3LL * md.atom_off + i;
    double mass = bt.mass[md.atom_off + i / 3];
    double vold = bt.vel[e];
    // explicit roundings: no FMA contraction, same operations as the reference loop
    double vnew = __dsub_rn(vold, __ddiv_rn(__dmul_rn(tstep, bt.grad[e]), mass));
    double vavg = __dmul_rn(0.5, __dadd_rn(vold, vnew));
    bt.vel[e] = vnew;
    bt.xyz[e] = __dadd_rn(bt.xyz[e], __dmul_rn(tstep, vnew));
    ke += 0.5 * (mass * vavg * vavg);
  }
  for (int o = 16; o > 0; o >>= 1) ke += __shfl_xor_sync(0xffffffffu, ke, o);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) red[w] = ke;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < (int)(blockDim.x / 32); ++i) s += red[i];
    bt.ekin[mol] = s;
  }
}

void launch_leapfrog(const DevBatch& bt, double tstep, cudaStream_t st) {
  k_leapfrog<<<bt.nmol, 128, 0, st>>>(bt, tstep);
}

// ---------------------------------------------------------------------------
// Fragment assignment of every molecule (src/fragments.f90:93-182,
// fragment_structure): atoms i, j are bonded when r_ij < rcut * 0.5 * (R_i +
// R_j) with the QCxMS radii rad (src/covalent_radii.f90:89, in Bohr). The
// reference grows fragment 1 from atom at1 and each further fragment from the
// lowest-numbered atom not yet assigned; that is the connected components of
// the bond graph, numbered with at1's component first and the others in the
// order of their lowest atom. Here every atom starts with its own index as
// label and bonded pairs take the minimum (sweeps until nothing changes, at
// most nat), which leaves each component labelled by its lowest atom. The
// distance test uses the reference's operation order with explicit roundings,
// so the bonds, and with them the labels, are exactly the reference's.
// at1/at2 are 1-based as in the reference (at1 = at2 = 0: one fragment;
// at2 != 0: the at1-at2 bond does not count). CTA per molecule.
// ---------------------------------------------------------------------------
constexpr int kFragThreads = 256;

__global__ void __launch_bounds__(kFragThreads) k_fragments(DevBatch bt, const double* rad, double rcut, int at1,
                                                            int at2, int* frag, int* nfrag, int skip_last) {
  extern __shared__ int fsm[];
  const int mol = bt.order ? bt.order[blockIdx.x] : blockIdx.x;
  const MolDesc md = bt.mol[mol];
  // skip_last: the last atom (a collision gas atom) is not part of the ion; it gets fragment 0
  const int nat = md.nat - (skip_last && md.nat > 1 ? 1 : 0), off = md.atom_off;
  if (nat < md.nat && threadIdx.x == 0) frag[off + nat] = 0;
  int* lab = fsm;             // [nat]
  int* flag = fsm + nat;      // [1]
  if (at1 == 0 && at2 == 0) {
    for (int i = threadIdx.x; i < nat; i += blockDim.x) frag[off + i] = 1;
    if (threadIdx.x == 0) nfrag[mol] = 1;
    return;
  }
  for (int i = threadIdx.x; i < nat; i += blockDim.x) lab[i] = i;
  const double half_rcut = __dmul_rn(rcut, 0.5);
  for (int sweep = 0; sweep <= nat; ++sweep) {
    if (threadIdx.x == 0) *flag = 0;
    __syncthreads();
    for (int e = threadIdx.x; e < nat * nat; e += blockDim.x) {
      const int i = e / nat, j = e - i * nat;
      if (j <= i) continue;
      if (at2 != 0 && ((i == at1 - 1 && j == at2 - 1) || (i == at2 - 1 && j == at1 - 1))) continue;
      const double* ri = bt.xyz + 3LL * (off + i);
      const double* rj = bt.xyz + 3LL * (off + j);
      const double dx = __dsub_rn(ri[0], rj[0]), dy = __dsub_rn(ri[1], rj[1]), dz = __dsub_rn(ri[2], rj[2]);
      const double r = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
      const double rcov = __dmul_rn(half_rcut, __dadd_rn(rad[bt.Z[off + i]], rad[bt.Z[off + j]]));
      if (!(r < rcov)) continue;
      const int li = lab[i], lj = lab[j];
      if (li != lj) {
        const int m = li < lj ? li : lj;
        atomicMin(&lab[i], m);
        atomicMin(&lab[j], m);
        *flag = 1;
      }
    }
    __syncthreads();
    const int changed = *flag;
    __syncthreads();
    if (!changed) break;
  }
  // number the components: at1's first, the others by their lowest atom
  const int r1 = lab[at1 - 1];
  for (int i = threadIdx.x; i < nat; i += blockDim.x) {
    const int li = lab[i];
    int f = 1;
    if (li != r1) {
      f = 2;
      for (int k = 0; k < li; ++k)
        if (lab[k] == k && k != r1) ++f;
    }
    frag[off + i] = f;
  }
  if (threadIdx.x == 0) {
    int roots = 0;
    for (int k = 0; k < nat; ++k) roots += lab[k] == k;
    nfrag[mol] = roots;
  }
}

void launch_fragments(const DevBatch& bt, int max_nat, const double* rad, double rcut, int at1, int at2, int* frag,
                      int* nfrag, cudaStream_t st, int skip_last) {
  k_fragments<<<bt.nmol, kFragThreads, sizeof(int) * (max_nat + 1), st>>>(bt, rad, rcut, at1, at2, frag, nfrag,
                                                                          skip_last);
}

}  // namespace qcx
