// Shell-pair integral kernels: overlap S, H0, dipole and traceless quadrupole
// integrals (operator centred on the bra atom), and the integral-derivative
// part of the analytic gradient.
//
// One thread handles one ordered shell pair; the angular momenta of the two
// shells are template parameters so that the cartesian accumulators stay in
// registers for s/p shells. Contracted Gaussians are evaluated with the
// Obara-Saika one-dimensional overlap recursion; multipole operators centred
// on the bra atom only raise the bra power, and derivatives wrt the bra
// centre follow from d/dA [(x-A)^i e^{-a(x-A)^2}] = 2a(x-A)^{i+1}e - i(x-A)^{i-1}e.
// The integrals depend on A-B only, so d/dB = -d/dA.
#include "qcx_batch.cuh"
#include "qcx_kernels.h"

namespace qcx {

template <int L>
struct Cart;
template <>
struct Cart<0> {
  static constexpr int n = 1;
  __device__ static int p(int c, int k) { return 0; }
};
template <>
struct Cart<1> {
  static constexpr int n = 3;
  __device__ static int p(int c, int k) { return c == k ? 1 : 0; }
};
template <>
struct Cart<2> {
  static constexpr int n = 6;
  // xx, yy, zz, xy, xz, yz
  __device__ static int p(int c, int k) {
    const int t[6][3] = {{2, 0, 0}, {0, 2, 0}, {0, 0, 2}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}};
    return t[c][k];
  }
};

// coefficient of cartesian component c in spherical function i (real solid harmonics,
// d order: xy, yz, z2, xz, x2-y2)
template <int L>
__device__ inline double sph_coef(int i, int c) {
  if (L < 2) return i == c ? 1.0 : 0.0;
  const double c1 = 0.57735026918962584, c2 = 0.28867513459481287;
  switch (i) {
    case 0: return c == 3 ? 1.0 : 0.0;
    case 1: return c == 5 ? 1.0 : 0.0;
    case 2: return c == 2 ? c1 : ((c == 0 || c == 1) ? -c2 : 0.0);
    case 3: return c == 4 ? 1.0 : 0.0;
    default: return c == 0 ? 0.5 : (c == 1 ? -0.5 : 0.0);
  }
}

// 1D overlap table S1[k][i][j] for i <= IMAX, j <= LB. Every integral is a
// product of one entry per direction and each direction's recursion is linear
// in its start value, so the Gaussian factor exp(-mu r^2) of all three
// directions is carried by the x table alone: one exponential per primitive
// pair instead of three (FP64 exponentials dominate these kernels).
template <int IMAX, int LB>
__device__ inline void os_table(double a, double b, const double d[3], double S1[3][IMAX + 1][LB + 1]) {
  // one FP64 division per primitive pair (a division is a multi-instruction
  // sequence at the FP64 rate)
  const double ip = 1.0 / (a + b), o2p = 0.5 * ip, mu = a * b * ip;
  const double sp = sqrt(QCX_PI * ip);
  const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
  const double s0 = sp * exp(-mu * r2);
  const double bp = b * ip, ap = a * ip;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    double xpa = -bp * d[k], xpb = ap * d[k];
    S1[k][0][0] = k == 0 ? s0 : sp;
#pragma unroll
    for (int i = 0; i < IMAX; ++i) S1[k][i + 1][0] = xpa * S1[k][i][0] + (i > 0 ? i * o2p * S1[k][i - 1][0] : 0.0);
#pragma unroll
    for (int j = 0; j < LB; ++j)
#pragma unroll
      for (int i = 0; i <= IMAX; ++i)
        S1[k][i][j + 1] = xpb * S1[k][i][j] + o2p * ((i > 0 ? i * S1[k][i - 1][j] : 0.0) + (j > 0 ? j * S1[k][i][j - 1] : 0.0));
  }
}

__device__ inline void qidx(int q, int& c1, int& c2) {
  const int t[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
  c1 = t[q][0];
  c2 = t[q][1];
}

// ---------------------------------------------------------------------------
// forward integrals of one ordered shell pair
// ---------------------------------------------------------------------------
template <int LA, int LB>
__device__ void pair_integrals(const DevBatch& bt, const MolDesc& md, int s, int t, int A, int B) {
  const Params& P = *bt.prm;
  constexpr int NA = Cart<LA>::n, NB = Cart<LB>::n, SA = 2 * LA + 1, SB = 2 * LB + 1;
  int za = bt.Z[A], zb = bt.Z[B], ka = bt.sh_k[s], kb = bt.sh_k[t];
  double d[3] = {bt.xyz[3 * A] - bt.xyz[3 * B], bt.xyz[3 * A + 1] - bt.xyz[3 * B + 1], bt.xyz[3 * A + 2] - bt.xyz[3 * B + 2]};
  double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
  double Sc[NA][NB], Dc[3][NA][NB], Mc[6][NA][NB];
#pragma unroll
  for (int i = 0; i < NA; ++i)
#pragma unroll
    for (int j = 0; j < NB; ++j) {
      Sc[i][j] = 0.0;
#pragma unroll
      for (int c = 0; c < 3; ++c) Dc[c][i][j] = 0.0;
#pragma unroll
      for (int q = 0; q < 6; ++q) Mc[q][i][j] = 0.0;
    }
  int npa = P.sh_nprim[za][ka], npb = P.sh_nprim[zb][kb];
  for (int ip = 0; ip < npa; ++ip)
    for (int jp = 0; jp < npb; ++jp) {
      double a = P.alpha[za][ka][ip], b = P.alpha[zb][kb][jp];
      if (a * b / (a + b) * r2 > QCX_PRIM_SCREEN) continue;
      double cc = P.cnorm[za][ka][ip] * P.cnorm[zb][kb][jp];
      double S1[3][LA + 3][LB + 1];
      os_table<LA + 2, LB>(a, b, d, S1);
#pragma unroll
      for (int ca = 0; ca < NA; ++ca)
#pragma unroll
        for (int cb = 0; cb < NB; ++cb) {
          int e0 = Cart<LA>::p(ca, 0), e1 = Cart<LA>::p(ca, 1), e2 = Cart<LA>::p(ca, 2);
          int f0 = Cart<LB>::p(cb, 0), f1 = Cart<LB>::p(cb, 1), f2 = Cart<LB>::p(cb, 2);
          double x0 = S1[0][e0][f0], y0 = S1[1][e1][f1], z0 = S1[2][e2][f2];
          double x1 = S1[0][e0 + 1][f0], y1 = S1[1][e1 + 1][f1], z1 = S1[2][e2 + 1][f2];
          double x2 = S1[0][e0 + 2][f0], y2 = S1[1][e1 + 2][f1], z2 = S1[2][e2 + 2][f2];
          Sc[ca][cb] += cc * x0 * y0 * z0;
          Dc[0][ca][cb] += cc * x1 * y0 * z0;
          Dc[1][ca][cb] += cc * x0 * y1 * z0;
          Dc[2][ca][cb] += cc * x0 * y0 * z1;
          Mc[0][ca][cb] += cc * x2 * y0 * z0;
          Mc[1][ca][cb] += cc * x0 * y2 * z0;
          Mc[2][ca][cb] += cc * x0 * y0 * z2;
          Mc[3][ca][cb] += cc * x1 * y1 * z0;
          Mc[4][ca][cb] += cc * x1 * y0 * z1;
          Mc[5][ca][cb] += cc * x0 * y1 * z1;
        }
    }
  // spherical transform and store
  int n = md.nao;
  int a0 = bt.sh_ao[s], b0 = bt.sh_ao[t];
  double* Sm = mat_ptr(bt, md, kS);
  double* Hm = mat_ptr(bt, md, kH0);
  bool upper = s <= t;
  double fac = 0.0, dfac, kxyp;
  if (upper && A != B) {
    double r = sqrt(r2);
    double hA = P.selfenergy[za][ka] + P.kcn[za][ka] * bt.cn[A];
    double hB = P.selfenergy[zb][kb] + P.kcn[zb][kb] * bt.cn[B];
    h0_factor(P, za, ka, zb, kb, r, hA, hB, fac, dfac, kxyp);
  }
  double hdiag = P.selfenergy[za][ka] + P.kcn[za][ka] * bt.cn[A];
#pragma unroll
  for (int ia = 0; ia < SA; ++ia)
#pragma unroll
    for (int jb = 0; jb < SB; ++jb) {
      double sv = 0.0, dv[3] = {0, 0, 0}, mv[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
      for (int ca = 0; ca < NA; ++ca) {
        double ta = sph_coef<LA>(ia, ca);
        if (ta == 0.0) continue;
#pragma unroll
        for (int cb = 0; cb < NB; ++cb) {
          double tt = ta * sph_coef<LB>(jb, cb);
          if (tt == 0.0) continue;
          sv += tt * Sc[ca][cb];
#pragma unroll
          for (int c = 0; c < 3; ++c) dv[c] += tt * Dc[c][ca][cb];
#pragma unroll
          for (int q = 0; q < 6; ++q) mv[q] += tt * Mc[q][ca][cb];
        }
      }
      long long ij = (long long)(a0 + ia) * n + (b0 + jb);
      long long nn = (long long)n * n;
      double* Dm = mat_ptr(bt, md, kDm0);
      double* Qm = mat_ptr(bt, md, kQm0);
#pragma unroll
      for (int c = 0; c < 3; ++c) Dm[c * nn + ij] = dv[c];
      double tr = mv[0] + mv[1] + mv[2];
#pragma unroll
      for (int q = 0; q < 3; ++q) Qm[q * nn + ij] = 1.5 * mv[q] - 0.5 * tr;
#pragma unroll
      for (int q = 3; q < 6; ++q) Qm[q * nn + ij] = 1.5 * mv[q];
      if (upper) {
        long long ji = (long long)(b0 + jb) * n + (a0 + ia);
        Sm[ij] = sv;
        Sm[ji] = sv;
        double h;
        if (A != B) h = fac * sv;
        else h = (s == t && ia == jb) ? hdiag : 0.0;
        Hm[ij] = h;
        Hm[ji] = h;
      }
    }
}

// one kernel per angular-momentum class, so that each gets its own register allocation
template <int LA, int LB>
__global__ void k_integrals(DevBatch bt) {
  constexpr int cls = LA * 3 + LB;
  int idx = bt.pair_off[cls] + blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= bt.pair_off[cls + 1]) return;
  ShellPair sp = bt.pairs[idx];
  int A = bt.sh_atom[sp.s], B = bt.sh_atom[sp.t];
  if (!bt.active[bt.atom_mol[A]]) return;
  const MolDesc md = bt.mol[bt.atom_mol[A]];
  pair_integrals<LA, LB>(bt, md, sp.s, sp.t, A, B);
}

// ---------------------------------------------------------------------------
// gradient: integral derivatives contracted with P, W and the SCC potentials
// ---------------------------------------------------------------------------
template <int LA, int LB>
__device__ void pair_gradient(const DevBatch& bt, const MolDesc& md, int s, int t, int A, int B) {
  const Params& P = *bt.prm;
  constexpr int NA = Cart<LA>::n, NB = Cart<LB>::n, SA = 2 * LA + 1, SB = 2 * LB + 1;
  int za = bt.Z[A], zb = bt.Z[B], ka = bt.sh_k[s], kb = bt.sh_k[t];
  double d[3] = {bt.xyz[3 * A] - bt.xyz[3 * B], bt.xyz[3 * A + 1] - bt.xyz[3 * B + 1], bt.xyz[3 * A + 2] - bt.xyz[3 * B + 2]};
  double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
  double r = sqrt(r2);
  double hA = P.selfenergy[za][ka] + P.kcn[za][ka] * bt.cn[A];
  double hB = P.selfenergy[zb][kb] + P.kcn[zb][kb] * bt.cn[B];
  double fac, dfac, kxyp;
  h0_factor(P, za, ka, zb, kb, r, hA, hB, fac, dfac, kxyp);
  int n = md.nao;
  int a0 = bt.sh_ao[s], b0 = bt.sh_ao[t];
  const double* Pm = mat_ptr(bt, md, kP);
  const double* Wm = mat_ptr(bt, md, kW);
  VecLayout vl = VecLayout::make(md.nat, md.nsh, md.nao, md.len, md.nmem);
  const double* vec = bt.vecs + md.vec_off;
  int sl = s - md.sh_off, al = A - md.atom_off;
  double vs = vec[vl.vsh + sl];
  double wd[3], wq[6];
#pragma unroll
  for (int c = 0; c < 3; ++c) wd[c] = -vec[vl.vdp + 3 * al + c];
  {
    double v[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) v[q] = -vec[vl.vqp + 6 * al + q];
    double tr = v[0] + v[1] + v[2];
#pragma unroll
    for (int q = 0; q < 3; ++q) wq[q] = 1.5 * v[q] - 0.5 * tr;
#pragma unroll
    for (int q = 3; q < 6; ++q) wq[q] = 1.5 * v[q];
  }
  // cartesian weights
  double Pc[NA][NB], Wc[NA][NB];
#pragma unroll
  for (int ca = 0; ca < NA; ++ca)
#pragma unroll
    for (int cb = 0; cb < NB; ++cb) {
      Pc[ca][cb] = 0.0;
      Wc[ca][cb] = 0.0;
    }
#pragma unroll
  for (int ia = 0; ia < SA; ++ia)
#pragma unroll
    for (int jb = 0; jb < SB; ++jb) {
      long long ij = (long long)(a0 + ia) * n + (b0 + jb);
      double p = Pm[ij], w = Wm[ij];
      double ws = fac * p - w - vs * p;
#pragma unroll
      for (int ca = 0; ca < NA; ++ca) {
        double ta = sph_coef<LA>(ia, ca);
        if (ta == 0.0) continue;
#pragma unroll
        for (int cb = 0; cb < NB; ++cb) {
          double tt = ta * sph_coef<LB>(jb, cb);
          Pc[ca][cb] += tt * p;
          Wc[ca][cb] += tt * ws;
        }
      }
    }
  double g[3] = {0, 0, 0}, gS = 0.0;
  int npa = P.sh_nprim[za][ka], npb = P.sh_nprim[zb][kb];
  for (int ip = 0; ip < npa; ++ip)
    for (int jp = 0; jp < npb; ++jp) {
      double a = P.alpha[za][ka][ip], b = P.alpha[zb][kb][jp];
      if (a * b / (a + b) * r2 > QCX_PRIM_SCREEN) continue;
      double cc = P.cnorm[za][ka][ip] * P.cnorm[zb][kb][jp];
      double S1[3][LA + 4][LB + 1];
      os_table<LA + 3, LB>(a, b, d, S1);
#pragma unroll
      for (int ca = 0; ca < NA; ++ca)
#pragma unroll
        for (int cb = 0; cb < NB; ++cb) {
          int e[3] = {Cart<LA>::p(ca, 0), Cart<LA>::p(ca, 1), Cart<LA>::p(ca, 2)};
          int f[3] = {Cart<LB>::p(cb, 0), Cart<LB>::p(cb, 1), Cart<LB>::p(cb, 2)};
          // T[k][u] = S1[k][e_k+u][f_k]  (u = extra bra power 0..3)
          double T[3][4], dT[3][3];
#pragma unroll
          for (int k = 0; k < 3; ++k) {
#pragma unroll
            for (int u = 0; u < 4; ++u) T[k][u] = S1[k][e[k] + u][f[k]];
            // derivative wrt A_k of the 1D factor with extra power u (u = 0..2)
#pragma unroll
            for (int u = 0; u < 3; ++u) {
              int pw = e[k] + u;
              dT[k][u] = 2.0 * a * S1[k][pw + 1][f[k]] - (pw > 0 ? pw * S1[k][pw - 1][f[k]] : 0.0);
            }
          }
          double pc = cc * Pc[ca][cb], wc = cc * Wc[ca][cb];
          gS += pc * T[0][0] * T[1][0] * T[2][0];
#pragma unroll
          for (int m = 0; m < 3; ++m) {
            // factor of the 3D product for extra powers (u0,u1,u2) differentiated in m
            auto F = [&](int u0, int u1, int u2) {
              double x = (m == 0) ? dT[0][u0] : T[0][u0];
              double y = (m == 1) ? dT[1][u1] : T[1][u1];
              double z = (m == 2) ? dT[2][u2] : T[2][u2];
              return x * y * z;
            };
            double v = wc * F(0, 0, 0);
            double dd = wd[0] * F(1, 0, 0) + wd[1] * F(0, 1, 0) + wd[2] * F(0, 0, 1);
            double dq = wq[0] * F(2, 0, 0) + wq[1] * F(0, 2, 0) + wq[2] * F(0, 0, 2) + wq[3] * F(1, 1, 0) +
                        wq[4] * F(1, 0, 1) + wq[5] * F(0, 1, 1);
            g[m] += v + pc * (dd + dq);
          }
        }
    }
#pragma unroll
  for (int k = 0; k < 3; ++k) g[k] += dfac * (d[k] / r) * gS;
  for (int k = 0; k < 3; ++k) {
    atomicAdd(&bt.grad[3 * A + k], g[k]);
    atomicAdd(&bt.grad[3 * B + k], -g[k]);
  }
  atomicAdd(&bt.dedcn[A], P.kcn[za][ka] * kxyp * gS);
}

template <int LA, int LB>
__global__ void k_grad_pairs(DevBatch bt) {
  constexpr int cls = LA * 3 + LB;
  int idx = bt.pair_off[cls] + blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= bt.pair_off[cls + 1]) return;
  ShellPair sp = bt.pairs[idx];
  int A = bt.sh_atom[sp.s], B = bt.sh_atom[sp.t];
  if (A == B) return;
  if (!bt.active[bt.atom_mol[A]] || scc_pending(bt, bt.atom_mol[A])) return;
  const MolDesc md = bt.mol[bt.atom_mol[A]];
  pair_gradient<LA, LB>(bt, md, sp.s, sp.t, A, B);
}

#define QCX_CLASS_KERNELS(KERNEL)                                                                   \
  static void (*const KERNEL##_table[9])(DevBatch) = {                                              \
      KERNEL<0, 0>, KERNEL<0, 1>, KERNEL<0, 2>, KERNEL<1, 0>, KERNEL<1, 1>, KERNEL<1, 2>,             \
      KERNEL<2, 0>, KERNEL<2, 1>, KERNEL<2, 2>};

QCX_CLASS_KERNELS(k_integrals)
QCX_CLASS_KERNELS(k_grad_pairs)

static int launch_classes(void (*const table[9])(DevBatch), const DevBatch& bt, cudaStream_t st) {
  int n = 0;
  const int threads = 128;
  for (int c = 0; c < 9; ++c) {
    int cnt = bt.pair_off[c + 1] - bt.pair_off[c];
    if (cnt <= 0) continue;
    table[c]<<<(cnt + threads - 1) / threads, threads, 0, st>>>(bt);
    ++n;
  }
  return n;
}

int launch_integrals(const DevBatch& bt, cudaStream_t st) { return launch_classes(k_integrals_table, bt, st); }

int launch_grad_pairs(const DevBatch& bt, cudaStream_t st) { return launch_classes(k_grad_pairs_table, bt, st); }

}  // namespace qcx
