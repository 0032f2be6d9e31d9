// Device-side parameter block and the per-pair physics shared by the kernels.
//
// The model is the GFN2-xTB functional form that QCxMS obtains from tblite
// (src/tblite.f90:123,133,136): STO-nG basis, CN-dependent H0, shell-resolved
// isotropic electrostatics, on-site third order, damped anisotropic
// electrostatics up to quadrupoles, self-consistent D4-type dispersion with a
// three-body term, and exponential repulsion.
#pragma once
#include <cstdint>

#include "qcx_consts.h"
#include "qcx_params.h"

namespace qcx {

constexpr int kMaxZ = QCX_MAXZ;
constexpr int kMaxSh = QCX_MAXSH;
constexpr int kMaxPrim = QCX_MAXPRIM;
constexpr int kMaxRef = QCX_MAXREF;

// Flattened copy of qcx_params.h that lives in device memory.
struct Params {
  int nsh[kMaxZ + 1];
  int sh_l[kMaxZ + 1][kMaxSh];
  int sh_nprim[kMaxZ + 1][kMaxSh];
  double zeta[kMaxZ + 1][kMaxSh];
  double refocc[kMaxZ + 1][kMaxSh];
  double selfenergy[kMaxZ + 1][kMaxSh];
  double kcn[kMaxZ + 1][kMaxSh];
  double kpoly[kMaxZ + 1][kMaxSh];
  double hardness[kMaxZ + 1][kMaxSh];
  double gamma3[kMaxZ + 1][kMaxSh];
  double alpha[kMaxZ + 1][kMaxSh][kMaxPrim];
  double cnorm[kMaxZ + 1][kMaxSh][kMaxPrim];  // contraction coeff x primitive norm
  double en[kMaxZ + 1];
  double rcov[kMaxZ + 1];
  double rep_alpha[kMaxZ + 1];
  double rep_zeff[kMaxZ + 1];
  double aes_dk[kMaxZ + 1];
  double aes_qk[kMaxZ + 1];
  double aes_rad0[kMaxZ + 1];
  double aes_valcn[kMaxZ + 1];
  int d4_nref[kMaxZ + 1];
  double d4_cnref[kMaxZ + 1][kMaxRef];
  double d4_alpha0[kMaxZ + 1][kMaxRef];
  double d4_omega[kMaxZ + 1][kMaxRef];
  double d4_eta[kMaxZ + 1];
  double r4r2[kMaxZ + 1];
};

__host__ __device__ inline int nsph(int l) { return 2 * l + 1; }
__host__ __device__ inline int ncart(int l) { return (l + 1) * (l + 2) / 2; }

// ---------------------------------------------------------------------------
// coordination numbers
// ---------------------------------------------------------------------------
__device__ inline void cn_exp_pair(double r, double rc, double& f, double& df) {
  double e = exp(-QCX_KCN * (rc / r - 1.0));
  f = 1.0 / (1.0 + e);
  df = -f * f * e * QCX_KCN * rc / (r * r);
}

__device__ inline void cn_erf_pair(double r, double rc, double& f, double& df) {
  double t = QCX_KERF * (r / rc - 1.0);
  f = 0.5 * erfc(t);
  df = -QCX_KERF / (rc * sqrt(QCX_PI)) * exp(-t * t);
}

// ---------------------------------------------------------------------------
// H0 scaling  H0_{mu nu} = fac(R) * S_{mu nu}
// ---------------------------------------------------------------------------
__device__ inline double kpair(int l1, int l2) {
  if (l1 == 2 || l2 == 2) return QCX_K_XD;
  if (l1 == 0 && l2 == 0) return QCX_K_SS;
  if (l1 == 1 && l2 == 1) return QCX_K_PP;
  return QCX_K_SP;
}

__device__ inline void h0_factor(const Params& p, int za, int ka, int zb, int kb, double r, double hA, double hB,
                                 double& fac, double& dfac, double& kxyp) {
  double zeta_a = p.zeta[za][ka], zeta_b = p.zeta[zb][kb];
  double y = sqrt(2.0 * sqrt(zeta_a * zeta_b) / (zeta_a + zeta_b));
  double den = p.en[za] - p.en[zb];
  double x = 1.0 + QCX_KEN * den * den;
  double rr = sqrt(r / (p.rcov[za] + p.rcov[zb]));
  double pa = 1.0 + p.kpoly[za][ka] * rr, pb = 1.0 + p.kpoly[zb][kb] * rr;
  double pi = pa * pb;
  double dpi = (p.kpoly[za][ka] * pb + p.kpoly[zb][kb] * pa) * 0.5 * rr / r;
  double base = kpair(p.sh_l[za][ka], p.sh_l[zb][kb]) * x * y;
  fac = 0.5 * base * (hA + hB) * pi;
  dfac = 0.5 * base * (hA + hB) * dpi;
  kxyp = base * pi;
}

// ---------------------------------------------------------------------------
// electrostatics / dispersion helpers
// ---------------------------------------------------------------------------
__device__ inline void mpole_radius(const Params& p, int z, double cn, double& r, double& dr) {
  double r0 = p.aes_rad0[z];
  double t = exp(-QCX_AES_KMP * (cn - p.aes_valcn[z] - QCX_AES_SHIFT));
  double s = 1.0 / (1.0 + t);
  r = r0 + (QCX_AES_RMAX - r0) * s;
  dr = (QCX_AES_RMAX - r0) * s * s * t * QCX_AES_KMP;
}

// f_n(R) = 1 / (R^n (1 + 6 (R0/R)^a)), derivatives wrt R and R0
__device__ inline void mp_kernel(int n, double a, double r, double r0, double& f, double& dfr, double& dfr0) {
  double t = 6.0 * pow(r0 / r, a);
  double fd = 1.0 / (1.0 + t);
  double rn = (n == 3) ? r * r * r : r * r * r * r * r;
  f = fd / rn;
  double dfd_r = a * t / (r * (1.0 + t) * (1.0 + t));
  double dfd_r0 = -a * t / (r0 * (1.0 + t) * (1.0 + t));
  dfr = dfd_r / rn - n * fd / (rn * r);
  dfr0 = dfd_r0 / rn;
}

__device__ inline double c6ref(const Params& p, int za, int i, int zb, int j) {
  double aa = p.d4_alpha0[za][i], ab = p.d4_alpha0[zb][j];
  double wa = p.d4_omega[za][i], wb = p.d4_omega[zb][j];
  return 1.5 * aa * ab * wa * wb / (wa + wb);
}

__device__ inline void d4_weights(const Params& p, int z, double cn, double* w, double* dw) {
  int nr = p.d4_nref[z];
  double ex[kMaxRef], mx = -1e300;
  for (int i = 0; i < nr; ++i) {
    double t = cn - p.d4_cnref[z][i];
    ex[i] = -QCX_D4_WF * t * t;
    mx = ex[i] > mx ? ex[i] : mx;
  }
  double sum = 0.0, dsum = 0.0, g[kMaxRef], dg[kMaxRef];
  for (int i = 0; i < nr; ++i) {
    g[i] = exp(ex[i] - mx);
    dg[i] = -2.0 * QCX_D4_WF * (cn - p.d4_cnref[z][i]) * g[i];
    sum += g[i];
    dsum += dg[i];
  }
  for (int i = 0; i < kMaxRef; ++i) {
    w[i] = 0.0;
    dw[i] = 0.0;
  }
  for (int i = 0; i < nr; ++i) {
    w[i] = g[i] / sum;
    dw[i] = (dg[i] * sum - g[i] * dsum) / (sum * sum);
  }
}

__device__ inline void d4_zeta(const Params& p, int z, double q, double& zeta, double& dzeta) {
  double t = QCX_D4_GC * p.d4_eta[z] / (double)z;
  double ex = exp(t * q);
  zeta = exp(QCX_D4_GA * (1.0 - ex));
  dzeta = zeta * (-QCX_D4_GA * ex * t);
}

__device__ inline double bj_radius(const Params& p, int za, int zb) {
  return QCX_D4_A1 * sqrt(3.0 * p.r4r2[za] * p.r4r2[zb]) + QCX_D4_A2;
}

__device__ inline void bj_kernel(const Params& p, int za, int zb, double r, double& g, double& dg) {
  double qq = 3.0 * p.r4r2[za] * p.r4r2[zb];
  double r0 = QCX_D4_A1 * sqrt(qq) + QCX_D4_A2;
  double r2 = r * r, r6 = r2 * r2 * r2, r8 = r6 * r2;
  double r02 = r0 * r0, r06 = r02 * r02 * r02, r08 = r06 * r02;
  double t6 = 1.0 / (r6 + r06), t8 = 1.0 / (r8 + r08);
  g = QCX_D4_S6 * t6 + QCX_D4_S8 * qq * t8;
  dg = -QCX_D4_S6 * 6.0 * r * r2 * r2 * t6 * t6 - QCX_D4_S8 * qq * 8.0 * r6 * r * t8 * t8;
}

}  // namespace qcx
