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
#include "qcx_d4ref.h"
#include "qcx_params.h"

namespace qcx {

constexpr int kMaxZ = QCX_MAXZ;
constexpr int kMaxSh = QCX_MAXSH;
constexpr int kMaxPrim = QCX_MAXPRIM;
constexpr int kMaxRef = QCX_D4_MAXREF;  // D4 reference systems per element

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
  // D4 model of QCxMS's src/dftd4.f90 with its reference data (qcx_d4ref.h)
  int d4_refn[kMaxZ + 1];                 // reference systems per element
  int d4_refc[kMaxZ + 1][kMaxRef];        // Gaussians per reference (d4dim)
  double d4_refcovcn[kMaxZ + 1][kMaxRef];  // covalent CN of each reference
  double d4_refq[kMaxZ + 1][kMaxRef];      // charge of each reference
  double d4_gam[kMaxZ + 1];                // chemical hardness (charge scaling)
  double d4_zeff[kMaxZ + 1];               // effective nuclear charge
  double d4_en[kMaxZ + 1];                 // Pauling electronegativity (covalent CN)
  double d4_rcov[kMaxZ + 1];               // covalent radius (Bohr, covalent CN)
  double r4r2[kMaxZ + 1];                  // <r^4>/<r^2> expectation ratio (C8, damping)
  double d4_c6r[kMaxZ + 1][kMaxZ + 1][kMaxRef][kMaxRef];  // C6 of every reference pair
  float d4_c6r32[kMaxZ + 1][kMaxZ + 1][kMaxRef][kMaxRef]; // the same in FP32 (FP32 iterations)
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

// Covalent coordination number of the D4 model (covncoord / gcovncoord,
// src/dftd4.f90:292-325, 1033-1068): a pair within r^2 <= 1600 Bohr^2 adds
// den / (1 + exp(-k1 (rcov_ab / r - 1))), den = k4 exp(-(|EN_a - EN_b| + k5)^2 / k6);
// df = d(contribution)/dr.
constexpr double kD4K1 = 16.0, kD4K4 = 4.10451, kD4K5 = 19.08857, kD4K6 = 2 * 11.28174 * 11.28174;
constexpr double kD4CnThr = 1600.0;
__device__ inline void d4_cn_pair(const Params& p, int za, int zb, double r2, double& f, double& df) {
  f = 0.0;
  df = 0.0;
  if (r2 > kD4CnThr) return;
  const double r = sqrt(r2);
  const double x = fabs(p.d4_en[za] - p.d4_en[zb]) + kD4K5;
  const double den = kD4K4 * exp(-(x * x) / kD4K6);
  const double rco = p.d4_rcov[za] + p.d4_rcov[zb];
  const double ex = exp(-kD4K1 * (rco / r - 1.0));
  f = den / (1.0 + ex);
  df = (-kD4K1 * rco * ex * den) / (r2 * ((1.0 + ex) * (1.0 + ex)));
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

// Reference weights of an atom at covalent CN cn (src/dftd4.f90:1150-1193):
// gw_i = sum_{k <= refc_i} exp(-k wf (cn - cn_i)^2) / norm and d gw_i / d cn; a
// weight that overflows to NaN becomes 1 for the reference with the largest CN
// and 0 otherwise (derivative 0).
__device__ inline void d4_weights(const Params& p, int z, double cn, double* w, double* dw) {
  const int nr = p.d4_refn[z];
  double norm = 0.0, dnorm = 0.0, maxcn = -1e300;
  for (int i = 0; i < nr; ++i) {
    const double cr = p.d4_refcovcn[z][i], d = cn - cr;
    maxcn = cr > maxcn ? cr : maxcn;
    for (int k = 1; k <= p.d4_refc[z][i]; ++k) {
      const double twf = k * QCX_D4_WF, t = exp(-twf * d * d);
      norm += t;
      dnorm += 2.0 * twf * (cr - cn) * t;
    }
  }
  norm = 1.0 / norm;
  for (int i = 0; i < kMaxRef; ++i) {
    w[i] = 0.0;
    dw[i] = 0.0;
  }
  for (int i = 0; i < nr; ++i) {
    const double cr = p.d4_refcovcn[z][i], d = cn - cr;
    double e = 0.0, de = 0.0;
    for (int k = 1; k <= p.d4_refc[z][i]; ++k) {
      const double twf = k * QCX_D4_WF, t = exp(-twf * d * d);
      e += t;
      de += 2.0 * twf * (cr - cn) * t;
    }
    double wi = e * norm, dwi = de * norm - e * dnorm * norm * norm;
    if (wi != wi) wi = cr == maxcn ? 1.0 : 0.0;
    if (dwi != dwi) dwi = 0.0;
    w[i] = wi;
    dw[i] = dwi;
  }
}

// Charge scaling of reference i of element z at atomic charge q
// (zeta / dzeta, src/dftd4.f90:423-450): exp(ga (1 - exp(c (1 - qref/qmod))))
// with c = gam * gc, qref = refq_i + zeff, qmod = q + zeff; exp(ga) for qmod < 0.
__device__ inline void d4_zeta(const Params& p, int z, int i, double q, double& zeta, double& dzeta) {
  const double iz = p.d4_zeff[z], c = p.d4_gam[z] * QCX_D4_GC;
  const double qref = p.d4_refq[z][i] + iz, qmod = q + iz;
  if (qmod < 0.0) {
    zeta = exp(QCX_D4_GA);
    dzeta = 0.0;
    return;
  }
  const double t = exp(c * (1.0 - qref / qmod));
  zeta = exp(QCX_D4_GA * (1.0 - t));
  dzeta = -QCX_D4_GA * c * t * zeta * qref / (qmod * qmod);
}

// sum_ij wa_i wb_j C6(za, i, zb, j)
__device__ inline double d4_c6(const Params& p, int za, const double* wa, int zb, const double* wb) {
  double s = 0.0;
  for (int i = 0; i < p.d4_refn[za]; ++i) {
    double t = 0.0;
    for (int j = 0; j < p.d4_refn[zb]; ++j) t += wb[j] * p.d4_c6r[za][zb][i][j];
    s += wa[i] * t;
  }
  return s;
}
// both sums_ij wa_i wb_j C6_ij and da_i wb_j C6_ij with one pass over the table
__device__ inline void d4_c6_pair(const Params& p, int za, const double* wa, const double* da, int zb,
                                  const double* wb, double& c6, double& dc6) {
  double s = 0.0, ds = 0.0;
  for (int i = 0; i < p.d4_refn[za]; ++i) {
    double t = 0.0;
    for (int j = 0; j < p.d4_refn[zb]; ++j) t += wb[j] * p.d4_c6r[za][zb][i][j];
    s += wa[i] * t;
    ds += da[i] * t;
  }
  c6 = s;
  dc6 = ds;
}
__device__ inline float d4_c6(const Params& p, int za, const float* wa, int zb, const float* wb) {
  float s = 0.0f;
  for (int i = 0; i < p.d4_refn[za]; ++i) {
    float t = 0.0f;
    for (int j = 0; j < p.d4_refn[zb]; ++j) t += wb[j] * p.d4_c6r32[za][zb][i][j];
    s += wa[i] * t;
  }
  return s;
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
