// Host-side set-up of the D4 part of the parameter block: the reference data
// of qcx_d4ref.h (QCxMS's include/param_d4.fh and the element tables of
// src/dftd4.f90) and the quantities the kernels need from it, computed once:
//   - reference polarisabilities with the secondary-system (hydrogen)
//     contributions removed, and the number of Gaussians of each reference,
//     as d4dim does (src/dftd4.f90:531-595);
//   - C6 of every pair of references, 3/pi times the Casimir-Polder integral
//     of the two polarisabilities by trapzd (src/dftd4.f90:452-497, 665).
#pragma once
#include <cmath>

#include "qcx_device.cuh"

namespace qcx {

// trapzd (src/dftd4.f90:452-497): the mean of the two staggered trapezoid sums
// over the 23 imaginary frequencies
inline double d4_trapzd_host(const double* pol) {
  static const double freq[QCX_D4_NFREQ] = {0.000001, 0.05, 0.1, 0.2, 0.3, 0.4, 0.5, 0.6, 0.7, 0.8, 0.9, 1.0,
                                            1.2,      1.4,  1.6, 1.8, 2.0, 2.5, 3.0, 4.0, 5.0, 7.5, 10.0};
  double even = 0.0, odd = 0.0;
  for (int k = 0; k + 1 < QCX_D4_NFREQ; ++k) {
    const double t = (freq[k + 1] - freq[k]) * (pol[k + 1] + pol[k]);
    if (k % 2 == 0) even = even + t;
    else odd = odd + t;
  }
  return 0.5 * even + 0.5 * odd;
}

// zeta of the charge scaling (src/dftd4.f90:423-434)
inline double d4_zeta_host(double a, double c, double qref, double qmod) {
  if (qmod < 0.0) return std::exp(a);
  return std::exp(a * (1.0 - std::exp(c * (1.0 - qref / qmod))));
}

inline void fill_d4_params(Params& p) {
  double refal[kMaxZ + 1][kMaxRef][QCX_D4_NFREQ];  // 24 KB
  for (int z = 0; z <= kMaxZ; ++z) {
    p.d4_refn[z] = qcx_d4_refn[z];
    p.d4_gam[z] = qcx_d4_gam[z];
    p.d4_zeff[z] = (double)qcx_d4_zeff[z];
    p.d4_en[z] = qcx_d4_en[z];
    p.d4_rcov[z] = qcx_d4_rcov[z];
    p.r4r2[z] = qcx_d4_r4r2[z];
    int cncount[16] = {0};
    cncount[0] = 1;
    for (int j = 0; j < kMaxRef; ++j) {
      p.d4_refcovcn[z][j] = qcx_d4_refcovcn[z][j];
      p.d4_refq[z][j] = qcx_d4_refq[z][j];
      p.d4_refc[z][j] = 0;
      for (int k = 0; k < QCX_D4_NFREQ; ++k) refal[z][j][k] = 0.0;
      if (z == 0 || j >= qcx_d4_refn[z]) continue;
      const int is = qcx_d4_refsys[z][j];
      const double iz = (double)qcx_d4_zeff[is];
      const double zs =
          d4_zeta_host(QCX_D4_GA, qcx_d4_gam[is] * QCX_D4_GC, qcx_d4_secq[is] + iz, qcx_d4_refh[z][j] + iz);
      for (int k = 0; k < QCX_D4_NFREQ; ++k) {
        const double sec = qcx_d4_sscale[is] * qcx_d4_secaiw[is][k] * zs;
        const double v = qcx_d4_ascale[z][j] * (qcx_d4_alphaiw[z][j][k] - qcx_d4_hcount[z][j] * sec);
        refal[z][j][k] = v > 0.0 ? v : 0.0;
      }
      cncount[(int)std::lround(qcx_d4_refcn[z][j])] += 1;
    }
    for (int j = 0; z > 0 && j < qcx_d4_refn[z]; ++j) {
      const int icn = cncount[(int)std::lround(qcx_d4_refcn[z][j])];
      p.d4_refc[z][j] = icn * (icn + 1) / 2;
    }
  }
  const double thopi = 3.0 / QCX_PI;
  for (int za = 0; za <= kMaxZ; ++za)
    for (int zb = 0; zb <= kMaxZ; ++zb)
      for (int i = 0; i < kMaxRef; ++i)
        for (int j = 0; j < kMaxRef; ++j) {
          double c6 = 0.0;
          if (za > 0 && zb > 0 && i < qcx_d4_refn[za] && j < qcx_d4_refn[zb]) {
            double pol[QCX_D4_NFREQ];
            for (int k = 0; k < QCX_D4_NFREQ; ++k) pol[k] = refal[za][i][k] * refal[zb][j][k];
            c6 = thopi * d4_trapzd_host(pol);
          }
          p.d4_c6r[za][zb][i][j] = c6;
          p.d4_c6r32[za][zb][i][j] = (float)c6;
        }
}

}  // namespace qcx
