// Fragment ionisation potentials and their Boltzmann weights: the GFN2 part of
// the charge assignment QCxMS runs when a trajectory ends in fragments.
//
// analyse (src/analyse.f90:13-467) splits the final structure into fragments
// (avg_frag_struc, src/analyse.f90:471-503: each fragment keeps its atoms in
// their original order), then for every fragment computes the energy of the
// neutral and of the ions of charge 1..|mchrg| (sign of mchrg) through eqm
// (src/iniqm.f90:241-427) at etemp = 300 K for GFN2 (src/analyse.f90:244-248),
// and stores fragip(i,c) = (E_ion(c) - E_neutral) * autoev
// (src/analyse.f90:367-368). Here every such single point of every trajectory
// is one molecule of a single batch, so all of them run in one pass of the
// batched kernels. boltz (src/utility.f90:469-498) turns IPs into weights.
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/qcxgpu.h"
#include "qcx_consts.h"
#include "qcx_kernels.h"
#include "qcx_params.h"

namespace {

// src/xtb_mctc_convert.f90:27,30
constexpr double kAutoEV = 27.21138505;
constexpr double kAutoKcal = 627.50947428;

// eself (src/iniqm.f90:430-450): energy of a fragment without electrons,
// sum over atoms of z^2/2 * gam + z^3/3 * gam3 with z = valence electrons.
// gam and gam3 are the atomic hardness and third-order parameter of the
// method; in this parameter set those are the first shell's values.
double self_energy(const int32_t* num, const std::vector<int>& atoms) {
  double e = 0.0;
  for (int a : atoms) {
    int z = num[a];
    double zv = qcx_nvalence[z];
    e += 0.5 * zv * zv * qcx_sh_hardness[z][0] + zv * zv * zv * qcx_sh_gamma3[z][0] / 3.0;
  }
  return e;
}

// In mixed mode, fragments with fewer atomic orbitals run FP64 SCC iterations
// only. Measured on 142 fragment single points of 9-33 AOs: with FP32
// iterations 6 did not converge within 100 iterations (their FP32 phase
// stalled above the hand-over residual), with FP64 iterations 3-4; at these
// sizes the FP32 iterations save little time.
constexpr int kFragMixedMinNao = 48;

// IP bounds of src/analyse.f90:386-403 (eV); outside them the IPs are rejected
bool ip_in_bounds(int mchrg, double ip) {
  if (mchrg < 0) return !(ip > 40.0 || ip < -35.0);
  if (mchrg == 1) return !(ip < 0.0 || ip > 50.0);
  return !(ip < 0.0 || ip > 100.0);
}

}  // namespace

extern "C" {

int qcx_fragment_ips(int method, int ntraj, const int32_t* nat, const int32_t* num, const double* xyz,
                     const int32_t* frag, int mchrg, double etemp, int precision, double* fragip, double* efrag,
                     int32_t* ipok) {
  if (method != QCX_METHOD_GFN2) {
    qcx::set_last_error("qcx_fragment_ips: only GFN2 (method 2) is parameterised");
    return 5;
  }
  const int nch = mchrg < 0 ? -mchrg : mchrg;
  if (ntraj < 1 || !nat || !num || !xyz || !frag || !fragip || !ipok || nch < 1 ||
      nch > QCX_FRAGIP_MAX_CHARGE || !(etemp >= 0.0) || (precision != 0 && precision != 1)) {
    qcx::set_last_error("qcx_fragment_ips: invalid arguments (ntraj >= 1, 1 <= |mchrg| <= QCX_FRAGIP_MAX_CHARGE, "
                        "etemp >= 0, precision 0 or 1, non-NULL arrays)");
    return -1;
  }
  const int sgn = mchrg < 0 ? -1 : 1;
  const int per_traj = QCX_MAX_FRAGMENTS * nch;
  // single points: trajectory t, fragment i (0-based), charge index c (0 = neutral)
  struct Point {
    int t, i, c;
    std::vector<int> atoms;
  };
  std::vector<Point> pts;
  std::vector<int> nfrag(ntraj, 0);
  std::vector<double> energy((size_t)ntraj * QCX_MAX_FRAGMENTS * (nch + 1), 0.0);
  std::vector<char> failed((size_t)ntraj, 0);
  long long aoff = 0;
  for (int t = 0; t < ntraj; ++t) {
    if (nat[t] < 1) {
      qcx::set_last_error("qcx_fragment_ips: trajectory with no atoms");
      return -1;
    }
    int nf = 0;
    for (int a = 0; a < nat[t]; ++a) {
      if (num[aoff + a] < 1 || num[aoff + a] > 18) {
        qcx::set_last_error("qcx_fragment_ips: atomic number outside the parameterised range 1..18");
        return -1;
      }
      int f = frag[aoff + a];
      if (f < 1 || f > QCX_MAX_FRAGMENTS) {
        qcx::set_last_error("qcx_fragment_ips: fragment numbers must lie in 1..QCX_MAX_FRAGMENTS");
        return -1;
      }
      nf = f > nf ? f : nf;
    }
    std::vector<std::vector<int>> members(nf);
    for (int a = 0; a < nat[t]; ++a) members[frag[aoff + a] - 1].push_back((int)(aoff + a));
    for (int i = 0; i < nf; ++i)
      if (members[i].empty()) {
        qcx::set_last_error("qcx_fragment_ips: fragment numbers of a trajectory must be 1..nfrag without gaps");
        return -1;
      }
    nfrag[t] = nf;
    aoff += nat[t];
    // one fragment: no IPs (src/analyse.f90:137-142 returns before them)
    if (nf < 2) continue;
    for (int i = 0; i < nf; ++i) {
      int nval = 0;
      for (int a : members[i]) nval += (int)qcx_nvalence[num[a]];
      for (int c = 0; c <= nch; ++c) {
        int nel = nval - sgn * c;  // electrons_amount, src/iniqm.f90:45-63
        double* e = &energy[((size_t)t * QCX_MAX_FRAGMENTS + i) * (nch + 1) + c];
        if (nel == 0) {
          *e = self_energy(num, members[i]);
        } else if (nel < 0) {
          failed[t] = 1;  // more charge than valence electrons: no calculation possible
        } else {
          pts.push_back({t, i, c, members[i]});
        }
      }
    }
  }
  if (!pts.empty()) {
    const int np = (int)pts.size();
    std::vector<int32_t> pnat(np), pnum;
    std::vector<double> pch(np), pet(np, etemp), pxyz, pe(np);
    std::vector<int32_t> pst(np);
    for (int k = 0; k < np; ++k) {
      pnat[k] = (int32_t)pts[k].atoms.size();
      pch[k] = (double)(sgn * pts[k].c);
      for (int a : pts[k].atoms) {
        pnum.push_back(num[a]);
        for (int d = 0; d < 3; ++d) pxyz.push_back(xyz[3 * (size_t)a + d]);
      }
    }
    qcx_batch* b = qcx_batch_create(np, pnat.data(), pnum.data(), pch.data(), pet.data());
    if (!b) return -1;
    qcx::batch_set_mixed_min_nao(b, kFragMixedMinNao);
    qcx::batch_set_checkqc(b, 0);  // eqm (src/iniqm.f90:241-427) does not call checkqc
    int rc = qcx_batch_set_precision(b, precision);
    if (!rc) rc = qcx_batch_set_state(b, pxyz.data(), nullptr, nullptr);
    if (!rc) rc = qcx_batch_egrad(b);
    if (!rc) rc = qcx_batch_get(b, nullptr, nullptr, nullptr, pe.data(), nullptr, nullptr, pst.data(), nullptr);
    qcx_batch_destroy(b);
    if (rc) return -1;
    for (int k = 0; k < np; ++k) {
      const Point& p = pts[k];
      // a failed calculation leaves energy 0, which eqm reports as a QM code failure
      double e = (pst[k] == 0 && std::isfinite(pe[k])) ? pe[k] : 0.0;
      energy[((size_t)p.t * QCX_MAX_FRAGMENTS + p.i) * (nch + 1) + p.c] = e;
    }
  }
  for (int t = 0; t < ntraj; ++t) {
    double* ip = fragip + (size_t)t * per_traj;
    for (int k = 0; k < per_traj; ++k) ip[k] = 0.0;
    bool ok = !failed[t];
    for (int i = 0; i < nfrag[t] && nfrag[t] > 1; ++i) {
      const double* e = &energy[((size_t)t * QCX_MAX_FRAGMENTS + i) * (nch + 1)];
      for (int c = 0; c <= nch; ++c)
        if (std::fabs(e[c]) < 1e-10) ok = false;  // src/iniqm.f90:415-421
      for (int c = 1; c <= nch; ++c) {
        if (e[c] != 0.0 && e[0] != 0.0) {
          ip[i * nch + c - 1] = (e[c] - e[0]) * kAutoEV;
          if (!ip_in_bounds(mchrg, ip[i * nch + c - 1])) ok = false;
        }
      }
    }
    ipok[t] = ok ? 1 : 0;
    if (efrag) {
      double* out = efrag + (size_t)t * QCX_MAX_FRAGMENTS * (nch + 1);
      const double* e = &energy[(size_t)t * QCX_MAX_FRAGMENTS * (nch + 1)];
      for (int k = 0; k < QCX_MAX_FRAGMENTS * (nch + 1); ++k) out[k] = e[k];
    }
  }
  return 0;
}

int qcx_fragment_formula(int nat, const int32_t* num, const int32_t* frag, const double* mass, int32_t* nfrag,
                         double* fragm_amu, char* formula) {
  if (nat < 1 || !num || !frag || !mass || !nfrag) {
    qcx::set_last_error("qcx_fragment_formula: invalid arguments");
    return -1;
  }
  static const char* const sym[] = {"",  "H",  "He", "Li", "Be", "B",  "C",  "N",  "O",  "F",
                                    "Ne", "Na", "Mg", "Al", "Si", "P",  "S",  "Cl", "Ar"};
  // src/xtb_mctc_convert.f90:47-52: autoamu = (1/amutokg) * metokg
  constexpr double kgtoamu = 1.0 / 1.660539040e-27;
  constexpr double autoamu = kgtoamu * 9.10938356e-31;
  double fm[QCX_MAX_FRAGMENTS] = {0.0};
  int el[QCX_MAX_FRAGMENTS][19] = {{0}};
  for (int i = 0; i < nat; ++i) {
    if (frag[i] < 1 || frag[i] > QCX_MAX_FRAGMENTS || num[i] < 1 || num[i] > 18) {
      qcx::set_last_error("qcx_fragment_formula: fragment numbers 1..QCX_MAX_FRAGMENTS, elements 1..18");
      return -1;
    }
    fm[frag[i] - 1] += mass[i];
    el[frag[i] - 1][num[i]] += 1;
  }
  int n = 0;
  for (int f = 0; f < QCX_MAX_FRAGMENTS; ++f) {
    if (!(fm[f] > 0.0)) continue;
    // elements in order of atomic number, each with its count
    std::string s;
    for (int z = 1; z <= 18; ++z)
      if (el[f][z]) s += std::string(sym[z]) + std::to_string(el[f][z]);
    if (fragm_amu) fragm_amu[n] = fm[f] * autoamu;
    if (formula) {
      std::snprintf(formula + 80 * n, 80, "%s", s.c_str());
    }
    ++n;
  }
  *nfrag = n;
  return 0;
}

int qcx_boltz(int units, int nfrag, int mchrg, double temp, const double* ip, double* fragchrg2) {
  if ((units != 1 && units != 2) || nfrag < 1 || mchrg < 1 || !ip || !fragchrg2) {
    qcx::set_last_error("qcx_boltz: units must be 1 (kcal/mol) or 2 (eV), nfrag >= 1, mchrg >= 1");
    return -1;
  }
  const double f = temp * QCX_KTOAU * (units == 1 ? kAutoKcal : kAutoEV);
  // Fortran order ip(nfrag, mchrg); the sum runs fragment-major as the reference loops do
  double esum = 0.0;
  for (int i = 0; i < nfrag; ++i)
    for (int j = 0; j < mchrg; ++j) esum += std::exp(-ip[i + (size_t)j * nfrag] / f);
  for (int i = 0; i < nfrag; ++i)
    for (int j = 0; j < mchrg; ++j) fragchrg2[i + (size_t)j * nfrag] = std::exp(-ip[i + (size_t)j * nfrag] / f) / esum;
  return 0;
}

}  // extern "C"
