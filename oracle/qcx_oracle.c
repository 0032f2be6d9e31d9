/*
 * CPU FP64 oracle for the QCxMS trajectory-step hot path -- TEST INFRASTRUCTURE.
 *
 * Only tests, the smoke check and bench.py's CPU-baseline leg load this file's
 * library, and only as the checker. Parity with tblite is UNPINNED (tblite and
 * the GFN2 parameter tables are not part of the QCxMS sources; QCxMS ships no
 * reference energies). See qcx_oracle.h for what it restates.
 *
 * Model (GFN2-xTB functional form, Bannwarth/Ehlert/Grimme JCTC 2019):
 *   E = E_band + E_ies + E_3 + E_aes + E_axc + E_disp + E_atm + E_rep + E_ts
 * evaluated self-consistently in the Mulliken shell charges, atomic dipoles
 * and traceless quadrupoles, spin-restricted with Fermi smearing (QCxMS builds
 * the tblite wavefunction with one spin channel, src/tblite.f90:111,133).
 */
#include "qcx_oracle.h"

#include <math.h>
#include <time.h>
#include <stdlib.h>
#include <string.h>

#include "../qcxms_gb300/csrc/qcx_consts.h"
#include "../qcxms_gb300/csrc/qcx_params.h"
#include "../qcxms_gb300/csrc/qcx_d4ref.h"

#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* molecule / basis bookkeeping                                              */
/* ------------------------------------------------------------------------ */
typedef struct {
  int nat, nsh, nao;
  const int* Z;
  const double* xyz;
  int *sh_atom, *sh_l, *sh_k, *sh_ao0, *sh_nao;
  int *ao_sh, *ao_atom;
  int *at_sh0, *at_nsh;
} mol_t;

static const int NSPH[3] = {1, 3, 5};
static const int NCART[3] = {1, 3, 6};
static const int CPOW[3][6][3] = {
    {{0, 0, 0}},
    {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}},
    {{2, 0, 0}, {0, 2, 0}, {0, 0, 2}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}}};

static void mol_free(mol_t* m) {
  free(m->sh_atom); free(m->sh_l); free(m->sh_k); free(m->sh_ao0); free(m->sh_nao);
  free(m->ao_sh); free(m->ao_atom); free(m->at_sh0); free(m->at_nsh);
}

static int mol_init(mol_t* m, int nat, const int* Z, const double* xyz) {
  memset(m, 0, sizeof(*m));
  m->nat = nat; m->Z = Z; m->xyz = xyz;
  int nsh = 0, nao = 0;
  for (int a = 0; a < nat; ++a) {
    if (Z[a] < 1 || Z[a] > QCX_MAXZ) return -1;
    nsh += qcx_nsh[Z[a]];
    for (int k = 0; k < qcx_nsh[Z[a]]; ++k) nao += NSPH[qcx_sh_l[Z[a]][k]];
  }
  m->nsh = nsh; m->nao = nao;
  m->sh_atom = malloc(sizeof(int) * nsh); m->sh_l = malloc(sizeof(int) * nsh);
  m->sh_k = malloc(sizeof(int) * nsh); m->sh_ao0 = malloc(sizeof(int) * nsh);
  m->sh_nao = malloc(sizeof(int) * nsh);
  m->ao_sh = malloc(sizeof(int) * (nao + 1)); m->ao_atom = malloc(sizeof(int) * (nao + 1));
  m->at_sh0 = malloc(sizeof(int) * nat); m->at_nsh = malloc(sizeof(int) * nat);
  int s = 0, mu = 0;
  for (int a = 0; a < nat; ++a) {
    m->at_sh0[a] = s; m->at_nsh[a] = qcx_nsh[Z[a]];
    for (int k = 0; k < qcx_nsh[Z[a]]; ++k, ++s) {
      int l = qcx_sh_l[Z[a]][k];
      m->sh_atom[s] = a; m->sh_l[s] = l; m->sh_k[s] = k; m->sh_ao0[s] = mu; m->sh_nao[s] = NSPH[l];
      for (int i = 0; i < NSPH[l]; ++i, ++mu) { m->ao_sh[mu] = s; m->ao_atom[mu] = a; }
    }
  }
  return 0;
}

int qcxo_nao(int nat, const int* Z) {
  int n = 0;
  for (int a = 0; a < nat; ++a) {
    if (Z[a] < 1 || Z[a] > QCX_MAXZ) return -1;
    for (int k = 0; k < qcx_nsh[Z[a]]; ++k) n += NSPH[qcx_sh_l[Z[a]][k]];
  }
  return n;
}

int qcxo_nsh(int nat, const int* Z) {
  int n = 0;
  for (int a = 0; a < nat; ++a) {
    if (Z[a] < 1 || Z[a] > QCX_MAXZ) return -1;
    n += qcx_nsh[Z[a]];
  }
  return n;
}

void qcxo_default_opts(qcxo_opts* o) {
  o->max_iter = QCX_SCC_MAXITER;
  o->econv = QCX_SCC_ECONV;
  o->pconv = QCX_SCC_PCONV;
  o->broyden_alpha = QCX_BROYDEN_ALPHA;
}

/* ------------------------------------------------------------------------ */
/* coordination numbers                                                     */
/* ------------------------------------------------------------------------ */
/* exponential counting function (H0 self-energies, multipole radii) */
static void cn_exp_pair(double r, double rc, double* f, double* df) {
  double e = exp(-QCX_KCN * (rc / r - 1.0));
  *f = 1.0 / (1.0 + e);
  *df = -(*f) * (*f) * e * QCX_KCN * rc / (r * r);
}

/* Covalent coordination number of the D4 model, covncoord / gcovncoord
 * (src/dftd4.f90:292-325, 1033-1068): pairs within r^2 <= 1600 Bohr^2 add
 * den / (1 + exp(-k1 (rcov_ij / r - 1))) with den = k4 exp(-(|EN_i - EN_j| + k5)^2 / k6),
 * k1 = 16, k4 = 4.10451, k5 = 19.08857, k6 = 2 * 11.28174^2 (src/dftd4.f90:10-19),
 * the D3 covalent radii and Pauling electronegativities of src/dftd4.f90.
 * *df = d(contribution)/dr. */
#define D4_K1 16.0
#define D4_K4 4.10451
#define D4_K5 19.08857
#define D4_K6 (2 * 11.28174 * 11.28174)
#define D4_CN_THR 1600.0
static void d4_cn_pair(int za, int zb, double r2, double* f, double* df) {
  *f = 0.0; *df = 0.0;
  if (r2 > D4_CN_THR) return;
  double r = sqrt(r2);
  double den = D4_K4 * exp(-pow(fabs(qcx_d4_en[za] - qcx_d4_en[zb]) + D4_K5, 2) / D4_K6);
  double rco = qcx_d4_rcov[za] + qcx_d4_rcov[zb];
  double ex = exp(-D4_K1 * (rco / r - 1.0));
  *f = den / (1.0 + ex);
  *df = (-D4_K1 * rco * ex * den) / (r2 * ((1.0 + ex) * (1.0 + ex)));
}

static void compute_cn(const mol_t* m, double* cn, double* cnd) {
  for (int a = 0; a < m->nat; ++a) { cn[a] = 0.0; cnd[a] = 0.0; }
  for (int a = 0; a < m->nat; ++a)
    for (int b = 0; b < a; ++b) {
      double d[3], r2 = 0;
      for (int k = 0; k < 3; ++k) { d[k] = m->xyz[3 * a + k] - m->xyz[3 * b + k]; r2 += d[k] * d[k]; }
      double r = sqrt(r2);
      double rc = qcx_rcov[m->Z[a]] + qcx_rcov[m->Z[b]], f, df;
      cn_exp_pair(r, rc, &f, &df); cn[a] += f; cn[b] += f;
      d4_cn_pair(m->Z[a], m->Z[b], r2, &f, &df); cnd[a] += f; cnd[b] += f;
    }
}

/* ------------------------------------------------------------------------ */
/* one-electron integrals over a shell pair                                  */
/* ------------------------------------------------------------------------ */
static double prim_norm(double a, int l) { return pow(2.0 * a / QCX_PI, 0.75) * pow(4.0 * a, 0.5 * l); }

/* cartesian -> spherical (real solid harmonics), d order: xy, yz, z2, xz, x2-y2 */
static void cart2sph(int l, const double* c, double* s) {
  if (l < 2) { for (int i = 0; i < NCART[l]; ++i) s[i] = c[i]; return; }
  const double c1 = 1.0 / sqrt(3.0), c2 = 0.5 / sqrt(3.0);
  s[0] = c[3]; s[1] = c[5]; s[2] = c[2] * c1 - (c[0] + c[1]) * c2; s[3] = c[4]; s[4] = 0.5 * (c[0] - c[1]);
}

typedef struct {
  /* blocks [bra ao][ket ao] in spherical functions */
  double S[5][5], D[3][5][5], Q[6][5][5];
  double dS[3][5][5], dD[3][3][5][5], dQ[6][3][5][5]; /* derivative index = d(A-B) component */
} spair_t;

/* Integrals <bra on A | op centred at A | ket on B>, d = A - B. */
static void shell_pair(int za, int ka, int zb, int kb, const double d[3], int deriv, spair_t* out) {
  int la = qcx_sh_l[za][ka], lb = qcx_sh_l[zb][kb];
  int npa = qcx_sh_nprim[za][ka], npb = qcx_sh_nprim[zb][kb];
  double Sc[6][6] = {{0}}, Dc[3][6][6] = {{{0}}}, Mc[6][6][6] = {{{0}}};
  double dSc[3][6][6] = {{{0}}}, dDc[3][3][6][6] = {{{{0}}}}, dMc[6][3][6][6] = {{{{0}}}};
  double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
  /* second-moment component list xx,yy,zz,xy,xz,yz */
  static const int QI[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
  for (int i = 0; i < npa; ++i)
    for (int j = 0; j < npb; ++j) {
      double a = qcx_prim_alpha[za][ka][i], b = qcx_prim_alpha[zb][kb][j];
      double p = a + b, mu = a * b / p;
      if (mu * r2 > QCX_PRIM_SCREEN) continue;
      double cc = qcx_prim_coeff[za][ka][i] * qcx_prim_coeff[zb][kb][j] * prim_norm(a, la) * prim_norm(b, lb);
      double S1[3][6][3];
      for (int k = 0; k < 3; ++k) {
        double xpa = -b * d[k] / p, xpb = a * d[k] / p, o2p = 0.5 / p;
        S1[k][0][0] = sqrt(QCX_PI / p) * exp(-mu * d[k] * d[k]);
        for (int ii = 0; ii < la + 3; ++ii)
          S1[k][ii + 1][0] = xpa * S1[k][ii][0] + (ii > 0 ? ii * o2p * S1[k][ii - 1][0] : 0.0);
        for (int jj = 0; jj < lb; ++jj)
          for (int ii = 0; ii <= la + 3; ++ii)
            S1[k][ii][jj + 1] = xpb * S1[k][ii][jj] +
                                o2p * ((ii > 0 ? ii * S1[k][ii - 1][jj] : 0.0) + (jj > 0 ? jj * S1[k][ii][jj - 1] : 0.0));
      }
      for (int ca = 0; ca < NCART[la]; ++ca)
        for (int cb = 0; cb < NCART[lb]; ++cb) {
          const int* ea = CPOW[la][ca];
          const int* eb = CPOW[lb][cb];
          /* f(e): product over k of S1[k][e_k][eb_k]; g(e,m): derivative wrt A_m */
#define PROD(e0, e1, e2) (S1[0][e0][eb[0]] * S1[1][e1][eb[1]] * S1[2][e2][eb[2]])
          int e[3] = {ea[0], ea[1], ea[2]};
          Sc[ca][cb] += cc * PROD(e[0], e[1], e[2]);
          for (int c = 0; c < 3; ++c) {
            int f[3] = {e[0], e[1], e[2]}; f[c]++;
            Dc[c][ca][cb] += cc * PROD(f[0], f[1], f[2]);
          }
          for (int q = 0; q < 6; ++q) {
            int f[3] = {e[0], e[1], e[2]}; f[QI[q][0]]++; f[QI[q][1]]++;
            Mc[q][ca][cb] += cc * PROD(f[0], f[1], f[2]);
          }
          if (deriv) {
            for (int m = 0; m < 3; ++m) {
              /* derivative of a product with bra powers f wrt A_m */
#define DPROD(f0, f1, f2, res)                                                              \
  do {                                                                                      \
    int ff[3] = {f0, f1, f2};                                                               \
    double t[3];                                                                            \
    for (int k = 0; k < 3; ++k) t[k] = S1[k][ff[k]][eb[k]];                                 \
    double dm = 2.0 * a * S1[m][ff[m] + 1][eb[m]] - (ff[m] > 0 ? ff[m] * S1[m][ff[m] - 1][eb[m]] : 0.0); \
    t[m] = dm;                                                                              \
    res = t[0] * t[1] * t[2];                                                               \
  } while (0)
              double v;
              DPROD(e[0], e[1], e[2], v);
              dSc[m][ca][cb] += cc * v;
              for (int c = 0; c < 3; ++c) {
                int f[3] = {e[0], e[1], e[2]}; f[c]++;
                DPROD(f[0], f[1], f[2], v);
                dDc[c][m][ca][cb] += cc * v;
              }
              for (int q = 0; q < 6; ++q) {
                int f[3] = {e[0], e[1], e[2]}; f[QI[q][0]]++; f[QI[q][1]]++;
                DPROD(f[0], f[1], f[2], v);
                dMc[q][m][ca][cb] += cc * v;
              }
#undef DPROD
            }
          }
#undef PROD
        }
    }
  /* transform both sides to spherical functions */
  int na = NSPH[la], nb = NSPH[lb];
#define TRANSFORM(src, dst)                                               \
  do {                                                                    \
    double tmp[6][5], col[6], res[5];                                     \
    for (int ca = 0; ca < NCART[la]; ++ca) {                              \
      for (int cb = 0; cb < NCART[lb]; ++cb) col[cb] = src[ca][cb];       \
      cart2sph(lb, col, res);                                             \
      for (int jb = 0; jb < nb; ++jb) tmp[ca][jb] = res[jb];              \
    }                                                                     \
    for (int jb = 0; jb < nb; ++jb) {                                     \
      for (int ca = 0; ca < NCART[la]; ++ca) col[ca] = tmp[ca][jb];       \
      cart2sph(la, col, res);                                             \
      for (int ia = 0; ia < na; ++ia) dst[ia][jb] = res[ia];              \
    }                                                                     \
  } while (0)
  TRANSFORM(Sc, out->S);
  for (int c = 0; c < 3; ++c) TRANSFORM(Dc[c], out->D[c]);
  double Ms[6][5][5];
  for (int q = 0; q < 6; ++q) TRANSFORM(Mc[q], Ms[q]);
  for (int ia = 0; ia < na; ++ia)
    for (int jb = 0; jb < nb; ++jb) {
      double tr = Ms[0][ia][jb] + Ms[1][ia][jb] + Ms[2][ia][jb];
      for (int q = 0; q < 3; ++q) out->Q[q][ia][jb] = 1.5 * Ms[q][ia][jb] - 0.5 * tr;
      for (int q = 3; q < 6; ++q) out->Q[q][ia][jb] = 1.5 * Ms[q][ia][jb];
    }
  if (deriv) {
    for (int m = 0; m < 3; ++m) {
      TRANSFORM(dSc[m], out->dS[m]);
      for (int c = 0; c < 3; ++c) TRANSFORM(dDc[c][m], out->dD[c][m]);
      double dMs[6][5][5];
      for (int q = 0; q < 6; ++q) TRANSFORM(dMc[q][m], dMs[q]);
      for (int ia = 0; ia < na; ++ia)
        for (int jb = 0; jb < nb; ++jb) {
          double tr = dMs[0][ia][jb] + dMs[1][ia][jb] + dMs[2][ia][jb];
          for (int q = 0; q < 3; ++q) out->dQ[q][m][ia][jb] = 1.5 * dMs[q][ia][jb] - 0.5 * tr;
          for (int q = 3; q < 6; ++q) out->dQ[q][m][ia][jb] = 1.5 * dMs[q][ia][jb];
        }
    }
  }
#undef TRANSFORM
}

/* ------------------------------------------------------------------------ */
/* H0 pieces                                                                  */
/* ------------------------------------------------------------------------ */
static double kpair(int l1, int l2) {
  if (l1 == 2 || l2 == 2) return QCX_K_XD;
  if (l1 == 0 && l2 == 0) return QCX_K_SS;
  if (l1 == 1 && l2 == 1) return QCX_K_PP;
  return QCX_K_SP;
}

static double selfenergy(int z, int k, double cn) { return qcx_sh_selfenergy[z][k] + qcx_sh_kcn[z][k] * cn; }

/* H0_{mu nu} = pref * Pi(R) * S_{mu nu}; returns pref*Pi and its R derivative,
 * plus the h-independent factor K*X*Y*Pi (for the CN chain rule). */
static void h0_factor(int za, int ka, int zb, int kb, double r, double hA, double hB, double* fac,
                      double* dfac, double* kxyp) {
  double zeta_a = qcx_sh_zeta[za][ka], zeta_b = qcx_sh_zeta[zb][kb];
  double y = sqrt(2.0 * sqrt(zeta_a * zeta_b) / (zeta_a + zeta_b));
  double den = qcx_en[za] - qcx_en[zb];
  double x = 1.0 + QCX_KEN * den * den;
  double rr = sqrt(r / (qcx_rcov[za] + qcx_rcov[zb]));
  double pa = 1.0 + qcx_sh_kpoly[za][ka] * rr, pb = 1.0 + qcx_sh_kpoly[zb][kb] * rr;
  double pi = pa * pb;
  double dpi = (qcx_sh_kpoly[za][ka] * pb + qcx_sh_kpoly[zb][kb] * pa) * 0.5 * rr / r;
  double k = kpair(qcx_sh_l[za][ka], qcx_sh_l[zb][kb]);
  double base = k * x * y;
  *fac = 0.5 * base * (hA + hB) * pi;
  *dfac = 0.5 * base * (hA + hB) * dpi;
  *kxyp = base * pi;
}

static void build_integrals(const mol_t* m, const double* cn, double* S, double* H0, double* Dm, double* Qm) {
  int n = m->nao;
  size_t nn = (size_t)n * n;
  memset(S, 0, sizeof(double) * nn);
  memset(H0, 0, sizeof(double) * nn);
  if (Dm) memset(Dm, 0, sizeof(double) * 3 * nn);
  if (Qm) memset(Qm, 0, sizeof(double) * 6 * nn);
  spair_t sp;
  for (int s = 0; s < m->nsh; ++s)
    for (int t = 0; t < m->nsh; ++t) {
      int A = m->sh_atom[s], B = m->sh_atom[t];
      int za = m->Z[A], zb = m->Z[B], ka = m->sh_k[s], kb = m->sh_k[t];
      double d[3], r = 0;
      for (int k = 0; k < 3; ++k) { d[k] = m->xyz[3 * A + k] - m->xyz[3 * B + k]; r += d[k] * d[k]; }
      r = sqrt(r);
      shell_pair(za, ka, zb, kb, d, 0, &sp);
      int a0 = m->sh_ao0[s], b0 = m->sh_ao0[t];
      for (int i = 0; i < m->sh_nao[s]; ++i)
        for (int j = 0; j < m->sh_nao[t]; ++j) {
          size_t ij = (size_t)(a0 + i) * n + (b0 + j);
          if (Dm) for (int c = 0; c < 3; ++c) Dm[c * nn + ij] = sp.D[c][i][j];
          if (Qm) for (int q = 0; q < 6; ++q) Qm[q * nn + ij] = sp.Q[q][i][j];
          if (s <= t) {
            size_t ji = (size_t)(b0 + j) * n + (a0 + i);
            S[ij] = sp.S[i][j]; S[ji] = sp.S[i][j];
          }
        }
      if (s <= t) {
        if (A == B) {
          if (s == t)
            for (int i = 0; i < m->sh_nao[s]; ++i)
              H0[(size_t)(a0 + i) * n + a0 + i] = selfenergy(za, ka, cn[A]);
        } else {
          double fac, dfac, kxyp;
          h0_factor(za, ka, zb, kb, r, selfenergy(za, ka, cn[A]), selfenergy(zb, kb, cn[B]), &fac, &dfac, &kxyp);
          for (int i = 0; i < m->sh_nao[s]; ++i)
            for (int j = 0; j < m->sh_nao[t]; ++j) {
              double v = fac * sp.S[i][j];
              H0[(size_t)(a0 + i) * n + b0 + j] = v;
              H0[(size_t)(b0 + j) * n + a0 + i] = v;
            }
        }
      }
    }
}

int qcxo_integrals(int nat, const int* Z, const double* xyz, double* S, double* H0, double* Dm, double* Qm,
                   double* cn, double* cnd) {
  mol_t m;
  if (mol_init(&m, nat, Z, xyz)) { mol_free(&m); return -1; }
  compute_cn(&m, cn, cnd);
  build_integrals(&m, cn, S, H0, Dm, Qm);
  mol_free(&m);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* dense linear algebra                                                      */
/* ------------------------------------------------------------------------ */
/* Householder tridiagonalisation followed by the implicit-shift QL iteration
 * (Golub & Van Loan, Matrix Computations, sections 8.3.1 and 8.3.3). */
int qcxo_syev(int n, double* A, double* w, double* V) {
  double* e = calloc(n + 1, sizeof(double));
  double* v = malloc(sizeof(double) * n);
  double* pv = malloc(sizeof(double) * n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) V[i * n + j] = (i == j) ? 1.0 : 0.0;
  /* reduce: A <- H A H for k = 0..n-3, V <- V H */
  for (int k = 0; k < n - 2; ++k) {
    double alpha = 0.0;
    for (int i = k + 1; i < n; ++i) alpha += A[i * n + k] * A[i * n + k];
    alpha = sqrt(alpha);
    if (alpha == 0.0) continue;
    double x0 = A[(k + 1) * n + k];
    if (x0 > 0) alpha = -alpha;
    /* v = x - alpha e1 */
    for (int i = 0; i < n; ++i) v[i] = 0.0;
    for (int i = k + 1; i < n; ++i) v[i] = A[i * n + k];
    v[k + 1] -= alpha;
    double vv = 0.0;
    for (int i = k + 1; i < n; ++i) vv += v[i] * v[i];
    if (vv == 0.0) continue;
    double beta = 2.0 / vv;
    /* p = beta A v ; wv = p - (beta/2 p.v) v ; A -= v wv^T + wv v^T */
    for (int i = k; i < n; ++i) {
      double s = 0.0;
      for (int j = k + 1; j < n; ++j) s += A[i * n + j] * v[j];
      pv[i] = beta * s;
    }
    double pvv = 0.0;
    for (int i = k + 1; i < n; ++i) pvv += pv[i] * v[i];
    double c = 0.5 * beta * pvv;
    for (int i = k; i < n; ++i) pv[i] -= (i > k ? c * v[i] : 0.0);
    for (int i = k; i < n; ++i)
      for (int j = k; j < n; ++j) A[i * n + j] -= v[i] * pv[j] + pv[i] * v[j];
    /* V <- V (I - beta v v^T) */
    for (int i = 0; i < n; ++i) {
      double s = 0.0;
      for (int j = k + 1; j < n; ++j) s += V[i * n + j] * v[j];
      s *= beta;
      for (int j = k + 1; j < n; ++j) V[i * n + j] -= s * v[j];
    }
  }
  for (int i = 0; i < n; ++i) w[i] = A[i * n + i];
  for (int i = 0; i < n - 1; ++i) e[i] = A[(i + 1) * n + i];
  e[n - 1] = 0.0;
  /* implicit QL on (w, e) */
  int status = 0;
  for (int l = 0; l < n; ++l) {
    int iter = 0, mm;
    do {
      for (mm = l; mm < n - 1; ++mm) {
        double dd = fabs(w[mm]) + fabs(w[mm + 1]);
        if (fabs(e[mm]) <= 1e-15 * dd) break;
      }
      if (mm != l) {
        if (++iter > 60) { status = 1; break; }
        double g = (w[l + 1] - w[l]) / (2.0 * e[l]);
        double r = hypot(g, 1.0);
        g = w[mm] - w[l] + e[l] / (g + (g >= 0 ? fabs(r) : -fabs(r)));
        double s = 1.0, c = 1.0, p = 0.0;
        int i;
        for (i = mm - 1; i >= l; --i) {
          double f = s * e[i], b = c * e[i];
          r = hypot(f, g);
          e[i + 1] = r;
          if (r == 0.0) { w[i + 1] -= p; e[mm] = 0.0; break; }
          s = f / r; c = g / r;
          g = w[i + 1] - p;
          r = (w[i] - g) * s + 2.0 * c * b;
          p = s * r;
          w[i + 1] = g + p;
          g = c * r - b;
          for (int k = 0; k < n; ++k) {
            double t = V[k * n + i + 1];
            V[k * n + i + 1] = s * V[k * n + i] + c * t;
            V[k * n + i] = c * V[k * n + i] - s * t;
          }
        }
        if (r == 0.0 && i >= l) continue;
        w[l] -= p; e[l] = g; e[mm] = 0.0;
      }
    } while (mm != l);
  }
  /* sort ascending */
  for (int i = 0; i < n - 1; ++i) {
    int k = i;
    for (int j = i + 1; j < n; ++j) if (w[j] < w[k]) k = j;
    if (k != i) {
      double t = w[i]; w[i] = w[k]; w[k] = t;
      for (int r = 0; r < n; ++r) { t = V[r * n + i]; V[r * n + i] = V[r * n + k]; V[r * n + k] = t; }
    }
  }
  free(e); free(v); free(pv);
  return status;
}

/* Cholesky S = L L^T (lower, row-major). Returns nonzero if not positive definite. */
static int cholesky(int n, const double* S, double* L) {
  memset(L, 0, sizeof(double) * n * n);
  for (int j = 0; j < n; ++j) {
    double s = S[j * n + j];
    for (int k = 0; k < j; ++k) s -= L[j * n + k] * L[j * n + k];
    if (s <= 0.0) return 1;
    double d = sqrt(s);
    L[j * n + j] = d;
    for (int i = j + 1; i < n; ++i) {
      double t = S[i * n + j];
      for (int k = 0; k < j; ++k) t -= L[i * n + k] * L[j * n + k];
      L[i * n + j] = t / d;
    }
  }
  return 0;
}

/* X = L^{-T} (upper triangular), so that X^T S X = I */
static void chol_inverse_t(int n, const double* L, double* X) {
  /* Linv lower: solve L Linv = I */
  double* Li = calloc((size_t)n * n, sizeof(double));
  for (int j = 0; j < n; ++j) {
    Li[j * n + j] = 1.0 / L[j * n + j];
    for (int i = j + 1; i < n; ++i) {
      double s = 0.0;
      for (int k = j; k < i; ++k) s -= L[i * n + k] * Li[k * n + j];
      Li[i * n + j] = s / L[i * n + i];
    }
  }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) X[i * n + j] = Li[j * n + i];
  free(Li);
}

/* ------------------------------------------------------------------------ */
/* Fermi smearing (spin-restricted, occupation 0..2 per MO)                   */
/* ------------------------------------------------------------------------ */
static double fermi_f(double e, double mu, double kT) { return 1.0 / (1.0 + exp((e - mu) / kT)); }

/* returns electronic entropy term -T*S (<= 0) and sets occupations */
static double fermi_occ(int n, const double* eps, double nel, double kT, double* focc, double* efermi) {
  if (nel <= 0.0) { for (int i = 0; i < n; ++i) focc[i] = 0.0; *efermi = eps[0]; return 0.0; }
  if (nel >= 2.0 * n) { for (int i = 0; i < n; ++i) focc[i] = 2.0; *efermi = eps[n - 1]; return 0.0; }
  int ho = (int)ceil(nel / 2.0) - 1;
  if (ho < 0) ho = 0;
  int lu = ho + 1 < n ? ho + 1 : n - 1;
  double lo = eps[0] - 1.0, hi = eps[n - 1] + 1.0;
  double mu = 0.5 * (eps[ho] + eps[lu]);
  for (int it = 0; it < QCX_FERMI_ITERS; ++it) {
    double N = 0.0, dN = 0.0;
    for (int i = 0; i < n; ++i) {
      double f = fermi_f(eps[i], mu, kT);
      N += 2.0 * f; dN += 2.0 * f * (1.0 - f) / kT;
    }
    double r = N - nel;
    if (fabs(r) < 1e-13 * (nel > 1.0 ? nel : 1.0)) break;
    if (r < 0) lo = mu; else hi = mu;
    double mn = (dN > 1e-300) ? mu - r / dN : 0.5 * (lo + hi);
    if (!(mn > lo && mn < hi)) mn = 0.5 * (lo + hi);
    mu = mn;
  }
  double ts = 0.0;
  for (int i = 0; i < n; ++i) {
    double x = (eps[i] - mu) / kT, ax = fabs(x);
    double fs = 1.0 / (1.0 + exp(ax));     /* occupation of the far side */
    double s = -(fs * ax + log1p(exp(-ax)));  /* f ln f + (1-f) ln(1-f) */
    focc[i] = 2.0 * fermi_f(eps[i], mu, kT);
    ts += 2.0 * kT * s;
  }
  *efermi = mu;
  return ts;
}

/* ------------------------------------------------------------------------ */
/* electrostatics / dispersion / repulsion (per geometry)                   */
/* ------------------------------------------------------------------------ */
typedef struct {
  int nat, nsh;
  double* gam;      /* [nsh][nsh] */
  double* mrad;     /* [nat] multipole radius */
  double* dmrad;    /* [nat] d mrad / d CN */
  double* c6;       /* [nat][nat] C6 at zero charge (CN weighted): the three-body term's */
  double* gdisp;    /* [nat][nat] BJ-damped kernel g_AB(R) */
  double* dgdisp;   /* [nat][nat] dg/dR */
  double* gw;       /* [nat][D4_MAXREF] reference weights at the covalent CN */
  double* dgw;      /* [nat][D4_MAXREF] d gw / d CN */
  double* z0;       /* [nat][D4_MAXREF] charge scaling of the references at zero charge */
  double* zq;       /* [nat][D4_MAXREF] charge scaling at the current atomic charges */
  double* dzq;      /* [nat][D4_MAXREF] d zq / d q */
} es_t;

static void es_alloc(es_t* e, int nat, int nsh) {
  e->nat = nat; e->nsh = nsh;
  e->gam = calloc((size_t)nsh * nsh, sizeof(double));
  e->mrad = calloc(nat, sizeof(double)); e->dmrad = calloc(nat, sizeof(double));
  e->c6 = calloc((size_t)nat * nat, sizeof(double));
  e->gdisp = calloc((size_t)nat * nat, sizeof(double)); e->dgdisp = calloc((size_t)nat * nat, sizeof(double));
  size_t nr = (size_t)nat * QCX_D4_MAXREF;
  e->gw = calloc(nr, sizeof(double)); e->dgw = calloc(nr, sizeof(double)); e->z0 = calloc(nr, sizeof(double));
  e->zq = calloc(nr, sizeof(double)); e->dzq = calloc(nr, sizeof(double));
}
static void es_free(es_t* e) {
  free(e->gam); free(e->mrad); free(e->dmrad); free(e->c6);
  free(e->gdisp); free(e->dgdisp); free(e->gw); free(e->dgw); free(e->z0); free(e->zq); free(e->dzq);
}

/* ------------------------------------------------------------------------ */
/* D4 dispersion model of QCxMS's src/dftd4.f90 with its reference data      */
/* (include/param_d4.fh, converted to qcx_d4ref.h)                            */
/* ------------------------------------------------------------------------ */
/* zeta / dzeta (src/dftd4.f90:423-450): charge scaling of a reference */
static double d4_zeta_fn(double a, double c, double qref, double qmod) {
  if (qmod < 0.0) return exp(a);
  return exp(a * (1.0 - exp(c * (1.0 - qref / qmod))));
}
static double d4_dzeta_fn(double a, double c, double qref, double qmod) {
  if (qmod < 0.0) return 0.0;
  return -a * c * exp(c * (1.0 - qref / qmod)) * d4_zeta_fn(a, c, qref, qmod) * qref / (qmod * qmod);
}

/* trapzd (src/dftd4.f90:452-497): Casimir-Polder integral over the 23
 * imaginary frequencies, the mean of the two staggered trapezoid sums */
static double d4_trapzd(const double* pol) {
  static const double freq[23] = {0.000001, 0.050000, 0.100000, 0.200000, 0.300000, 0.400000, 0.500000, 0.600000,
                                  0.700000, 0.800000, 0.900000, 1.000000, 1.200000, 1.400000, 1.600000, 1.800000,
                                  2.000000, 2.500000, 3.000000, 4.000000, 5.000000, 7.500000, 10.00000};
  double t1 = 0.0, t2 = 0.0;
  for (int k = 0; k < 22; k += 2) t1 = t1 + (freq[k + 1] - freq[k]) * (pol[k + 1] + pol[k]);
  for (int k = 1; k < 22; k += 2) t2 = t2 + (freq[k + 1] - freq[k]) * (pol[k + 1] + pol[k]);
  return 0.5 * t1 + 0.5 * t2;
}

static int d4_refc[QCX_MAXZ + 1][QCX_D4_MAXREF];                       /* Gaussians per reference */
static double d4_refal[QCX_MAXZ + 1][QCX_D4_MAXREF][QCX_D4_NFREQ];     /* reference alpha(i omega) */
static double d4_c6r[QCX_MAXZ + 1][QCX_MAXZ + 1][QCX_D4_MAXREF][QCX_D4_MAXREF];

/* d4dim (src/dftd4.f90:531-595): polarisabilities of the references with the
 * hydrogen (secondary system) contributions removed, and the number of
 * Gaussians of each reference; then C6 of every reference pair,
 * 3/pi * trapzd(alpha_i alpha_j) (src/dftd4.f90:665). Filled at load. */
__attribute__((constructor)) static void d4_tables(void) {
  const double thopi = 3.0 / 3.141592653589793238462643383279502884197;
  for (int z = 1; z <= QCX_MAXZ; ++z) {
    int cncount[16] = {0};
    cncount[0] = 1;
    for (int j = 0; j < qcx_d4_refn[z]; ++j) {
      int is = qcx_d4_refsys[z][j];
      double iz = (double)qcx_d4_zeff[is];
      double zs = d4_zeta_fn(QCX_D4_GA, qcx_d4_gam[is] * QCX_D4_GC, qcx_d4_secq[is] + iz, qcx_d4_refh[z][j] + iz);
      for (int k = 0; k < QCX_D4_NFREQ; ++k) {
        double sec_al = qcx_d4_sscale[is] * qcx_d4_secaiw[is][k] * zs;
        double v = qcx_d4_ascale[z][j] * (qcx_d4_alphaiw[z][j][k] - qcx_d4_hcount[z][j] * sec_al);
        d4_refal[z][j][k] = v > 0.0 ? v : 0.0;
      }
      cncount[(int)lround(qcx_d4_refcn[z][j])] += 1;
    }
    for (int j = 0; j < qcx_d4_refn[z]; ++j) {
      int icn = cncount[(int)lround(qcx_d4_refcn[z][j])];
      d4_refc[z][j] = icn * (icn + 1) / 2;
    }
  }
  for (int za = 1; za <= QCX_MAXZ; ++za)
    for (int zb = 1; zb <= QCX_MAXZ; ++zb)
      for (int i = 0; i < qcx_d4_refn[za]; ++i)
        for (int j = 0; j < qcx_d4_refn[zb]; ++j) {
          double pol[QCX_D4_NFREQ];
          for (int k = 0; k < QCX_D4_NFREQ; ++k) pol[k] = d4_refal[za][i][k] * d4_refal[zb][j][k];
          d4_c6r[za][zb][i][j] = thopi * d4_trapzd(pol);
        }
}

/* Reference weights of one atom at covalent CN cn (src/dftd4.f90:1150-1193):
 * gw_i = sum_{k<=refc_i} exp(-k wf (cn - cn_i)^2) / norm, and d gw / d cn;
 * a weight that overflows to NaN becomes 1 for the reference with the largest
 * CN and 0 otherwise (its derivative 0). */
static void d4_weights(int z, double cn, double* gw, double* dgw) {
  int nr = qcx_d4_refn[z];
  double norm = 0.0, dnorm = 0.0, maxcn = -1e300;
  for (int i = 0; i < nr; ++i) {
    if (qcx_d4_refcovcn[z][i] > maxcn) maxcn = qcx_d4_refcovcn[z][i];
    for (int k = 1; k <= d4_refc[z][i]; ++k) {
      double twf = k * QCX_D4_WF, d = cn - qcx_d4_refcovcn[z][i];
      double tgw = exp(-twf * d * d);
      norm = norm + tgw;
      dnorm = dnorm + 2 * twf * (qcx_d4_refcovcn[z][i] - cn) * tgw;
    }
  }
  norm = 1.0 / norm;
  for (int i = 0; i < QCX_D4_MAXREF; ++i) { gw[i] = 0.0; dgw[i] = 0.0; }
  for (int i = 0; i < nr; ++i) {
    double expw = 0.0, dexpw = 0.0;
    for (int k = 1; k <= d4_refc[z][i]; ++k) {
      double twf = QCX_D4_WF * k, d = cn - qcx_d4_refcovcn[z][i];
      double tgw = exp(-twf * d * d);
      expw = expw + tgw;
      dexpw = dexpw + 2 * twf * (qcx_d4_refcovcn[z][i] - cn) * tgw;
    }
    gw[i] = expw * norm;
    if (gw[i] != gw[i]) gw[i] = qcx_d4_refcovcn[z][i] == maxcn ? 1.0 : 0.0;
    dgw[i] = dexpw * norm - expw * dnorm * norm * norm;
    if (dgw[i] != dgw[i]) dgw[i] = 0.0;
  }
}

/* charge scaling of atom z's references at atomic charge q: zeta(g_a, gam*g_c,
 * refq_i + zeff, q + zeff) and its q derivative (src/dftd4.f90:1181-1190) */
static void d4_zeta_atom(int z, double q, double* zt, double* dzt) {
  double iz = (double)qcx_d4_zeff[z], c = qcx_d4_gam[z] * QCX_D4_GC;
  for (int i = 0; i < QCX_D4_MAXREF; ++i) {
    zt[i] = 0.0;
    if (dzt) dzt[i] = 0.0;
  }
  for (int i = 0; i < qcx_d4_refn[z]; ++i) {
    zt[i] = d4_zeta_fn(QCX_D4_GA, c, qcx_d4_refq[z][i] + iz, q + iz);
    if (dzt) dzt[i] = d4_dzeta_fn(QCX_D4_GA, c, qcx_d4_refq[z][i] + iz, q + iz);
  }
}

/* sum_ij (wa_i) (wb_j) C6(za, i, zb, j) */
static double d4_c6(int za, const double* wa, int zb, const double* wb) {
  double s = 0.0;
  for (int i = 0; i < qcx_d4_refn[za]; ++i)
    for (int j = 0; j < qcx_d4_refn[zb]; ++j) s += wa[i] * wb[j] * d4_c6r[za][zb][i][j];
  return s;
}

/* C6 of one reference pair (exported for the data tests) */
double qcxo_d4_c6ref(int za, int i, int zb, int j) {
  if (za < 1 || za > QCX_MAXZ || zb < 1 || zb > QCX_MAXZ || i < 0 || j < 0 || i >= qcx_d4_refn[za] ||
      j >= qcx_d4_refn[zb])
    return -1.0;
  return d4_c6r[za][zb][i][j];
}

/* molecular C6 of every atom pair at covalent CNs and charges q (zero charges
 * if q == NULL), c6 [nat][nat]; exported for the data tests */
void qcxo_d4_c6(int nat, const int* Z, const double* xyz, const double* q, double* c6) {
  double* w = calloc((size_t)nat * QCX_D4_MAXREF, sizeof(double));
  double gw[QCX_D4_MAXREF], dgw[QCX_D4_MAXREF], zt[QCX_D4_MAXREF];
  for (int a = 0; a < nat; ++a) {
    double cn = 0.0;
    for (int b = 0; b < nat; ++b) {
      if (b == a) continue;
      double r2 = 0.0, f, df;
      for (int k = 0; k < 3; ++k) { double d = xyz[3 * b + k] - xyz[3 * a + k]; r2 += d * d; }
      d4_cn_pair(Z[a], Z[b], r2, &f, &df);
      cn += f;
    }
    d4_weights(Z[a], cn, gw, dgw);
    d4_zeta_atom(Z[a], q ? q[a] : 0.0, zt, NULL);
    for (int i = 0; i < QCX_D4_MAXREF; ++i) w[a * QCX_D4_MAXREF + i] = gw[i] * zt[i];
  }
  for (int a = 0; a < nat; ++a)
    for (int b = 0; b < nat; ++b)
      c6[a * nat + b] = a == b ? 0.0 : d4_c6(Z[a], w + a * QCX_D4_MAXREF, Z[b], w + b * QCX_D4_MAXREF);
  free(w);
}

/* Becke-Johnson kernel of a pair (src/dftd4.f90:386-409, 1250-1258):
 * g = s6 / (r^6 + R0^6) + s8 * 3 r4r2_a r4r2_b / (r^8 + R0^8), R0 = a1 sqrt(3 r4r2_a r4r2_b) + a2 */
static void bj_kernel(int za, int zb, double r, double* g, double* dg) {
  double qq = 3.0 * qcx_d4_r4r2[za] * qcx_d4_r4r2[zb];
  double r0 = QCX_D4_A1 * sqrt(qq) + QCX_D4_A2;
  double r2 = r * r, r6 = r2 * r2 * r2, r8 = r6 * r2;
  double r06 = pow(r0, 6), r08 = r06 * r0 * r0;
  double t6 = 1.0 / (r6 + r06), t8 = 1.0 / (r8 + r08);
  *g = QCX_D4_S6 * t6 + QCX_D4_S8 * qq * t8;
  *dg = -QCX_D4_S6 * 6.0 * r * r2 * r2 * t6 * t6 - QCX_D4_S8 * qq * 8.0 * r6 * r * t8 * t8;
}

static double bj_radius(int za, int zb) {
  return QCX_D4_A1 * sqrt(3.0 * qcx_d4_r4r2[za] * qcx_d4_r4r2[zb]) + QCX_D4_A2;
}

static void mpole_radius(int z, double cn, double* r, double* dr) {
  double r0 = qcx_aes_rad0[z];
  double t = exp(-QCX_AES_KMP * (cn - qcx_aes_valcn[z] - QCX_AES_SHIFT));
  double s = 1.0 / (1.0 + t);
  *r = r0 + (QCX_AES_RMAX - r0) * s;
  *dr = (QCX_AES_RMAX - r0) * s * s * t * QCX_AES_KMP;
}

/* damped multipole kernel f_n(R) = 1/(R^n (1 + 6 (R0/R)^a)) and derivatives */
static void mp_kernel(int n, double a, double r, double r0, double* f, double* dfr, double* dfr0) {
  double t = 6.0 * pow(r0 / r, a);
  double fd = 1.0 / (1.0 + t);
  double rn = pow(r, n);
  *f = fd / rn;
  double dfd_r = a * t / (r * (1.0 + t) * (1.0 + t));
  double dfd_r0 = -a * t / (r0 * (1.0 + t) * (1.0 + t));
  *dfr = dfd_r / rn - n * fd / (rn * r);
  *dfr0 = dfd_r0 / rn;
}

static void es_setup(const mol_t* m, const double* cn, const double* cnd, es_t* e) {
  int nat = m->nat, nsh = m->nsh;
  for (int s = 0; s < nsh; ++s)
    for (int t = 0; t < nsh; ++t) {
      int A = m->sh_atom[s], B = m->sh_atom[t];
      double ea = qcx_sh_hardness[m->Z[A]][m->sh_k[s]], eb = qcx_sh_hardness[m->Z[B]][m->sh_k[t]];
      double eta = 0.5 * (ea + eb), r2 = 0;
      for (int k = 0; k < 3; ++k) { double d = m->xyz[3 * A + k] - m->xyz[3 * B + k]; r2 += d * d; }
      e->gam[s * nsh + t] = 1.0 / sqrt(r2 + 1.0 / (eta * eta));
    }
  double w0[QCX_D4_MAXREF * 2];
  double* wz = calloc((size_t)nat * QCX_D4_MAXREF, sizeof(double)); /* gw * z0 */
  for (int a = 0; a < nat; ++a) {
    mpole_radius(m->Z[a], cn[a], &e->mrad[a], &e->dmrad[a]);
    d4_weights(m->Z[a], cnd[a], &e->gw[a * QCX_D4_MAXREF], &e->dgw[a * QCX_D4_MAXREF]);
    d4_zeta_atom(m->Z[a], 0.0, &e->z0[a * QCX_D4_MAXREF], w0);
    for (int i = 0; i < QCX_D4_MAXREF; ++i)
      wz[a * QCX_D4_MAXREF + i] = e->gw[a * QCX_D4_MAXREF + i] * e->z0[a * QCX_D4_MAXREF + i];
  }
  for (int a = 0; a < nat; ++a)
    for (int b = 0; b < nat; ++b) {
      int za = m->Z[a], zb = m->Z[b];
      e->c6[a * nat + b] = d4_c6(za, wz + a * QCX_D4_MAXREF, zb, wz + b * QCX_D4_MAXREF);
      if (a != b) {
        double r2 = 0;
        for (int k = 0; k < 3; ++k) { double d = m->xyz[3 * a + k] - m->xyz[3 * b + k]; r2 += d * d; }
        bj_kernel(za, zb, sqrt(r2), &e->gdisp[a * nat + b], &e->dgdisp[a * nat + b]);
      }
    }
  free(wz);
}

/* moment vector layout: [qsh (nsh) | dipm (3 nat) | qp (6 nat)] */
typedef struct {
  double e_ies, e_3, e_aes, e_axc, e_disp;
} es_energy_t;

/* Potentials and energies for given moments. vsh [nsh], vdp [3 nat], vqp [6 nat] */
static void es_potential(const mol_t* m, es_t* e, const double* x, double* vsh, double* vdp, double* vqp,
                         es_energy_t* en) {
  int nat = m->nat, nsh = m->nsh;
  const double* qsh = x;
  const double* dp = x + nsh;
  const double* qp = x + nsh + 3 * nat;
  double* qat = calloc(nat, sizeof(double));
  double* vat = calloc(nat, sizeof(double));
  for (int s = 0; s < nsh; ++s) qat[m->sh_atom[s]] += qsh[s];
  memset(vdp, 0, sizeof(double) * 3 * nat);
  memset(vqp, 0, sizeof(double) * 6 * nat);
  double eies = 0.0, e3 = 0.0, eaes = 0.0, eaxc = 0.0, edisp = 0.0;
  for (int s = 0; s < nsh; ++s) {
    double v = 0.0;
    for (int t = 0; t < nsh; ++t) v += e->gam[s * nsh + t] * qsh[t];
    eies += 0.5 * qsh[s] * v;
    int A = m->sh_atom[s];
    double g3 = qcx_sh_gamma3[m->Z[A]][m->sh_k[s]];
    e3 += g3 * qsh[s] * qsh[s] * qsh[s] / 3.0;
    vsh[s] = v + g3 * qsh[s] * qsh[s];
  }
  /* anisotropic electrostatics (pairs A<B) */
  for (int a = 0; a < nat; ++a)
    for (int b = 0; b < a; ++b) {
      double r[3], r2 = 0;
      for (int k = 0; k < 3; ++k) { r[k] = m->xyz[3 * a + k] - m->xyz[3 * b + k]; r2 += r[k] * r[k]; }
      double R = sqrt(r2), r0 = 0.5 * (e->mrad[a] + e->mrad[b]);
      double f3, f5, d1, d2;
      mp_kernel(3, QCX_AES_A3, R, r0, &f3, &d1, &d2);
      mp_kernel(5, QCX_AES_A5, R, r0, &f5, &d1, &d2);
      const double* ma = dp + 3 * a; const double* mb = dp + 3 * b;
      const double* ta = qp + 6 * a; const double* tb = qp + 6 * b;
      double mar = ma[0] * r[0] + ma[1] * r[1] + ma[2] * r[2];
      double mbr = mb[0] * r[0] + mb[1] * r[1] + mb[2] * r[2];
      double mab = ma[0] * mb[0] + ma[1] * mb[1] + ma[2] * mb[2];
      double rr[6] = {r[0] * r[0], r[1] * r[1], r[2] * r[2], 2 * r[0] * r[1], 2 * r[0] * r[2], 2 * r[1] * r[2]};
      double rta = 0, rtb = 0;
      for (int q = 0; q < 6; ++q) { rta += ta[q] * rr[q]; rtb += tb[q] * rr[q]; }
      eaes += f3 * (qat[a] * mbr - qat[b] * mar) + f5 * (qat[a] * rtb + qat[b] * rta + mab * r2 - 3.0 * mar * mbr);
      vat[a] += f3 * mbr + f5 * rtb;
      vat[b] += -f3 * mar + f5 * rta;
      for (int k = 0; k < 3; ++k) {
        vdp[3 * a + k] += -f3 * qat[b] * r[k] + f5 * (mb[k] * r2 - 3.0 * mbr * r[k]);
        vdp[3 * b + k] += f3 * qat[a] * r[k] + f5 * (ma[k] * r2 - 3.0 * mar * r[k]);
      }
      for (int q = 0; q < 6; ++q) { vqp[6 * a + q] += f5 * qat[b] * rr[q]; vqp[6 * b + q] += f5 * qat[a] * rr[q]; }
    }
  /* multipole exchange-correlation kernels */
  for (int a = 0; a < nat; ++a) {
    int z = m->Z[a];
    const double* ma = dp + 3 * a; const double* ta = qp + 6 * a;
    double fd = qcx_aes_dkernel[z], fq = qcx_aes_qkernel[z];
    eaxc += fd * (ma[0] * ma[0] + ma[1] * ma[1] + ma[2] * ma[2]);
    eaxc += fq * (ta[0] * ta[0] + ta[1] * ta[1] + ta[2] * ta[2] + 2.0 * (ta[3] * ta[3] + ta[4] * ta[4] + ta[5] * ta[5]));
    for (int k = 0; k < 3; ++k) vdp[3 * a + k] += 2.0 * fd * ma[k];
    for (int q = 0; q < 3; ++q) vqp[6 * a + q] += 2.0 * fq * ta[q];
    for (int q = 3; q < 6; ++q) vqp[6 * a + q] += 4.0 * fq * ta[q];
  }
  /* self-consistent dispersion (edisp / disppot, src/dftd4.f90:807-1034):
   * E = -sum_{A<B} g_AB sum_ij (gw zeta(q_A))_i (gw zeta(q_B))_j C6_ij, and its
   * derivative with respect to the atomic charges as potential */
  {
    const int R = QCX_D4_MAXREF;
    double* wq = calloc((size_t)nat * R, sizeof(double));
    double* dwq = calloc((size_t)nat * R, sizeof(double));
    for (int a = 0; a < nat; ++a) {
      d4_zeta_atom(m->Z[a], qat[a], &e->zq[a * R], &e->dzq[a * R]);
      for (int i = 0; i < R; ++i) {
        wq[a * R + i] = e->gw[a * R + i] * e->zq[a * R + i];
        dwq[a * R + i] = e->gw[a * R + i] * e->dzq[a * R + i];
      }
    }
    for (int a = 0; a < nat; ++a) {
      double v = 0.0;
      for (int b = 0; b < nat; ++b) {
        if (b == a) continue;
        double g = e->gdisp[a * nat + b];
        v -= g * d4_c6(m->Z[a], dwq + a * R, m->Z[b], wq + b * R);
        if (b < a) edisp -= g * d4_c6(m->Z[a], wq + a * R, m->Z[b], wq + b * R);
      }
      vat[a] += v;
    }
    free(wq); free(dwq);
  }
  for (int s = 0; s < nsh; ++s) vsh[s] += vat[m->sh_atom[s]];
  en->e_ies = eies; en->e_3 = e3; en->e_aes = eaes; en->e_axc = eaxc; en->e_disp = edisp;
  free(qat); free(vat);
}

static double rep_energy_grad(const mol_t* m, double* grad) {
  double e = 0.0;
  for (int a = 0; a < m->nat; ++a)
    for (int b = 0; b < a; ++b) {
      int za = m->Z[a], zb = m->Z[b];
      double r[3], r2 = 0;
      for (int k = 0; k < 3; ++k) { r[k] = m->xyz[3 * a + k] - m->xyz[3 * b + k]; r2 += r[k] * r[k]; }
      double R = sqrt(r2);
      double al = sqrt(qcx_rep_alpha[za] * qcx_rep_alpha[zb]);
      double rk = pow(R, QCX_REP_KEXP);
      double v = qcx_rep_zeff[za] * qcx_rep_zeff[zb] / R * exp(-al * rk);
      e += v;
      if (grad) {
        double dv = v * (-1.0 / R - QCX_REP_KEXP * al * rk / R);
        for (int k = 0; k < 3; ++k) { grad[3 * a + k] += dv * r[k] / R; grad[3 * b + k] -= dv * r[k] / R; }
      }
    }
  return e;
}

/* Axilrod-Teller-Muto three-body term with zero-charge C6 (CN dependent),
 * as apprabc / dabcappr (src/dftd4.f90:1339-1400, 1610-1780) with the zero-charge
 * weights of dispgrad (src/dftd4.f90:1181-1190): C9 = s9 sqrt(C6_ab C6_bc C6_ca),
 * damping 1 / (1 + 6 ((R0_ab R0_bc R0_ca / (r_ab r_bc r_ca))^(1/3))^alp).
 * Adds dE/dCN' to dedcnd when grad != NULL. */
static double atm_energy_grad(const mol_t* m, const es_t* e, double* grad, double* dedcnd) {
  int nat = m->nat;
  double etot = 0.0;
  for (int a = 0; a < nat; ++a)
    for (int b = 0; b < a; ++b)
      for (int c = 0; c < b; ++c) {
        int za = m->Z[a], zb = m->Z[b], zc = m->Z[c];
        double rab[3], rbc[3], rca[3], ab2 = 0, bc2 = 0, ca2 = 0;
        for (int k = 0; k < 3; ++k) {
          rab[k] = m->xyz[3 * a + k] - m->xyz[3 * b + k];
          rbc[k] = m->xyz[3 * b + k] - m->xyz[3 * c + k];
          rca[k] = m->xyz[3 * c + k] - m->xyz[3 * a + k];
          ab2 += rab[k] * rab[k]; bc2 += rbc[k] * rbc[k]; ca2 += rca[k] * rca[k];
        }
        double c6ab = e->c6[a * nat + b], c6bc = e->c6[b * nat + c], c6ca = e->c6[c * nat + a];
        double c9 = QCX_D4_S9 * sqrt(c6ab * c6bc * c6ca);
        double r0 = cbrt(bj_radius(za, zb) * bj_radius(zb, zc) * bj_radius(zc, za));
        double rab_ = sqrt(ab2), rbc_ = sqrt(bc2), rca_ = sqrt(ca2);
        double rrr = rab_ * rbc_ * rca_;
        double rbar = cbrt(rrr);
        double t = 6.0 * pow(r0 / rbar, QCX_ATM_ALP);
        double fd = 1.0 / (1.0 + t);
        /* angular factor in distances: 3 cos a cos b cos c + 1 */
        double num = (ab2 + ca2 - bc2) * (ab2 + bc2 - ca2) * (bc2 + ca2 - ab2);
        double ang = 3.0 * num / (8.0 * ab2 * bc2 * ca2) + 1.0;
        double r3 = rrr * rrr * rrr;
        double en = c9 * ang * fd / r3;
        etot += en;
        if (grad) {
          /* derivatives wrt squared distances x=ab2, y=bc2, z=ca2 */
          double x = ab2, y = bc2, z = ca2;
          double u1 = x + z - y, u2 = x + y - z, u3 = y + z - x;
          double dnum_dx = u2 * u3 + u1 * u3 - u1 * u2;
          double dnum_dy = -u2 * u3 + u1 * u3 + u1 * u2;
          double dnum_dz = u2 * u3 - u1 * u3 + u1 * u2;
          double den = 8.0 * x * y * z;
          double dang_dx = 3.0 * (dnum_dx / den - num / (den * x));
          double dang_dy = 3.0 * (dnum_dy / den - num / (den * y));
          double dang_dz = 3.0 * (dnum_dz / den - num / (den * z));
          /* radial part h = fd / rrr^3 with rrr^2 = x y z; d/dx of ln(rrr) = 1/(2x) */
          double alp3 = QCX_ATM_ALP;
          /* d fd / d ln(rbar) = fd^2 * t * alp3 ; d ln rbar / d x = 1/(6x) */
          double dlnh_dlnr = (fd * t * alp3) - 9.0; /* d ln(h)/d ln(rbar) */
          double dh_dx = fd / r3 * dlnh_dlnr / (6.0 * x);
          double dh_dy = fd / r3 * dlnh_dlnr / (6.0 * y);
          double dh_dz = fd / r3 * dlnh_dlnr / (6.0 * z);
          double h = fd / r3;
          double ex = c9 * (dang_dx * h + ang * dh_dx);
          double ey = c9 * (dang_dy * h + ang * dh_dy);
          double ez = c9 * (dang_dz * h + ang * dh_dz);
          for (int k = 0; k < 3; ++k) {
            double gx = 2.0 * ex * rab[k], gy = 2.0 * ey * rbc[k], gz = 2.0 * ez * rca[k];
            grad[3 * a + k] += gx - gz;
            grad[3 * b + k] += -gx + gy;
            grad[3 * c + k] += -gy + gz;
          }
          /* CN' dependence through the three C6 */
          double ec = en; /* en = c9 * ang * h, c9 ~ sqrt(c6ab c6bc c6ca) */
          int atoms[3] = {a, b, c};
          for (int ii = 0; ii < 3; ++ii) {
            int p = atoms[ii];
            int zp = m->Z[p];
            double dsum = 0.0;
            for (int jj = 0; jj < 3; ++jj) {
              if (jj == ii) continue;
              int o = atoms[jj], zo = m->Z[o];
              double c6po = e->c6[p * nat + o];
              const int R = QCX_D4_MAXREF;
              double wp[QCX_D4_MAXREF], wo[QCX_D4_MAXREF];
              for (int i = 0; i < R; ++i) {
                wp[i] = e->dgw[p * R + i] * e->z0[p * R + i];
                wo[i] = e->gw[o * R + i] * e->z0[o * R + i];
              }
              double dc6 = d4_c6(zp, wp, zo, wo);
              dsum += 0.5 * dc6 / c6po;
            }
            dedcnd[p] += ec * dsum;
          }
        }
      }
  return etot;
}

/* ------------------------------------------------------------------------ */
/* modified Broyden mixing (D. D. Johnson, PRB 38, 12807 (1988)) over a      */
/* sliding window of the last QCX_BROYDEN_WINDOW iterations                   */
/* ------------------------------------------------------------------------ */
typedef struct {
  int len, maxit, it;
  double alpha;
  double *df, *u, *a, *xlast, *flast;
} broyden_t;

static void broyden_init(broyden_t* b, int len, int maxit, double alpha) {
  b->len = len; b->maxit = maxit; b->it = 0; b->alpha = alpha;
  b->df = calloc((size_t)len * maxit, sizeof(double));
  b->u = calloc((size_t)len * maxit, sizeof(double));
  b->a = calloc((size_t)maxit * maxit, sizeof(double));
  b->xlast = calloc(len, sizeof(double));
  b->flast = calloc(len, sizeof(double));
}
static void broyden_free(broyden_t* b) { free(b->df); free(b->u); free(b->a); free(b->xlast); free(b->flast); }

/* small dense solve (Gaussian elimination with partial pivoting), in place */
static void solve_small(int n, double* M, double* rhs) {
  for (int k = 0; k < n; ++k) {
    int p = k;
    for (int i = k + 1; i < n; ++i) if (fabs(M[i * n + k]) > fabs(M[p * n + k])) p = i;
    if (p != k) {
      for (int j = 0; j < n; ++j) { double t = M[k * n + j]; M[k * n + j] = M[p * n + j]; M[p * n + j] = t; }
      double t = rhs[k]; rhs[k] = rhs[p]; rhs[p] = t;
    }
    for (int i = k + 1; i < n; ++i) {
      double f = M[i * n + k] / M[k * n + k];
      for (int j = k; j < n; ++j) M[i * n + j] -= f * M[k * n + j];
      rhs[i] -= f * rhs[k];
    }
  }
  for (int k = n - 1; k >= 0; --k) {
    double s = rhs[k];
    for (int j = k + 1; j < n; ++j) s -= M[k * n + j] * rhs[j];
    rhs[k] = s / M[k * n + k];
  }
}

/* x_in (updated in place) and x_out -> next input */
static void broyden_step(broyden_t* b, double* x, const double* xout) {
  int len = b->len;
  double* f = malloc(sizeof(double) * len);
  for (int i = 0; i < len; ++i) f[i] = xout[i] - x[i];
  int it = b->it;
  if (it == 0) {
    for (int i = 0; i < len; ++i) { b->xlast[i] = x[i]; b->flast[i] = f[i]; x[i] += b->alpha * f[i]; }
  } else {
    int m = (it - 1) % b->maxit; /* history slot (sliding window of maxit entries) */
    int k = it < b->maxit ? it : b->maxit; /* valid slots */
    double* dfm = b->df + (size_t)m * len;
    double* um = b->u + (size_t)m * len;
    double nrm = 0.0;
    for (int i = 0; i < len; ++i) { dfm[i] = f[i] - b->flast[i]; nrm += dfm[i] * dfm[i]; }
    nrm = sqrt(nrm);
    if (nrm < 1e-300) nrm = 1e-300;
    for (int i = 0; i < len; ++i) {
      dfm[i] /= nrm;
      um[i] = b->alpha * dfm[i] + (x[i] - b->xlast[i]) / nrm;
    }
    for (int j = 0; j < k; ++j) {
      double s = 0.0;
      const double* dfj = b->df + (size_t)j * len;
      for (int i = 0; i < len; ++i) s += dfj[i] * dfm[i];
      b->a[j * b->maxit + m] = s; b->a[m * b->maxit + j] = s;
    }
    double* M = malloc(sizeof(double) * k * k);
    double* c = malloc(sizeof(double) * k);
    for (int i = 0; i < k; ++i) {
      for (int j = 0; j < k; ++j) M[i * k + j] = b->a[i * b->maxit + j];
      M[i * k + i] += QCX_BROYDEN_W0 * QCX_BROYDEN_W0;
      double s = 0.0;
      const double* dfi = b->df + (size_t)i * len;
      for (int l = 0; l < len; ++l) s += dfi[l] * f[l];
      c[i] = s;
    }
    solve_small(k, M, c); /* gamma = (w0^2 + a)^{-1} c */
    for (int i = 0; i < len; ++i) { b->xlast[i] = x[i]; b->flast[i] = f[i]; }
    for (int i = 0; i < len; ++i) {
      double s = 0.0;
      for (int j = 0; j < k; ++j) s += c[j] * b->u[(size_t)j * len + i];
      x[i] += b->alpha * f[i] - s;
    }
    free(M); free(c);
  }
  b->it++;
  free(f);
}

/* ------------------------------------------------------------------------ */
/* SCC                                                                         */
/* ------------------------------------------------------------------------ */
typedef struct {
  mol_t m;
  double *cn, *cnd, *S, *H0, *Dm, *Qm, *X;
  double *P, *W, *eps, *focc, *x_out, *vsh, *vdp, *vqp;
  double* C; /* MO coefficients of the last iteration, C[i*n + k]: AO i, orbital k by energy */
  es_t es;
  es_energy_t esen;
  double e_band, e_ts, e_elec, efermi;
  int iterations, converged;
  double nel;
} scc_t;

static void scc_free(scc_t* c) {
  free(c->cn); free(c->cnd); free(c->S); free(c->H0); free(c->Dm); free(c->Qm); free(c->X);
  free(c->P); free(c->W); free(c->eps); free(c->focc); free(c->x_out); free(c->vsh); free(c->vdp); free(c->vqp);
  free(c->C);
  es_free(&c->es);
  mol_free(&c->m);
}

/* output moments from density */
static void moments(const mol_t* m, const double* P, const double* S, const double* Dm, const double* Qm, double* x) {
  int n = m->nao, nsh = m->nsh, nat = m->nat;
  size_t nn = (size_t)n * n;
  double* qsh = x; double* dp = x + nsh; double* qp = x + nsh + 3 * nat;
  for (int s = 0; s < nsh; ++s) qsh[s] = qcx_sh_refocc[m->Z[m->sh_atom[s]]][m->sh_k[s]];
  memset(dp, 0, sizeof(double) * 3 * nat);
  memset(qp, 0, sizeof(double) * 6 * nat);
  for (int mu = 0; mu < n; ++mu) {
    int s = m->ao_sh[mu], A = m->ao_atom[mu];
    double pop = 0.0, d[3] = {0, 0, 0}, q[6] = {0, 0, 0, 0, 0, 0};
    for (int nu = 0; nu < n; ++nu) {
      double p = P[(size_t)mu * n + nu];
      pop += p * S[(size_t)mu * n + nu];
      for (int c = 0; c < 3; ++c) d[c] += p * Dm[c * nn + (size_t)mu * n + nu];
      for (int c = 0; c < 6; ++c) q[c] += p * Qm[c * nn + (size_t)mu * n + nu];
    }
    qsh[s] -= pop;
    for (int c = 0; c < 3; ++c) dp[3 * A + c] -= d[c];
    for (int c = 0; c < 6; ++c) qp[6 * A + c] -= q[c];
  }
}

static void build_fock(const mol_t* m, const double* H0, const double* S, const double* Dm, const double* Qm,
                       const double* vsh, const double* vdp, const double* vqp, double* F) {
  int n = m->nao;
  size_t nn = (size_t)n * n;
  for (int mu = 0; mu < n; ++mu)
    for (int nu = 0; nu < n; ++nu) {
      int A = m->ao_atom[mu], B = m->ao_atom[nu];
      size_t ij = (size_t)mu * n + nu, ji = (size_t)nu * n + mu;
      double f = H0[ij] - 0.5 * S[ij] * (vsh[m->ao_sh[mu]] + vsh[m->ao_sh[nu]]);
      for (int c = 0; c < 3; ++c) f -= 0.5 * (vdp[3 * A + c] * Dm[c * nn + ij] + vdp[3 * B + c] * Dm[c * nn + ji]);
      for (int c = 0; c < 6; ++c) f -= 0.5 * (vqp[6 * A + c] * Qm[c * nn + ij] + vqp[6 * B + c] * Qm[c * nn + ji]);
      F[ij] = f;
    }
}

static int run_scc(int nat, const int* Z, const double* xyz, double charge, double kT, const qcxo_opts* o, scc_t* c) {
  memset(c, 0, sizeof(*c));
  if (mol_init(&c->m, nat, Z, xyz)) return -1;
  mol_t* m = &c->m;
  int n = m->nao, nsh = m->nsh;
  size_t nn = (size_t)n * n;
  int len = nsh + 9 * nat;
  c->cn = calloc(nat, sizeof(double)); c->cnd = calloc(nat, sizeof(double));
  c->S = malloc(sizeof(double) * nn); c->H0 = malloc(sizeof(double) * nn);
  c->Dm = malloc(sizeof(double) * 3 * nn); c->Qm = malloc(sizeof(double) * 6 * nn);
  c->X = malloc(sizeof(double) * nn);
  c->P = calloc(nn, sizeof(double)); c->W = calloc(nn, sizeof(double));
  c->eps = calloc(n, sizeof(double)); c->focc = calloc(n, sizeof(double));
  c->x_out = calloc(len, sizeof(double));
  c->vsh = calloc(nsh, sizeof(double)); c->vdp = calloc(3 * nat, sizeof(double)); c->vqp = calloc(6 * nat, sizeof(double));
  es_alloc(&c->es, nat, nsh);
  compute_cn(m, c->cn, c->cnd);
  build_integrals(m, c->cn, c->S, c->H0, c->Dm, c->Qm);
  es_setup(m, c->cn, c->cnd, &c->es);
  double nel = -charge;
  for (int s = 0; s < nsh; ++s) nel += qcx_sh_refocc[Z[m->sh_atom[s]]][m->sh_k[s]];
  c->nel = nel;
  {
    double* L = malloc(sizeof(double) * nn);
    if (cholesky(n, c->S, L)) { free(L); return -2; }
    chol_inverse_t(n, L, c->X);
    free(L);
  }
  double* x = calloc(len, sizeof(double));
  double* F = malloc(sizeof(double) * nn);
  double* T = malloc(sizeof(double) * nn);
  double* A = malloc(sizeof(double) * nn);
  double* V = malloc(sizeof(double) * nn);
  double* C = malloc(sizeof(double) * nn);
  broyden_t br;
  broyden_init(&br, len, QCX_BROYDEN_WINDOW, o->broyden_alpha);
  double eprev = 0.0;
  double rbest = 1e300; /* best residual since the mixer's last restart */
  int rsince = 0;       /* iterations without a 10 % improvement of it */
  c->converged = 0;
  int it;
  for (it = 1; it <= o->max_iter; ++it) {
    es_energy_t dummy;
    es_potential(m, &c->es, x, c->vsh, c->vdp, c->vqp, &dummy);
    build_fock(m, c->H0, c->S, c->Dm, c->Qm, c->vsh, c->vdp, c->vqp, F);
    /* A = X^T F X */
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        double s = 0.0;
        for (int k = 0; k < n; ++k) s += F[i * n + k] * c->X[k * n + j];
        T[i * n + j] = s;
      }
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        double s = 0.0;
        for (int k = 0; k < n; ++k) s += c->X[k * n + i] * T[k * n + j];
        A[i * n + j] = s;
      }
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < i; ++j) { double s = 0.5 * (A[i * n + j] + A[j * n + i]); A[i * n + j] = s; A[j * n + i] = s; }
    qcxo_syev(n, A, c->eps, V);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        double s = 0.0;
        for (int k = 0; k < n; ++k) s += c->X[i * n + k] * V[k * n + j];
        C[i * n + j] = s;
      }
    c->e_ts = fermi_occ(n, c->eps, nel, kT, c->focc, &c->efermi);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j <= i; ++j) {
        double p = 0.0, w = 0.0;
        for (int k = 0; k < n; ++k) {
          double t = c->focc[k] * C[i * n + k] * C[j * n + k];
          p += t; w += t * c->eps[k];
        }
        c->P[i * n + j] = p; c->P[j * n + i] = p;
        c->W[i * n + j] = w; c->W[j * n + i] = w;
      }
    moments(m, c->P, c->S, c->Dm, c->Qm, c->x_out);
    es_potential(m, &c->es, c->x_out, c->vsh, c->vdp, c->vqp, &c->esen);
    double eb = 0.0;
    for (size_t k = 0; k < nn; ++k) eb += c->P[k] * c->H0[k];
    c->e_band = eb;
    double eel = eb + c->esen.e_ies + c->esen.e_3 + c->esen.e_aes + c->esen.e_axc + c->esen.e_disp + c->e_ts;
    double res = 0.0;
    for (int i = 0; i < len; ++i) { double d = c->x_out[i] - x[i]; res += d * d; }
    res = sqrt(res / len);
    double de = fabs(eel - eprev);
    eprev = eel;
    c->e_elec = eel;
    if (it > 1 && de < o->econv && res < o->pconv) { c->converged = 1; break; }
    if (it == o->max_iter) break;
    /* restart the mixer after QCX_BROYDEN_RESTART iterations of stagnation */
    if (res < 0.9 * rbest) {
      rbest = res;
      rsince = 0;
    } else if (++rsince >= QCX_BROYDEN_RESTART) {
      br.it = 0;
      rbest = res;
      rsince = 0;
    }
    broyden_step(&br, x, c->x_out);
  }
  c->iterations = it > o->max_iter ? o->max_iter : it;
  broyden_free(&br);
  free(x); free(F); free(T); free(A); free(V);
  c->C = C;
  return 0;
}

int qcxo_scc(int nat, const int* Z, const double* xyz, double charge, double kT, const qcxo_opts* opts, double* P,
             double* qsh, double* dipm, double* qp, double* eps, double* focc, qcxo_info* info) {
  qcxo_opts o;
  if (opts) o = *opts; else qcxo_default_opts(&o);
  scc_t c;
  int rc = run_scc(nat, Z, xyz, charge, kT, &o, &c);
  if (rc) { scc_free(&c); return -1; }
  int n = c.m.nao, nsh = c.m.nsh;
  if (P) memcpy(P, c.P, sizeof(double) * n * n);
  if (qsh) memcpy(qsh, c.x_out, sizeof(double) * nsh);
  if (dipm) memcpy(dipm, c.x_out + nsh, sizeof(double) * 3 * nat);
  if (qp) memcpy(qp, c.x_out + nsh + 3 * nat, sizeof(double) * 6 * nat);
  if (eps) memcpy(eps, c.eps, sizeof(double) * n);
  if (focc) memcpy(focc, c.focc, sizeof(double) * n);
  if (info) {
    memset(info, 0, sizeof(*info));
    info->iterations = c.iterations; info->converged = c.converged; info->nao = n; info->nsh = nsh; info->nel = c.nel;
    info->e_band = c.e_band; info->e_ies = c.esen.e_ies; info->e_3 = c.esen.e_3; info->e_aes = c.esen.e_aes;
    info->e_axc = c.esen.e_axc; info->e_disp = c.esen.e_disp; info->e_ts = c.e_ts;
  }
  scc_free(&c);
  return 0;
}

/* MO populations of the spectrum path: get_xtb_egrad(spec_calc=.true.)
 * (src/tblite.f90:153-166) hands the overlap, the AO-to-atom map, the
 * coefficients, orbital energies and occupations of the converged SCC to
 * write_qmo (src/mo_energ.f90:7-80), which forms per orbital k and atom a
 *   qmo(k,a) = sum_{j on a} sum_l C(j,k) C(l,k) S(j,l) + 1e-10
 * (j ascending, l ascending, each term (C(j,k) C(l,k)) S(j,l)) and divides
 * every orbital's row by its sum over the atoms (atoms ascending).
 * ihomo = max(homo, 1) with tblite's homo of a spin-restricted wavefunction:
 * the aufbau count floor(nel / 2) of one spin channel (uhf = 0).
 * emo[nao] (Eh, ascending), focc[nao], qmo[nao][nat]. Returns 0, -1 (invalid
 * input or Cholesky failure) or 1 (SCC not converged; outputs still set). */
int qcxo_mo_spectrum(int nat, const int* Z, const double* xyz, double charge, double kT, const qcxo_opts* opts,
                     double* emo, double* focc, double* qmo, int* ihomo, qcxo_info* info) {
  qcxo_opts o;
  if (opts) o = *opts; else qcxo_default_opts(&o);
  scc_t c;
  int rc = run_scc(nat, Z, xyz, charge, kT, &o, &c);
  if (rc) { scc_free(&c); return -1; }
  const int n = c.m.nao;
  int* aoat = malloc(sizeof(int) * n);
  for (int s = 0; s < c.m.nsh; ++s)
    for (int i = 0; i < c.m.sh_nao[s]; ++i) aoat[c.m.sh_ao0[s] + i] = c.m.sh_atom[s];
  for (int a = 0; a < nat; ++a)
    for (int k = 0; k < n; ++k) {
      double sum = 0.0;
      for (int j = 0; j < n; ++j) {
        if (aoat[j] != a) continue;
        for (int l = 0; l < n; ++l) sum = sum + (c.C[j * n + k] * c.C[l * n + k]) * c.S[j * n + l];
      }
      qmo[(size_t)k * nat + a] = sum + 1e-10;
    }
  for (int k = 0; k < n; ++k) {
    double sum = 0.0;
    for (int a = 0; a < nat; ++a) sum = sum + qmo[(size_t)k * nat + a];
    for (int a = 0; a < nat; ++a) qmo[(size_t)k * nat + a] = qmo[(size_t)k * nat + a] / sum;
  }
  memcpy(emo, c.eps, sizeof(double) * n);
  memcpy(focc, c.focc, sizeof(double) * n);
  int homo = (int)floor(0.5 * c.nel);
  *ihomo = homo > 1 ? homo : 1;
  if (info) {
    memset(info, 0, sizeof(*info));
    info->iterations = c.iterations; info->converged = c.converged; info->nao = n; info->nsh = c.m.nsh;
    info->nel = c.nel; info->e_total = c.e_elec;
  }
  int conv = c.converged;
  free(aoat);
  scc_free(&c);
  return conv ? 0 : 1;
}

/* ------------------------------------------------------------------------ */
/* energy + analytic gradient                                                */
/* ------------------------------------------------------------------------ */
int qcxo_egrad(int nat, const int* Z, const double* xyz, double charge, double kT, const qcxo_opts* opts,
               double* energy, double* grad, double* qat, qcxo_info* info) {
  if (nat < 1) return -1;
  qcxo_opts o;
  if (opts) o = *opts; else qcxo_default_opts(&o);
  scc_t c;
  int rc = run_scc(nat, Z, xyz, charge, kT, &o, &c);
  if (rc) { scc_free(&c); return -1; }
  mol_t* m = &c.m;
  int n = m->nao, nsh = m->nsh;
  const double* qsh = c.x_out;
  const double* dp = c.x_out + nsh;
  const double* qp = c.x_out + nsh + 3 * nat;
  double* g = calloc(3 * nat, sizeof(double));
  double* dedcn = calloc(nat, sizeof(double));
  double* dedcnd = calloc(nat, sizeof(double));
  double* qa = calloc(nat, sizeof(double));
  for (int s = 0; s < nsh; ++s) qa[m->sh_atom[s]] += qsh[s];

  /* (1) integral-derivative terms over ordered shell pairs on different atoms */
  spair_t sp;
  for (int s = 0; s < nsh; ++s)
    for (int t = 0; t < nsh; ++t) {
      int A = m->sh_atom[s], B = m->sh_atom[t];
      if (A == B) continue;
      int za = Z[A], zb = Z[B], ka = m->sh_k[s], kb = m->sh_k[t];
      double d[3], r = 0;
      for (int k = 0; k < 3; ++k) { d[k] = xyz[3 * A + k] - xyz[3 * B + k]; r += d[k] * d[k]; }
      r = sqrt(r);
      shell_pair(za, ka, zb, kb, d, 1, &sp);
      double fac, dfac, kxyp;
      h0_factor(za, ka, zb, kb, r, selfenergy(za, ka, c.cn[A]), selfenergy(zb, kb, c.cn[B]), &fac, &dfac, &kxyp);
      double gv[3] = {0, 0, 0}, dcn = 0.0;
      int a0 = m->sh_ao0[s], b0 = m->sh_ao0[t];
      for (int i = 0; i < m->sh_nao[s]; ++i)
        for (int j = 0; j < m->sh_nao[t]; ++j) {
          size_t ij = (size_t)(a0 + i) * n + b0 + j;
          double p = c.P[ij], w = c.W[ij];
          dcn += p * kxyp * sp.S[i][j];
          for (int k = 0; k < 3; ++k) {
            double dh = fac * sp.dS[k][i][j] + dfac * (d[k] / r) * sp.S[i][j];
            double v = p * dh - w * sp.dS[k][i][j] - c.vsh[s] * p * sp.dS[k][i][j];
            for (int cc = 0; cc < 3; ++cc) v -= c.vdp[3 * A + cc] * p * sp.dD[cc][k][i][j];
            for (int q = 0; q < 6; ++q) v -= c.vqp[6 * A + q] * p * sp.dQ[q][k][i][j];
            gv[k] += v;
          }
        }
      dedcn[A] += qcx_sh_kcn[za][ka] * dcn;
      for (int k = 0; k < 3; ++k) { g[3 * A + k] += gv[k]; g[3 * B + k] -= gv[k]; }
    }
  /* (2) on-site self-energy CN dependence */
  for (int mu = 0; mu < n; ++mu) {
    int s = m->ao_sh[mu], A = m->ao_atom[mu];
    dedcn[A] += qcx_sh_kcn[Z[A]][m->sh_k[s]] * c.P[(size_t)mu * n + mu];
  }
  /* (3) isotropic electrostatics, (4) multipoles, (5) dispersion pair terms */
  for (int a = 0; a < nat; ++a)
    for (int b = 0; b < a; ++b) {
      double r[3], r2 = 0;
      for (int k = 0; k < 3; ++k) { r[k] = xyz[3 * a + k] - xyz[3 * b + k]; r2 += r[k] * r[k]; }
      double R = sqrt(r2);
      double dEdR = 0.0; /* scalar radial derivative, times r/R */
      for (int s = m->at_sh0[a]; s < m->at_sh0[a] + m->at_nsh[a]; ++s)
        for (int t = m->at_sh0[b]; t < m->at_sh0[b] + m->at_nsh[b]; ++t) {
          double ga = c.es.gam[s * nsh + t];
          dEdR += qsh[s] * qsh[t] * (-R * ga * ga * ga);
        }
      /* dispersion at the converged charges (dispgrad, src/dftd4.f90:1198-1262):
       * radial term -C6_AB(q) dg/dR, and dE/dCN through the reference weights */
      {
        const int R = QCX_D4_MAXREF;
        double wa[QCX_D4_MAXREF], wb[QCX_D4_MAXREF], dwa[QCX_D4_MAXREF], dwb[QCX_D4_MAXREF];
        for (int i = 0; i < R; ++i) {
          wa[i] = c.es.gw[a * R + i] * c.es.zq[a * R + i];
          wb[i] = c.es.gw[b * R + i] * c.es.zq[b * R + i];
          dwa[i] = c.es.dgw[a * R + i] * c.es.zq[a * R + i];
          dwb[i] = c.es.dgw[b * R + i] * c.es.zq[b * R + i];
        }
        double gdis = c.es.gdisp[a * nat + b];
        dEdR += -d4_c6(Z[a], wa, Z[b], wb) * c.es.dgdisp[a * nat + b];
        dedcnd[a] += -gdis * d4_c6(Z[a], dwa, Z[b], wb);
        dedcnd[b] += -gdis * d4_c6(Z[b], dwb, Z[a], wa);
      }
      /* multipoles */
      double r0 = 0.5 * (c.es.mrad[a] + c.es.mrad[b]);
      double f3, d3r, d3r0, f5, d5r, d5r0;
      mp_kernel(3, QCX_AES_A3, R, r0, &f3, &d3r, &d3r0);
      mp_kernel(5, QCX_AES_A5, R, r0, &f5, &d5r, &d5r0);
      const double* ma = dp + 3 * a; const double* mb = dp + 3 * b;
      const double* ta = qp + 6 * a; const double* tb = qp + 6 * b;
      double mar = ma[0] * r[0] + ma[1] * r[1] + ma[2] * r[2];
      double mbr = mb[0] * r[0] + mb[1] * r[1] + mb[2] * r[2];
      double mab = ma[0] * mb[0] + ma[1] * mb[1] + ma[2] * mb[2];
      double rr[6] = {r[0] * r[0], r[1] * r[1], r[2] * r[2], 2 * r[0] * r[1], 2 * r[0] * r[2], 2 * r[1] * r[2]};
      double rta = 0, rtb = 0;
      for (int q = 0; q < 6; ++q) { rta += ta[q] * rr[q]; rtb += tb[q] * rr[q]; }
      double s1 = qa[a] * mbr - qa[b] * mar;
      double s2 = qa[a] * rtb + qa[b] * rta + mab * r2 - 3.0 * mar * mbr;
      /* Theta r for both atoms */
      double tar[3], tbr[3];
      tar[0] = ta[0] * r[0] + ta[3] * r[1] + ta[4] * r[2];
      tar[1] = ta[3] * r[0] + ta[1] * r[1] + ta[5] * r[2];
      tar[2] = ta[4] * r[0] + ta[5] * r[1] + ta[2] * r[2];
      tbr[0] = tb[0] * r[0] + tb[3] * r[1] + tb[4] * r[2];
      tbr[1] = tb[3] * r[0] + tb[1] * r[1] + tb[5] * r[2];
      tbr[2] = tb[4] * r[0] + tb[5] * r[1] + tb[2] * r[2];
      double gv[3];
      for (int k = 0; k < 3; ++k) {
        double ds2 = 2.0 * qa[a] * tbr[k] + 2.0 * qa[b] * tar[k] + 2.0 * mab * r[k] - 3.0 * (mbr * ma[k] + mar * mb[k]);
        gv[k] = (d3r * s1 + d5r * s2 + dEdR) * r[k] / R + f3 * (qa[a] * mb[k] - qa[b] * ma[k]) + f5 * ds2;
      }
      for (int k = 0; k < 3; ++k) { g[3 * a + k] += gv[k]; g[3 * b + k] -= gv[k]; }
      double dedr0 = d3r0 * s1 + d5r0 * s2;
      dedcn[a] += dedr0 * 0.5 * c.es.dmrad[a];
      dedcn[b] += dedr0 * 0.5 * c.es.dmrad[b];
    }
  /* (6) three-body dispersion */
  double e_atm = atm_energy_grad(m, &c.es, g, dedcnd);
  /* (7) repulsion */
  double e_rep = rep_energy_grad(m, g);
  /* (8) coordination-number chain rule */
  for (int a = 0; a < nat; ++a)
    for (int b = 0; b < a; ++b) {
      double r[3], r2 = 0;
      for (int k = 0; k < 3; ++k) { r[k] = xyz[3 * a + k] - xyz[3 * b + k]; r2 += r[k] * r[k]; }
      double R = sqrt(r2), rc = qcx_rcov[Z[a]] + qcx_rcov[Z[b]], f, df1, df2;
      cn_exp_pair(R, rc, &f, &df1);
      d4_cn_pair(Z[a], Z[b], r2, &f, &df2);
      double s = (dedcn[a] + dedcn[b]) * df1 + (dedcnd[a] + dedcnd[b]) * df2;
      for (int k = 0; k < 3; ++k) { g[3 * a + k] += s * r[k] / R; g[3 * b + k] -= s * r[k] / R; }
    }
  double etot = c.e_elec + e_atm + e_rep;
  if (energy) *energy = etot;
  if (grad) memcpy(grad, g, sizeof(double) * 3 * nat);
  if (qat) memcpy(qat, qa, sizeof(double) * nat);
  if (info) {
    memset(info, 0, sizeof(*info));
    info->e_band = c.e_band; info->e_ies = c.esen.e_ies; info->e_3 = c.esen.e_3; info->e_aes = c.esen.e_aes;
    info->e_axc = c.esen.e_axc; info->e_disp = c.esen.e_disp; info->e_atm = e_atm; info->e_rep = e_rep;
    info->e_ts = c.e_ts; info->e_total = etot; info->iterations = c.iterations; info->converged = c.converged;
    info->nao = n; info->nsh = nsh; info->nel = c.nel;
  }
  int conv = c.converged;
  free(g); free(dedcn); free(dedcnd); free(qa);
  scc_free(&c);
  return conv ? 0 : 1;
}

/* ------------------------------------------------------------------------ */
/* MD helpers restated from QCxMS                                             */
/* ------------------------------------------------------------------------ */
/* src/md.f90:749-773 */
void qcxo_leapfrog(int nat, const double* grad, const double* mass, double tstep, double* xyz, double* vel,
                   double* ke) {
  double k = 0.0;
  for (int a = 0; a < nat; ++a) {
    double ms = mass[a];
    for (int j = 0; j < 3; ++j) {
      double vold = vel[3 * a + j];
      vel[3 * a + j] = vel[3 * a + j] - (tstep * grad[3 * a + j] / ms);
      double vavg = 0.5 * (vold + vel[3 * a + j]);
      xyz[3 * a + j] = xyz[3 * a + j] + (tstep * vel[3 * a + j]);
      k = k + 0.5 * (ms * vavg * vavg);
    }
  }
  *ke = k;
}

/* src/mdinit.f90:57-76 */
void qcxo_ekinet(int nat, const double* vel, const double* mass, double* ekin, double* temp) {
  double e = 0.0;
  for (int a = 0; a < nat; ++a)
    e += mass[a] * (vel[3 * a] * vel[3 * a] + vel[3 * a + 1] * vel[3 * a + 1] + vel[3 * a + 2] * vel[3 * a + 2]);
  e *= 0.5;
  *ekin = e;
  *temp = e / (0.5 * 3.0 * nat * QCX_KTOAU);
}

/* src/utility.f90:449-464 */
/* eself (src/iniqm.f90:430-450): energy of atoms without electrons,
 * sum of z^2/2 * gam + z^3/3 * gam3 with z = valence electrons; gam, gam3 are
 * the atomic hardness and third-order parameter (first shell of this set). */
double qcxo_eself(int nat, const int* Z) {
  double e = 0.0;
  for (int a = 0; a < nat; ++a) {
    double z = qcx_nvalence[Z[a]];
    e = e + 0.5 * z * z * qcx_sh_hardness[Z[a]][0] + z * z * z * qcx_sh_gamma3[Z[a]][0] / 3.0;
  }
  return e;
}

/* valence electrons minus charge, electrons_amount (src/iniqm.f90:45-63) */
int qcxo_nel(int nat, const int* Z, int charge) {
  int n = 0;
  for (int a = 0; a < nat; ++a) n += (int)qcx_nvalence[Z[a]];
  return n - charge;
}

int qcxo_getspin(int nat, const int* Z, int charge) {
  int j = 0;
  for (int a = 0; a < nat; ++a) j += Z[a];
  j -= abs(charge);
  int isp = 1 + j % 2;
  if (j < 1) isp = -1;
  return isp;
}

/* src/iniqm.f90:719-732, including its use of grad(2,i) twice and no z term */
double qcxo_gnorm(int nat, const double* grad) {
  double gn = 0.0;
  for (int a = 0; a < nat; ++a)
    gn = gn + grad[3 * a] * grad[3 * a] + grad[3 * a + 1] * grad[3 * a + 1] + grad[3 * a + 1] * grad[3 * a + 1];
  return sqrt(gn);
}

/* src/iniqm.f90:684-715; returns 1 if ok. Sets *e = 0 where the reference does. */
int qcxo_checkqc(int nat, double* e, const double* grad, const double* qat, int charge) {
  if (fabs(*e) < 1e-8) return 0;
  double gn = qcxo_gnorm(nat, grad);
  if (gn < 1e-8 || gn > 20.0) { *e = 0.0; return 0; }
  if (charge > 0) {
    double mx = -1e300;
    for (int a = 0; a < nat; ++a) if (qat[a] > mx) mx = qat[a];
    if (fabs(mx) < 1e-5) { *e = 0.0; return 0; }
  }
  return 1;
}

int qcxo_md_batch(int ntraj, const int* off, const int* Z, double* xyz, double* vel, const double* mass, double* grad,
                  double* epot, const double* charge, const double* kT, int nsteps, double tstep, const qcxo_opts* opts,
                  int nthreads, int* scc_iters, int* active, int* steps_done, double* busy_s) {
  int fails = 0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : fails)
#endif
  for (int t = 0; t < ntraj; ++t) {
    int a0 = off[t], nat = off[t + 1] - off[t];
    int iters = 0, done = 0;
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    double* qat = malloc(sizeof(double) * nat);
    for (int st = 0; st < nsteps; ++st) {
      if (active && !active[t]) break;
      double ke;
      qcxo_leapfrog(nat, grad + 3 * a0, mass + a0, tstep, xyz + 3 * a0, vel + 3 * a0, &ke);
      qcxo_info info;
      int rc = qcxo_egrad(nat, Z + a0, xyz + 3 * a0, charge[t], kT[t], opts, &epot[t], grad + 3 * a0, qat, &info);
      iters += info.iterations;
      /* a failed calculation, or a result checkqc rejects with E = 0, ends the
       * run (src/md.f90:317); with active == NULL every step is taken */
      if (rc == 0) qcxo_checkqc(nat, &epot[t], grad + 3 * a0, qat, (int)charge[t]);
      if (rc != 0 || epot[t] == 0.0) {
        fails++;
        if (active) active[t] = 0;
      } else {
        ++done;
      }
    }
    free(qat);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    if (scc_iters) scc_iters[t] = iters;
    if (steps_done) steps_done[t] = done;
    if (busy_s) busy_s[t] = (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
  }
  return fails;
}

int qcxo_egrad_batch(int nmol, const int* off, const int* Z, const double* xyz, const double* charge, const double* kT,
                     const qcxo_opts* opts, int nthreads, double* energy, double* grad, double* qat, int* rc) {
  int fails = 0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : fails)
#endif
  for (int t = 0; t < nmol; ++t) {
    int a0 = off[t], nat = off[t + 1] - off[t];
    qcxo_info info;
    rc[t] = qcxo_egrad(nat, Z + a0, xyz + 3 * a0, charge[t], kT[t], opts, &energy[t], grad + 3 * a0, qat + a0, &info);
    if (rc[t] != 0) fails++;
  }
  return fails;
}

/* ------------------------------------------------------------------------- */
/* Fragment assignment: restatement of fragment_structure                    */
/* (src/fragments.f90:93-182) with the QCxMS radii of src/covalent_radii.f90:89 */
/* (Angstrom, converted with autoaa = 0.52917726, src/xtb_mctc_convert.f90:24). */
/* ------------------------------------------------------------------------- */
static const double kFragRadAA[19] = {0.0,  0.32, 0.37, 1.30, 0.99, 0.84, 0.75, 0.71, 0.64, 0.60,
                                      0.62, 1.60, 1.40, 1.24, 1.14, 1.09, 1.04, 1.00, 1.01};

int qcxo_fragments(int nat, const int* Z, const double* xyz, double rcut, int at1, int at2, int* frag) {
  const double aatoau = 1.0 / 0.52917726;
  unsigned char* connect = (unsigned char*)calloc((size_t)nat * nat, 1);
  for (int i = 0; i < nat - 1; ++i)
    for (int j = i + 1; j < nat; ++j) {
      double dx = xyz[3 * i] - xyz[3 * j], dy = xyz[3 * i + 1] - xyz[3 * j + 1], dz = xyz[3 * i + 2] - xyz[3 * j + 2];
      double r = sqrt(dx * dx + dy * dy + dz * dz);
      double rcov = rcut * 0.5 * (aatoau * kFragRadAA[Z[i]] + aatoau * kFragRadAA[Z[j]]);
      if (r < rcov) connect[(size_t)i * nat + j] = connect[(size_t)j * nat + i] = 1;
    }
  int nfrag = 1;
  if (at1 == 0 && at2 == 0) {
    for (int i = 0; i < nat; ++i) frag[i] = 1;
  } else {
    for (int i = 0; i < nat; ++i) frag[i] = 0;
    frag[at1 - 1] = 1;
    int total = 1, current = 0;
    if (at2 != 0) connect[(size_t)(at1 - 1) * nat + at2 - 1] = connect[(size_t)(at2 - 1) * nat + at1 - 1] = 0;
    while (total != nat) {
      ++current;
      int changed = 1;
      while (changed) {  /* sweep until the fragment stops growing */
        changed = 0;
        for (int i = 0; i < nat; ++i)
          if (frag[i] == current)
            for (int j = 0; j < nat; ++j)
              if (connect[(size_t)i * nat + j] && frag[j] == 0) {
                frag[j] = current;
                ++total;
                changed = 1;
              }
      }
      for (int i = 0; i < nat; ++i) /* first atom of the next fragment */
        if (frag[i] == 0) {
          frag[i] = current + 1;
          ++total;
          break;
        }
    }
    nfrag = 0;
    for (int i = 0; i < nat; ++i) nfrag = frag[i] > nfrag ? frag[i] : nfrag;
  }
  free(connect);
  return nfrag;
}
