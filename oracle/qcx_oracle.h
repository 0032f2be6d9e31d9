/*
 * CPU FP64 oracle for the QCxMS trajectory-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker that the CUDA path
 * (libqcxgpu.so) is compared against; only tests, the smoke check and the
 * CPU-baseline leg of bench.py load it. The product path never calls it.
 *
 * It restates, in plain C:
 *   - the GFN2-xTB energy + analytic gradient evaluation that QCxMS requests
 *     from tblite v0.2.1 through get_xtb_egrad (src/tblite.f90:65-175),
 *     following the published GFN2-xTB functional form (Bannwarth, Ehlert,
 *     Grimme, JCTC 15, 1652 (2019)) with the synthetic parameter set in
 *     qcxms_gb300/csrc/qcx_params.h;
 *   - leapfrog (src/md.f90:749-773), ekinet (src/mdinit.f90:57-76),
 *     getspin (src/utility.f90:449-464), checkqc/gnorm (src/iniqm.f90:684-732).
 *
 * Parity with tblite is UNPINNED: tblite and its GFN2 parameter tables are not
 * part of the QCxMS sources, and QCxMS ships no reference energies/gradients.
 */
#ifndef QCX_ORACLE_H
#define QCX_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int max_iter;          /* SCC iteration cap */
  double econv;          /* |E_i - E_{i-1}| threshold (Eh) */
  double pconv;          /* rms(x_out - x_in) threshold over the mixed moments */
  double broyden_alpha;  /* linear mixing parameter of the modified Broyden scheme */
} qcxo_opts;

typedef struct {
  double e_band, e_ies, e_3, e_aes, e_axc, e_disp, e_atm, e_rep, e_ts, e_total;
  int iterations, converged, nao, nsh;
  double nel;
} qcxo_info;

void qcxo_default_opts(qcxo_opts* o);
int qcxo_nao(int nat, const int* Z);
int qcxo_nsh(int nat, const int* Z);

/* Energy + gradient. xyz and grad are [nat][3] (Fortran xyz(3,nat)), Bohr.
 * kT in Hartree. Returns 0 on success, 1 if the SCC did not converge,
 * -1 on invalid input. */
int qcxo_egrad(int nat, const int* Z, const double* xyz, double charge, double kT,
               const qcxo_opts* opts, double* energy, double* grad, double* qat,
               qcxo_info* info);

/* Intermediate quantities for kernel-level parity tests.
 * S, H0: [nao][nao]; Dm: [3][nao][nao]; Qm: [6][nao][nao]; cn, cnd: [nat]. */
int qcxo_integrals(int nat, const int* Z, const double* xyz, double* S, double* H0,
                   double* Dm, double* Qm, double* cn, double* cnd);

/* Converged SCC quantities: P [nao][nao], qsh [nsh], dipm [nat][3], qp [nat][6],
 * eps [nao], focc [nao] (occupation per MO, 0..2). */
int qcxo_scc(int nat, const int* Z, const double* xyz, double charge, double kT,
             const qcxo_opts* opts, double* P, double* qsh, double* dipm, double* qp,
             double* eps, double* focc, qcxo_info* info);

/* Symmetric eigensolver used by the oracle (Householder + implicit QL).
 * A [n][n] is destroyed; V [n][n] holds eigenvectors as columns. */
int qcxo_syev(int n, double* A, double* w, double* V);
/* MO energies, occupations and normalised Mulliken populations per atom of
 * the converged SCC, as write_qmo forms them (src/mo_energ.f90:7-80); qmo is
 * [nao][nat]. Returns 0, 1 (SCC not converged) or -1. */
int qcxo_mo_spectrum(int nat, const int* Z, const double* xyz, double charge, double kT, const qcxo_opts* opts,
                     double* emo, double* focc, double* qmo, int* ihomo, qcxo_info* info);

/* D4 data checks: C6 of reference pair (za, i; zb, j) built from QCxMS's
 * reference polarisabilities (src/dftd4.f90:531-595, 665), -1 outside the
 * table; and the molecular C6 [nat][nat] at the covalent CNs and charges q
 * (zero charges if q is NULL). */
double qcxo_d4_c6ref(int za, int i, int zb, int j);
void qcxo_d4_c6(int nat, const int* Z, const double* xyz, const double* q, double* c6);

/* Reference MD helpers. */
void qcxo_leapfrog(int nat, const double* grad, const double* mass, double tstep,
                   double* xyz, double* vel, double* ke);
void qcxo_ekinet(int nat, const double* vel, const double* mass, double* ekin, double* temp);
int qcxo_getspin(int nat, const int* Z, int charge);
double qcxo_eself(int nat, const int* Z);
int qcxo_nel(int nat, const int* Z, int charge);
double qcxo_gnorm(int nat, const double* grad);
int qcxo_checkqc(int nat, double* e, const double* grad, const double* qat, int charge);

/* Fragment assignment (src/fragments.f90:93-182, fragment_structure): atoms i, j
 * are bonded when r_ij < rcut * 0.5 * (R_i + R_j) with the QCxMS radii
 * (src/covalent_radii.f90:89, Rad); at1/at2 are 1-based as in the reference
 * (at1 = at2 = 0: one fragment; at2 != 0: the at1-at2 bond is ignored).
 * frag[nat] gets 1-based fragment numbers; returns the number of fragments. */
int qcxo_fragments(int nat, const int* Z, const double* xyz, double rcut, int at1, int at2, int* frag);

/* Batched MD on the CPU: ntraj independent trajectories, each advanced nsteps
 * leapfrog + egrad steps (OpenMP over trajectories, dynamic schedule: pass them
 * largest first). Arrays are concatenated per trajectory using atom offsets
 * off[ntraj+1]. grad must hold the gradient at the initial geometry. With
 * active[ntraj] given, a trajectory whose calculation fails or whose result
 * checkqc rejects (E = 0) stops (active[t] = 0), as the MD run ends
 * (src/md.f90:317); steps_done[t] (may be NULL) counts its accepted steps and
 * busy_s[t] (may be NULL) the wall seconds its thread spent on it.
 * Returns the number of failed trajectory-steps. */
int qcxo_md_batch(int ntraj, const int* off, const int* Z, double* xyz, double* vel,
                  const double* mass, double* grad, double* epot, const double* charge,
                  const double* kT, int nsteps, double tstep, const qcxo_opts* opts,
                  int nthreads, int* scc_iters, int* active, int* steps_done, double* busy_s);

/* Energy + gradient of nmol structures (OpenMP over structures); rc[nmol] gets
 * each qcxo_egrad return code. Returns the number of failures. */
int qcxo_egrad_batch(int nmol, const int* off, const int* Z, const double* xyz, const double* charge,
                     const double* kT, const qcxo_opts* opts, int nthreads, double* energy, double* grad,
                     double* qat, int* rc);

#ifdef __cplusplus
}
#endif
#endif
