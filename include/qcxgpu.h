/*
 * libqcxgpu -- C ABI of the GB300 GFN2-xTB trajectory-step engine.
 *
 * Plain pointers and sizes only. Coordinates, velocities and gradients are
 * [nat][3] row-major doubles, which is the memory order of the Fortran
 * arrays xyz(3,nat) / grad(3,nat) used by QCxMS. Units: Bohr, Hartree,
 * atomic time units, electron masses (atomic units), Kelvin for etemp.
 *
 * Return codes follow the reference bridge (src/tblite.f90:55-58):
 *   0  success
 *   5  unknown or unsupported method
 *  -1  failure (SCC not converged, non-finite result, invalid input, CUDA error)
 * qcx_last_error() describes the last failure of the calling process.
 */
#ifndef QCXGPU_H
#define QCXGPU_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QCX_METHOD_GFN1 1
#define QCX_METHOD_GFN2 2
#define QCX_METHOD_IPEA1 11

/* status bits reported per trajectory by qcx_batch_get */
#define QCX_STATUS_SCC_NOT_CONVERGED 1
#define QCX_STATUS_NON_FINITE 2
#define QCX_STATUS_CHOLESKY_FAILED 4
#define QCX_STATUS_EIGEN_NOT_CONVERGED 8
/* checkqc (src/iniqm.f90:684-715) rejected the result: |E| < 1e-8, gnorm
 * outside [1e-8, 20], or a cation with max(qat) below 1e-5 in magnitude; the
 * last two set the energy to 0, as the reference does */
#define QCX_STATUS_CHECKQC 16
/* the SCC stopped at the per-launch budget of qcx_batch_set_scc_budget; the
 * next qcx_batch_step or qcx_batch_egrad continues it (not a failure) */
#define QCX_STATUS_SCC_PENDING 32

/* Library version (major*10000 + minor*100 + patch). */
int qcx_version(void);

/* Text of the last error in this process ("" if none). */
const char* qcx_last_error(void);

/*
 * Single-structure energy + gradient: the drop-in for
 *   get_xtb_egrad(num, xyz, charge, multiplicity, method, etemp,
 *                 output_file, qat, energy, gradient, stat, spec_calc)
 * of module qcxms_tblite (src/tblite.f90:65-175), as called by egrad
 * (src/iniqm.f90:641-655) on every MD step. The multiplicity is accepted but,
 * as in the reference (uhf = min(multiplicity-1, 0), src/tblite.f90:111),
 * the calculation is spin-restricted with Fermi smearing at etemp.
 * The device state for a given atom list, charge and etemp is cached between
 * calls, one per GPU (the calling thread's current device); calls are
 * serialised by a lock.
 * Writes energy (Eh), grad [nat][3] (Eh/Bohr) and qat [nat] (Mulliken charges).
 * The result then goes through checkqc as egrad does after the call
 * (src/iniqm.f90:650, 684-715): a rejected result returns -1, with the energy
 * set to 0 where checkqc sets it (a Fortran egrad that calls checkqc itself
 * sees the same outcome).
 */
int qcx_egrad(int method, int nat, const int32_t* num, const double* xyz, int charge, int multiplicity,
              double etemp, double* energy, double* grad, double* qat);

/*
 * checkqc (src/iniqm.f90:684-715) on the GPU for one result held by the
 * caller: the device function that qcx_egrad and every batch evaluation apply
 * (gnorm sums grad(1,i)**2 + grad(2,i)**2 + grad(2,i)**2 as the reference
 * does, src/iniqm.f90:719-732). grad [nat][3], qat [nat]; *energy is set to 0
 * where the reference sets it. Returns 0 when the result is accepted, 1 for
 * |E| < 1e-8, 2 for a gradient norm outside [1e-8, 20], 3 for a cation
 * (charge > 0) whose largest atomic charge is below 1e-5 in magnitude, -1 on
 * invalid arguments or a CUDA error.
 */
int qcx_checkqc(int nat, const double* grad, const double* qat, int charge, double* energy);

/*
 * Batched trajectories: nmol independent molecules advanced together on one
 * GPU. Replaces the one-process-per-trajectory fan-out of bin/pqcxms:88-99;
 * each molecule follows the md.f90 step: leapfrog (src/md.f90:749-773) then
 * egrad (src/md.f90:396).
 */
typedef struct qcx_batch qcx_batch;

/* nat[nmol]; num = atomic numbers of all molecules concatenated;
 * charge[nmol]; etemp[nmol] in Kelvin. Returns NULL on failure. */
qcx_batch* qcx_batch_create(int nmol, const int32_t* nat, const int32_t* num, const double* charge,
                            const double* etemp);
void qcx_batch_destroy(qcx_batch* b);

/* SCC controls (defaults: 250, 1e-7 Eh, 1e-6, 0.25). max_iter <= 250. */
int qcx_batch_set_scc(qcx_batch* b, int max_iter, double econv, double pconv, double mixing);

/* Arithmetic of the SCC loop: 0 = FP64 throughout (default); 1 = mixed.
 * Mixed mode runs its first iterations in FP32: Fock build, potentials,
 * transforms, eigensolve, Fermi level, density and moments, until the moment
 * residual drops below 1e-4 (or stops improving below 1e-3). The remaining
 * iterations (at least two) keep the coefficients and their O(n^3) products
 * in double-float arithmetic (hi + lo FP32 pairs, about 48 significant bits)
 * and their Fock build, potentials, Fermi level, energies and Broyden mixing
 * in FP64, and meet the same convergence thresholds as mode 0. Integrals and
 * the gradient are FP64 in both modes, except the three-body dispersion term,
 * which is summed in FP32 per triple and accumulated in FP64. */
#define QCX_PRECISION_FP64 0
#define QCX_PRECISION_MIXED 1
int qcx_batch_set_precision(qcx_batch* b, int precision);

/* Starting point of each SCC: QCX_GUESS_ZERO (default) starts from zero
 * moments, as the reference does by creating a fresh wavefunction on every
 * call (src/tblite.f90:133); QCX_GUESS_PREVIOUS starts a molecule's SCC from
 * its converged moments of the previous evaluation (when that SCC converged;
 * coordinates set in between do not matter), which needs fewer iterations
 * along a trajectory and reaches the same solution to the SCC tolerances.
 * This option has no counterpart in the reference. */
#define QCX_GUESS_ZERO 0
#define QCX_GUESS_PREVIOUS 1
int qcx_batch_set_guess(qcx_batch* b, int guess);

/* SCC iteration budget of one MD step (0, the default: none). QCxMS runs its
 * trajectories as independent processes (bin/pqcxms), each at its own pace;
 * a batch that steps all trajectories together waits in every step for the
 * slowest SCC. With a budget b, the SCC of a molecule of n AOs stops after
 * ceil(b (nmax / n)^2) iterations of one qcx_batch_step (nmax: the batch's
 * largest molecule, or in qcx_batch_step_groups/_paced the largest of the
 * molecule's group; mixed precision stops only between FP32 iterations) and
 * the next step continues it at the same coordinates: that trajectory does
 * not move and counts no step until its SCC has converged (status
 * QCX_STATUS_SCC_PENDING meanwhile), so trajectories advance at their own
 * pace, as the reference's processes do, and each trajectory's sequence of
 * steps is the one without a budget up to the SCC tolerances. The iteration
 * limit (qcx_batch_set_scc) counts every iteration of an SCC.
 * qcx_batch_egrad ignores the budget and completes every SCC, a suspended one
 * included. Returns 0 or -1. */
int qcx_batch_set_scc_budget(qcx_batch* b, int iters);

/* Size-bucketed stepping. The batch's molecules form qcx_batch_group_info
 * groups by size (group 0 the largest). qcx_batch_step_groups advances group g
 * by nsteps[g] MD steps (each as qcx_batch_step does it: leapfrog, energy +
 * gradient, the device loop rules when on), every group from its own captured
 * graph on its own stream, concurrently with the others; the batch stream
 * continues after all of them. Trajectories never interact (bin/pqcxms runs
 * each as its own process), so groups of small molecules can take several
 * steps while the largest molecules take one. qcx_batch_step_paced gives group
 * 0 nsteps steps and every other group as many as fit into the same time (at
 * most 16 nsteps), from the per-step times the previous paced call measured
 * (the first call gives every group nsteps). Both return 0 or -1. */
int qcx_batch_step_groups(qcx_batch* b, const int32_t* nsteps, double tstep);
int qcx_batch_step_paced(qcx_batch* b, int nsteps, double tstep);
/* Scale of the SCC budget in grouped and paced steps: per_group = 1 (the
 * default) scales it with the largest molecule of each molecule's group, 0
 * with the batch's largest. Returns 0 or -1. qcx_batch_get_scc_budget returns
 * the current budget and scale (either pointer may be NULL). */
int qcx_batch_set_scc_budget_scale(qcx_batch* b, int per_group);
int qcx_batch_get_scc_budget(qcx_batch* b, int32_t* iters, int32_t* per_group);
/* Autotuner of the per-step SCC budget for paced stepping: for every candidate
 * budget cand[c] (0: none) and both budget scales, one untimed paced call and
 * then `calls` timed ones of qcx_batch_step_paced(b, steps_per_call, tstep) on
 * the batch's own trajectories (real MD steps: the run continues), in two
 * passes over the configurations, the second in reverse order (the batch's
 * state drifts over the calls; the reverse pass cancels a linear drift);
 * rates (may be NULL, 2 ncand entries) = completed trajectory-steps per second
 * over both passes, rates[c] with the per-group scale and rates[ncand + c]
 * with the batch-wide one. The
 * batch keeps the fastest budget and scale; the call returns the budget (or
 * -1), qcx_batch_get_scc_budget the scale. qcx_batch_autotune_budget is the
 * same with steps_per_call = 1. */
int qcx_batch_autotune_paced(qcx_batch* b, double tstep, int steps_per_call, const int32_t* cand, int ncand,
                             int calls, double* rates);
int qcx_batch_autotune_budget(qcx_batch* b, double tstep, const int32_t* cand, int ncand, int calls,
                              double* rates);
/* Number of groups; group_of_mol [nmol], the step counts of the last grouped
 * call nsteps_last [ngroup] and the measured per-step times ms_per_step
 * [ngroup] (0: not measured yet) when not NULL. */
int qcx_batch_group_info(qcx_batch* b, int32_t* group_of_mol, int32_t* nsteps_last, double* ms_per_step);
/* SCC iterations run so far per molecule (all launches), iter_sum [nmol]. */
int qcx_batch_get_iterations(qcx_batch* b, int64_t* iter_sum);

/* Copy host state in. Any pointer may be NULL to keep the current value.
 * xyz, vel: [natom][3]; mass: [natom] (atomic units). New coordinates start
 * every trajectory afresh: stopped ones run again, suspended SCCs are dropped. */
int qcx_batch_set_state(qcx_batch* b, const double* xyz, const double* vel, const double* mass);

/* Copy coordinates and/or velocities ([natom][3], NULL keeps the current
 * value) in without starting new runs: stopped trajectories stay stopped and
 * the MD or collision rules stay on. For a host that reads the state after a
 * step and writes it back (or changes it) before the next one. The copies are
 * queued on the batch's stream; the host buffers must stay valid until the
 * next call that synchronises (qcx_batch_get, qcx_batch_sync). */
int qcx_batch_load_state(qcx_batch* b, const double* xyz, const double* vel);

/* Energy and gradient at the current coordinates. */
int qcx_batch_egrad(qcx_batch* b);

/* nsteps MD steps of tstep (atomic time units): leapfrog with the current
 * gradient, then energy + gradient at the new coordinates. The first call
 * captures one step in a CUDA graph and replays it. Requires a prior
 * qcx_batch_egrad (the gradient of the starting geometry). */
int qcx_batch_step(qcx_batch* b, int nsteps, double tstep);

/* Copy results out. Any pointer may be NULL. energy, ekin: [nmol];
 * status, iters: [nmol] (status bits QCX_STATUS_*, SCC iterations of the
 * last evaluation); xyz, vel, grad: [natom][3]; qat: [natom]. */
int qcx_batch_get(qcx_batch* b, double* xyz, double* vel, double* grad, double* energy, double* qat,
                  double* ekin, int32_t* status, int32_t* iters);

/* Energy decomposition of molecule i: band, isotropic ES, third order,
 * anisotropic ES, multipole XC, dispersion, three-body, repulsion, -TS,
 * total, Fermi level, number of FP64 SCC iterations (12 doubles). */
int qcx_batch_get_energy_terms(qcx_batch* b, int i, double* terms);

/* Dense matrices of molecule i for inspection: which = 0 S, 1 H0, 8 P,
 * 9 W (nao x nao, row-major); returns nao or -1. */
int qcx_batch_get_matrix(qcx_batch* b, int i, int which, double* out);

/* Number of kernel launches issued by the last qcx_batch_step /
 * qcx_batch_egrad call (graph replays count their kernel nodes). */
long long qcx_batch_kernel_launches(qcx_batch* b);

/* Per-trajectory progress: active[nmol] (1 while running; a failed energy
 * evaluation stops the trajectory, as src/md.f90:317-344 ends the MD run)
 * and steps_done[nmol] (successful energy + gradient evaluations so far).
 * Setting new coordinates with qcx_batch_set_state restarts all. */
int qcx_batch_get_progress(qcx_batch* b, int32_t* active, int64_t* steps_done);

/* Fragment assignment of every molecule at its current coordinates, as
 * fragment_structure (src/fragments.f90:93-182), which md.f90:450 calls every
 * step with rcut = 3.0, at1 = 1, at2 = 0: atoms are bonded when their distance
 * is below rcut times the mean of their QCxMS covalent radii
 * (src/covalent_radii.f90:89); fragment 1 is at1's, the others follow in the
 * order of their lowest-numbered atom. at1/at2 are 1-based atom numbers within
 * each molecule (at1 = at2 = 0: everything one fragment; at2 != 0: the at1-at2
 * bond does not count). frag[natom] gets the 1-based fragment number of every
 * atom, nfrag[nmol] the number of fragments; either may be NULL. */
int qcx_batch_fragments(qcx_batch* b, double rcut, int at1, int at2, int32_t* frag, int32_t* nfrag);

/*
 * MD bookkeeping and exit rules of an electron-impact fragmentation run on the
 * device (src/md.f90:285-682 with it > 0, isec = 1), evaluated after every step
 * of qcx_batch_step inside the captured step graph: per trajectory the step
 * count, the running mean temperature and total-energy error (exit when an
 * energy evaluation failed or |Eerror| > 0.1 Eh, src/md.f90:316-342), fragment
 * numbers at rcut 3.0 (src/md.f90:450) and the fragments' temperatures
 * (intenergy, src/md.f90:715-741), and the exits: more than 6 fragments, more
 * than nfragexit fragments, 2 or more fragments for over 1000 steps, nfragexit
 * fragments for more than `more` further steps (the reference uses 250), and
 * max_steps (src/md.f90:456-462, 620-679). A trajectory that exits stops (its
 * active flag drops to 0). Call after qcx_batch_egrad of the start geometry:
 * the first loop top uses that energy and the kinetic energy of the current
 * velocities (ekinet, src/mdinit.f90:57-76). New coordinates through
 * qcx_batch_set_state switch the rules off. The heating of the first steps is
 * set up by qcx_batch_set_md_heating, the per-step electronic temperature
 * by qcx_batch_set_md_etemp. Not covered: the CID branch, the output-file
 * averages.
 */
int qcx_batch_set_md_rules(qcx_batch* b, int nfragexit, int more, int max_steps);

/* Averaged structure of every trajectory, axyz = the mean of the coordinates
 * at the loop tops of the current window of avdump = 50 steps
 * (src/md.f90:352-362, 695); QCxMS hands it to analyse for the fragment IPs.
 * axyz [natom][3]; requires qcx_batch_set_md_rules. */
int qcx_batch_get_md_avg_xyz(qcx_batch* b, double* axyz);

/* Heating of the first steps of an electron-impact run (impactscale,
 * src/impact.f90:12-55, called by src/md.f90:439-441 while nstep <= nadd and
 * the molecule is one fragment): each step the velocities are scaled by
 * 1 + velof * scal, scal grown in steps of 0.0002 until the kinetic energy
 * reaches eimp * fadd * nstep + Ekin(start); nadd = (tadd + tstep)/tstep - 1
 * and fadd = tstep/(tadd + tstep) as src/md.f90:265-266. eimp[nmol] (Eh),
 * tadd[nmol] (atomic time units) and velof[natom] (NULL: all 1) come from each
 * trajectory's start file (rdstart); tstep is the step of qcx_batch_step. Call
 * before qcx_batch_set_md_rules, which reads these values. The running mean of
 * the total energy starts after the nadd steps (src/md.f90:304-309). A run whose
 * scaling needs 20000 increments ends (the reference stops the program). The
 * electronic temperature follows qcx_batch_set_md_etemp when that is on. */
int qcx_batch_set_md_heating(qcx_batch* b, const double* eimp, const double* tadd, const double* velof,
                             double tstep);

/* Electronic temperature of every MD step (EI runs): setetemp
 * (src/utility.f90:69-86), which src/md.f90:443-446 calls after every step
 * with dum = eimp - eimp*nstep/nadd and the step's fragment count before
 * fragment_structure: etemp = 5000 + 20000 ax, plus dum * ieetemp while
 * dum > 0 and the molecule is one fragment. The next evaluation runs at
 * kT = etemp * ktoau (src/tblite.f90:133). The start uses setetemp(1, eimp)
 * (src/md.f90:167-168), which this call sets right away, so call it after
 * qcx_batch_set_md_heating (eimp) and before the qcx_batch_egrad of the start
 * geometry, then qcx_batch_set_md_rules. ax and ieetemp are the input's (0
 * and 0 by default, src/input.f90:199). New coordinates through
 * qcx_batch_set_state switch it off and restore the batch's temperatures. */
int qcx_batch_set_md_etemp(qcx_batch* b, double ax, double ieetemp);
/* Electronic temperature (K) of every trajectory's next evaluation. */
int qcx_batch_get_md_etemp(qcx_batch* b, double* etemp);

/* State of the MD rules per trajectory (any pointer may be NULL): nstep,
 * nfrag (fragments at the last step), fragstate (1: exit on fragment count or
 * step limit, 2: fragments constant for 1000 steps, 0 otherwise), mdok (1: the
 * run counts), done (1: the run has ended), tav (sum of the step
 * temperatures, K), eerror (Eh), fragT [nmol][10] (K). */
int qcx_batch_get_md_state(qcx_batch* b, int32_t* nstep, int32_t* nfrag, int32_t* fragstate, int32_t* mdok,
                           int32_t* done, double* tav, double* eerror, double* fragT);

/* Synchronise the batch's stream. */
int qcx_batch_sync(qcx_batch* b);

/* The cudaStream_t the batch launches on (as void*), for callers that time
 * or order work against it. */
void* qcx_batch_stream(qcx_batch* b);

/* One energy + gradient evaluation with CUDA events between its kernels on
 * the batch's stream. ms[0..5] = coordination numbers, integrals, SCC,
 * gradient reset, integral-derivative gradient, atom-pair gradient. */
int qcx_batch_profile_egrad(qcx_batch* b, float* ms);

/* Timing marks inside the captured step graph (on = 1; the next
 * qcx_batch_step captures the graph again with them, on = 0 without). The
 * step's kernels run in G molecule groups on parallel streams; after a step,
 * qcx_batch_get_timing writes ms[0..1+4G] (n >= 2 + 4G floats): ms[0] = 0 at
 * the start of the step, ms[1 + 4g + k] the time of mark k of group g (0
 * integrals start, 1 SCC start, 2 SCC end, 3 gradient end) and ms[1 + 4G]
 * the end of the step, all in ms from the start of the last replayed step.
 * Returns G. */
int qcx_batch_set_timing(qcx_batch* b, int on);
int qcx_batch_get_timing(qcx_batch* b, float* ms, int n);

/* Atomic-orbital and atom counts of every molecule (nao[nmol], nat[nmol]);
 * used to count algorithmic work. */
int qcx_batch_get_sizes(qcx_batch* b, int32_t* nao, int32_t* nat);

/*
 * Fragment ionisation potentials (electron affinities for mchrg < 0) of ntraj
 * fragmented structures, all single points in one batch: the GFN2 path of
 * analyse (src/analyse.f90:13-467) that write_fragments
 * (src/write_fragments.f90:100-106) calls when a trajectory ends. nat[ntraj],
 * num and xyz ([natom][3], Bohr) of all trajectories concatenated, frag[natom]
 * the 1-based fragment number of every atom (qcx_batch_fragments, or
 * fragment_structure, src/fragments.f90:93-182), 1..nfrag without gaps,
 * nfrag <= QCX_MAX_FRAGMENTS. Each fragment keeps its atoms in their original
 * order (avg_frag_struc, src/analyse.f90:471-503); its neutral and its ions of
 * charge sign(mchrg)*1..|mchrg| are evaluated at etemp (analyse uses 300 K for
 * GFN2, src/analyse.f90:244-248), spin-restricted as eqm/get_xtb_egrad do. A
 * fragment left without electrons gets the self energy of eself
 * (src/iniqm.f90:430-450). Outputs, per trajectory t:
 *   fragip[t][i][c-1] = (E(charge c) - E(neutral)) * 27.21138505 eV for
 *     fragment i < nfrag and c = 1..|mchrg| (src/analyse.f90:367-368), 0 where
 *     an energy is 0 or for trajectories with one fragment;
 *   efrag[t][i][c] (may be NULL): the energies (Eh), c = 0 the neutral;
 *   ipok[t]: 0 if any of its calculations failed (SCC not converged, |E| <
 *     1e-10, src/iniqm.f90:415-421; more charge than valence electrons) or an
 *     IP lies outside the bounds of src/analyse.f90:386-403, else 1.
 * precision: QCX_PRECISION_FP64 or QCX_PRECISION_MIXED. Returns 0, 5 (method
 * not GFN2) or -1 (invalid input, CUDA error).
 */
#define QCX_MAX_FRAGMENTS 10
#define QCX_FRAGIP_MAX_CHARGE 4
int qcx_fragment_ips(int method, int ntraj, const int32_t* nat, const int32_t* num, const double* xyz,
                     const int32_t* frag, int mchrg, double etemp, int precision, double* fragip, double* efrag,
                     int32_t* ipok);

/*
 * Fragment masses and sum formulas, fragmass (src/fragments.f90:10-84), on
 * the host: frag[nat] holds fragment numbers 1..QCX_MAX_FRAGMENTS, mass[nat]
 * atomic masses in atomic units. Fragments with atoms are numbered in order
 * (*nfrag of them); fragm_amu[k] is fragment k's mass in amu and formula +
 * 80 k its formula with the elements in order of atomic number, each with its
 * count ("H4C2", "H2O1"). fragm_amu or formula may be NULL.
 */
int qcx_fragment_formula(int nat, const int32_t* num, const int32_t* frag, const double* mass, int32_t* nfrag,
                         double* fragm_amu, char* formula);

/*
 * Boltzmann weights of fragment IPs, boltz (src/utility.f90:469-498):
 * fragchrg2(i,j) = exp(-ip(i,j)/f) / sum exp(-ip/f), f = temp * kB * (627.50947428
 * for units 1, kcal/mol; 27.21138505 for units 2, eV). ip and fragchrg2 are
 * Fortran arrays (nfrag, mchrg): element (i,j) at [i + j*nfrag], 0-based.
 */
int qcx_boltz(int units, int nfrag, int mchrg, double temp, const double* ip, double* fragchrg2);

/*
 * Stop rules of the collision MD (CID, src/cid.f90:739-1052) on the device,
 * evaluated after every step of qcx_batch_step inside the step graph. Every
 * molecule is the ion followed by ONE collision gas atom (the last atom). Per
 * step: a failed energy evaluation ends the run (failed = 1); the ion's
 * centre-of-mass speed from its displacement, its internal temperature
 * (tinit at the first step) and the running mean avg_temp, and the collision
 * energy in the centre-of-mass frame ecom_ev (src/cid.f90:769-793, 1209-1215);
 * the ion's fragments (fragment_structure over the ion's atoms, rcut 3.0);
 * every 10 steps the gas atom's distance from the ion's centre of mass: after 5
 * growing checks in a row the collision is marked and the run ends
 * 800 * (2 tstep in fs) steps later, or add_steps (by ion size,
 * src/cid.f90:276-278) after a fragmentation that follows the collision; and
 * at ntot steps at the latest (src/cid.f90:955-1036). A run that ends stops
 * (active flag 0). Call after qcx_batch_egrad of the start geometry; replaces
 * the MD rules of qcx_batch_set_md_rules; new coordinates switch it off. Not
 * covered: the averaged structures and the output files.
 */
int qcx_batch_set_cid_rules(qcx_batch* b, double tinit, int ntot);
/* The averaged structure of every collision trajectory, as the collision loop
 * hands it to the fragment IPs (src/cid.f90:1095-1101): after the ion fell
 * into more fragments, the average over the steps counted while the fragments
 * kept their atom counts (at most cnt_steps = 50, src/cid.f90:802-909); else
 * the coordinate sum of the current window of dumpavg = 50 loop tops divided
 * by its length. axyz [natom][3], the gas atom's rows 0. For trajectories still
 * running: the value if the run ended now. Returns 0 or -1. */
int qcx_batch_get_cid_avg_xyz(qcx_batch* b, double* axyz);

/* State of the collision rules per trajectory (any pointer may be NULL). */
int qcx_batch_get_cid_state(qcx_batch* b, int32_t* nstep, int32_t* nfrag, int32_t* collided, int32_t* fragmented,
                            int32_t* total_steps, int32_t* done, int32_t* failed, double* avg_temp,
                            double* ecom_ev);

/*
 * Trajectory start files of a QCxMS ensemble (host only, no GPU work), so
 * that a batched driver can load TMPQCXMS/TMP.n/ of every trajectory instead
 * of starting one process per trajectory (bin/pqcxms:88-99).
 * qcx_read_xyz reads start.xyz (xyz format, Angstrom; elements 1..18) into
 * num[nat] and xyz[nat][3] in Bohr (1/0.52917726 Bohr per Angstrom,
 * src/xtb_mctc_convert.f90:24-25); with num = xyz = NULL it only returns the
 * atom count in *nat. qcx_read_start reads qcxms.start as rdstart
 * (src/utility.f90:379-422) does, in the layout wrstart writes
 * (src/utility.f90:321-373): the trajectory number, eimp, tadd, then per atom
 * vx vy vz velof (D22.14 fields). Any output pointer may be NULL.
 */
int qcx_read_xyz(const char* path, int max_nat, int32_t* nat, int32_t* num, double* xyz);
int qcx_read_start(const char* path, int nat, int32_t* itrj, double* eimp, double* tadd, double* vel,
                   double* velof);
/* Writes qcxms.start in wrstart's layout (src/utility.f90:321-373): itrj as
 * (i4), eimp and tadd as (D22.14), per atom vx vy vz velof as D22.14 fields
 * (14 significant digits, as the Fortran edit descriptor prints them). */
int qcx_write_start(const char* path, int itrj, int nat, double eimp, double tadd, const double* vel,
                    const double* velof);

/*
 * Self-check of the tensor-core product the SCC kernel uses (no counterpart in
 * the reference): one CTA computes C[M][N] = op(A) op(B) on the tcgen05 tensor
 * cores as split-TF32 (about 21 significant bits), reps times, from host
 * matrices. op(A) = A [M][K] (ta = 0) or A^T with A [K][M] (ta = 1); op(B) =
 * B [K][N] (tb = 0) or B^T with B [N][K] (tb = 1). M <= 512, N <= 256.
 * *ms (may be NULL) gets the kernel time. Returns 0, -1 (invalid arguments or
 * a CUDA error) or -2 (the completion wait ran out).
 */
int qcx_mma_selftest(int M, int N, int K, const float* A, int ta, const float* B, int tb, float* C, int reps,
                     float* ms);

/*
 * Self-check of the FP32 eigensolver of the SCC kernel's FP32 iterations (no
 * counterpart in the reference: it checks the cyclic parallel Jacobi alone).
 * One CTA of the SCC kernel's shape diagonalises the symmetric n x n matrix A
 * (row major, n <= 256) as the SCC does; warm = 1 starts from the orthonormal
 * rows in V (the basis A is expressed in), 0 from the identity. On return
 * Aout holds the rotated matrix (eigenvalues on the diagonal), V the
 * eigenvectors as rows, *sweeps the sweeps used (-1: max_sweeps were not
 * enough). Returns 0 or -1 (invalid arguments or a CUDA error).
 */
int qcx_jacobi32_selftest(int n, const float* A, float* Aout, float* V, int warm, double reltol, int max_sweeps,
                          int* sweeps);

/*
 * Ground-state sampling file qcxms.gs, as md writes it during the sampling run
 * (it = 0, src/md.f90:150-153, 379-385): the first line is nmax (list-directed,
 * a blank and 11 columns), then one record per MD loop top, each a line per
 * atom with x y z vx vy vz in Bohr and atomic units, format (6d16.8). xyz and
 * vel are [nrec][nat][3].
 */
int qcx_write_gs(const char* path, int nmax, int nat, int nrec, const double* xyz, const double* vel);

/*
 * One line of the fragment results file qcxms.res, as manage_fragments writes
 * it (src/write_fragments.f90:392-447, format (F10.7,i3,2i5,2i2,2x,i3,2x,
 * 20(i4,i3))): the fragment's assigned charge fragchrg3, the charge mchrg,
 * the trajectory number, for collision runs (cid != 0) the collision number,
 * the secondary-fragmentation number isec, the fragment number, and its
 * composition: nel elements in order of atomic number z[] with their counts
 * count[] (fragmass, src/fragments.f90:10-84). Electron-impact records have
 * no collision number, so the same format takes their items one position
 * earlier, as the reference's output does. Writes a NUL-terminated line of at
 * most len bytes and returns its length, or -1.
 */
int qcx_format_res(int cid, double fragchrg3, int mchrg, int itrj, int icoll, int isec, int ifrag, int nel,
                   const int32_t* z, const int32_t* count, char* line, int len);

/*
 * MO spectrum path: get_xtb_egrad(..., spec_calc=.true.) (src/tblite.f90:
 * 153-166) hands the converged orbitals to write_qmo (src/mo_energ.f90:7-80).
 *
 * qcx_batch_set_keep_mo(b, 1) makes the FP64 SCC (qcx_batch_set_precision(b,
 * 0)) keep its last orbitals on the device; after qcx_batch_egrad,
 * qcx_batch_mo_populations returns for molecule mol the orbital energies
 * emo[nao] (Eh, ascending), the occupations focc[nao] (0..2), the Mulliken
 * populations qmo[nao][nat] of every orbital on every atom as write_qmo forms
 * them (sum over the atom's AOs j and all AOs l of C(j,k) C(l,k) S(j,l), plus
 * 1e-10, each orbital's row divided by its sum over the atoms) and ihomo =
 * max(homo, 1), homo = floor(nel / 2), the aufbau count of one spin channel
 * of the spin-restricted wavefunction. Any output pointer may be NULL.
 * Returns nao, or -1 (no keep_mo, mixed precision or a CUDA error).
 */
int qcx_batch_set_keep_mo(qcx_batch* b, int on);
int qcx_batch_mo_populations(qcx_batch* b, int mol, double* emo, double* focc, double* qmo, int32_t* ihomo);

/*
 * get_xtb_egrad(spec_calc=.true.) for one structure, as getspec calls it
 * through eqm (src/mo_spec.f90:74): the FP64 single point (no checkqc), its
 * energy, nao, ihomo and the quantities of qcx_batch_mo_populations. emo and
 * focc hold max_nao values, qmo max_nao * nat. Returns 0, 5 (method not
 * implemented) or -1 (failed calculation, or more than max_nao orbitals:
 * *nao is set then).
 */
int qcx_mo_spectrum(int method, int nat, const int32_t* num, const double* xyz, int charge, int multiplicity,
                    double etemp, double* energy, int32_t* nao, int32_t* ihomo, double* emo, double* focc,
                    double* qmo, int max_nao);

/*
 * The two files of write_qmo (src/mo_energ.f90:26-79); either path may be
 * NULL. mspec_path (qcxms.Mspec.tbxtb): nao and ihomo list-directed, then per
 * orbital an empty line, (i3,1x,f10.3) the orbital number and emo in eV,
 * (1x,f6.2) focc and (10(1x,f6.2)) the populations in percent. tmp_path
 * (tmp.mspec, read back by readpopmo, src/mo_energ.f90:82-107): nao, ihomo,
 * then per orbital emo in eV, focc and the nat populations, one list-directed
 * item per line in gfortran's layout (17 significant digits). emo in Eh as
 * qcx_batch_mo_populations returns it. Returns 0 or -1.
 */
int qcx_write_qmo(const char* tmp_path, const char* mspec_path, int nat, int nao, int ihomo, const double* emo,
                  const double* focc, const double* qmo);

/*
 * Allocation-free variant of qcx_egrad for callers that cannot call
 * cudaMalloc (for example a host program whose device memory belongs to
 * another runtime's capped pool, or a path that must not trigger the device
 * synchronisation an allocation implies). It has no counterpart in the
 * reference. Same arguments, meaning and return codes as qcx_egrad, but all
 * device scratch is one static __device__ array of about 6 MB that every
 * GPU loading the library keeps until the process exits; nothing is
 * allocated on the device or the host heap. Limits: QCX_NOALLOC_MAX_ATOMS
 * atoms and QCX_NOALLOC_MAX_NAO atomic orbitals; larger inputs return -1
 * with the reason on stderr and in qcx_last_error(). The first call on a
 * device uploads the parameters into the array; make that first call before
 * any stream capture. Every call looks up the array's device address and
 * checks a marker word, so a call after cudaDeviceReset uploads them again.
 * Calls share the array: calls that overlap on the GPU race (one process
 * serialises its own calls on the host).
 */
#define QCX_NOALLOC_MAX_ATOMS 64
#define QCX_NOALLOC_MAX_NAO 160
int qcx_egrad_noalloc(int method, int nat, const int32_t* num, const double* xyz, int charge, int multiplicity,
                      double etemp, double* energy, double* grad, double* qat);

#ifdef __cplusplus
}
#endif
#endif
