// MD bookkeeping and exit rules of a fragmentation run on the device.
//
// The MD loop of QCxMS (src/md.f90:285-682) does, per trajectory and step:
//   top     nstep += 1; T, running sums of T, Epot, Ekin and Etot; the energy
//           error Eerror = <Etot> - Etot; an exit when Epot == 0 (failed
//           energy call) or |Eerror| > 0.1 Eh (src/md.f90:288-342)
//   step    leapfrog + egrad (src/md.f90:388-396)
//   after   morestep reset and first-fragmentation time (src/md.f90:426-428);
//           fragment_structure at rcut 3.0 and the fragments' temperatures
//           (intenergy, src/md.f90:450-454, 715-741); the exit rules of an
//           electron-impact run (src/md.f90:456-462, 620-666) and the step
//           limit (src/md.f90:671-679).
// Here that bookkeeping runs as one thread per trajectory after the step's
// fragment kernel, inside the captured step graph, so no host round trip is
// needed per step. The arithmetic keeps the reference's operation order and
// its single-precision literals (0.5*3*n, 0.1, float(nstep)) with explicit
// roundings. The heating of the first nadd steps (impactscale, src/md.f90:439-441)
// runs here too, and, when switched on, the electronic temperature of every
// next evaluation (setetemp, src/md.f90:443-446). Not covered: the CID branch,
// averages for the output files.
#include <cuda_runtime.h>

#include "qcx_consts.h"
#include "qcx_kernels.h"

namespace qcx {

namespace {

// e / (0.5*3*n*kB) with 0.5*3*n evaluated in default (single) real, as the
// reference writes it (src/md.f90:289, 736)
__device__ double temp_of(double e, int n) {
  const float f = 1.5f * (float)n;
  return __ddiv_rn(e, __dmul_rn((double)f, QCX_KTOAU));
}

// energy of molecule mol for the bookkeeping: 0 after a failed evaluation,
// which is how the reference's loop sees a failed energy call (checkqc's
// rejections have already set the energy to 0)
__device__ double epot_of(const DevBatch& bt, int mol) {
  if (bt.status[mol] & kFailedEval) return 0.0;
  return bt.energy[(long long)mol * kNumEnergy + kETotal];
}

// window of the averaged structure: avdump = 50 steps (src/md.f90:89)
constexpr int kAvDump = 50;

// top of the loop (src/md.f90:286-362); returns true when the run ends here.
// xyz/avxyz: this molecule's coordinates and running coordinate sum.
__device__ bool md_top(MdState& s, double epot, double ekin, int nuc, const double* xyz, double* avxyz, int lane,
                       int nlanes) {
  s.nstep += 1;
  const double t = temp_of(ekin, nuc);
  s.tav = __dadd_rn(s.tav, t);
  s.epav = __dadd_rn(s.epav, epot);
  s.ekav = __dadd_rn(s.ekav, ekin);
  // the running mean of Etot starts after the nadd heating steps
  double eav;
  if (s.nstep > s.nadd) {
    s.edum = __dadd_rn(__dadd_rn(s.edum, epot), ekin);
    eav = __ddiv_rn(s.edum, (double)(float)(s.nstep - s.nadd));
  } else {
    eav = __dadd_rn(epot, ekin);
  }
  s.eerror = __dsub_rn(__dsub_rn(eav, epot), ekin);
  if (s.nfrag == 1) s.fragT[0] = __ddiv_rn(s.tav, (double)s.nstep);
  const bool err = epot == 0.0 || fabs(s.eerror) > (double)0.1f;
  if (err) {
    // with fragments already formed the trajectory is taken anyway (isec = 1)
    s.mdok = (s.nfrag > 1 && s.nfrag <= 4) ? 1 : 0;
    s.done = 1;
    return true;
  }
  // averaged structure over the last avdump steps (src/md.f90:352-362)
  if (s.kdump > kAvDump - 1) {
    s.kdump = 0;
    for (int k = lane; k < 3 * nuc; k += nlanes) avxyz[k] = 0.0;
  }
  for (int k = lane; k < 3 * nuc; k += nlanes) avxyz[k] = __dadd_rn(avxyz[k], xyz[k]);
  return false;
}

// impactscale (src/impact.f90:12-55): grow the scaling factor in steps of
// 0.0002 until the kinetic energy reaches eimp * ff + e0 (within 0.001 Eh) or
// 20000 steps pass, then scale the velocities. Returns false after 20000 steps
// (the reference stops the program there). One warp: the lanes form the
// per-atom terms m |v (1 + velof scal)|^2 (ekinet, src/mdinit.f90:57-76) into
// terms[], lane 0 adds them in atom order, so the sum rounds as the reference's.
__device__ bool impact_scale(const DevBatch& bt, const MolDesc& md, const double* velof, double eimp, double ff,
                             double e0, double* terms, int lane) {
  const double esoll = __dadd_rn(__dmul_rn(eimp, ff), e0);
  double scal = 0.0;
  int k = 0;
  for (;;) {
    ++k;
    for (int i = lane; i < md.nat; i += 32) {
      const long long a = md.atom_off + i;
      const double f = __dadd_rn(1.0, __dmul_rn(velof ? velof[a] : 1.0, scal));
      const double* v = bt.vel + 3 * a;
      const double x = __dmul_rn(v[0], f), y = __dmul_rn(v[1], f), z = __dmul_rn(v[2], f);
      const double v2 = __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
      terms[i] = __dmul_rn(bt.mass[a], v2);
    }
    __syncwarp();
    double e = 0.0;
    if (lane == 0) {
      for (int i = 0; i < md.nat; ++i) e = __dadd_rn(e, terms[i]);
      e = __dmul_rn(e, 0.5);
    }
    e = __shfl_sync(0xffffffffu, e, 0);
    __syncwarp();  // terms[] is rewritten by the next pass
    scal = __dadd_rn(scal, (double)0.0002f);
    if (!(__dsub_rn(esoll, e) > (double)0.001f && k < 20000)) break;
  }
  for (int i = lane; i < md.nat; i += 32) {
    const long long a = md.atom_off + i;
    const double f = __dadd_rn(1.0, __dmul_rn(velof ? velof[a] : 1.0, scal));
    double* v = bt.vel + 3 * a;
    for (int d = 0; d < 3; ++d) v[d] = __dmul_rn(v[d], f);
  }
  __syncwarp();
  return k < 20000;
}

}  // namespace

// Start of the loop: Ekin of the current velocities (ekinet,
// src/mdinit.f90:57-76), Epot of the last evaluation, then the first top.
__global__ void k_md_begin(DevBatch bt, MdState* st, const double* heat, double* avxyz, const double* etemp0) {
  const int mol = blockIdx.x * blockDim.x + threadIdx.x;
  if (mol >= bt.nmol) return;
  MdState s = {};
  s.nfrag = 1;
  s.etemp = etemp0 ? etemp0[mol] : -1.0;
  s.kdump = kAvDump;
  if (heat) {
    s.eimp = heat[3 * mol];
    s.fadd = heat[3 * mol + 1];
    s.nadd = (int)heat[3 * mol + 2];
  }
  const MolDesc md = bt.mol[mol];
  if (!bt.active[mol]) {
    s.done = 1;
    st[mol] = s;
    return;
  }
  double ek = 0.0;
  for (int i = 0; i < md.nat; ++i) {
    const double* v = bt.vel + 3LL * (md.atom_off + i);
    const double v2 = __dadd_rn(__dadd_rn(__dmul_rn(v[0], v[0]), __dmul_rn(v[1], v[1])), __dmul_rn(v[2], v[2]));
    ek = __dadd_rn(ek, __dmul_rn(bt.mass[md.atom_off + i], v2));
  }
  ek = __dmul_rn(ek, 0.5);
  s.ekinstart = ek;
  const double epot = epot_of(bt, mol);
  if (epot == 0.0) {
    s.done = 1;  // src/md.f90:185: no run without a starting energy
  } else {
    md_top(s, epot, ek, md.nat, bt.xyz + 3LL * md.atom_off, avxyz + 3LL * md.atom_off, 0, 1);
  }
  if (s.done) bt.active[mol] = 0;
  st[mol] = s;
}

// After a step (leapfrog, egrad, fragment numbers of the new coordinates):
// the end of the loop body, then the top of the next iteration. One warp per
// trajectory: every lane keeps the same copy of the state (the scalar
// bookkeeping runs redundantly), the per-atom work is split over the lanes and
// lane 0 writes the state.
constexpr int kRulesWarps = 4;

__global__ void __launch_bounds__(32 * kRulesWarps) k_md_rules(DevBatch bt, MdState* st, const int* frag,
                                                               const int* nfrag, const double* velof,
                                                               double* avxyz, MdRules r) {
  extern __shared__ double md_terms[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int idx = blockIdx.x * kRulesWarps + warp;
  if (idx >= bt.nmol) return;
  const int mol = bt.order ? bt.order[idx] : idx;
  double* terms = md_terms + (size_t)warp * r.max_nat;
  MdState s = st[mol];
  if (s.done || scc_pending(bt, mol)) return;  // a pending SCC: the step has not happened yet
  const MolDesc md = bt.mol[mol];
  s.ttime = __dadd_rn(s.ttime, __ddiv_rn(r.tstep, QCX_FSTOAU));
  s.kdump += 1;  // src/md.f90:400
  // src/md.f90:426-428, with the fragment count of the previous step
  if (s.nfrag == 1) s.morestep = 0;
  if (s.nfrag > 1 && s.dtime < 1.0e-6) s.dtime = __ddiv_rn(s.ttime, 1000.0);
  // heating while not fragmented (src/md.f90:439-441), before the fragment check
  if (s.nstep <= s.nadd && s.nfrag == 1) {
    if (!impact_scale(bt, md, velof, s.eimp, __dmul_rn(s.fadd, (double)s.nstep), s.ekinstart, terms, lane)) {
      s.heat_failed = 1;
      s.done = 1;
      if (lane == 0) {
        bt.active[mol] = 0;
        st[mol] = s;
      }
      return;
    }
  }
  // electronic temperature of the next evaluation (src/md.f90:443-446), with
  // the previous step's fragment count: dum = eimp - eimp*float(nstep)/float(nadd),
  // evaluated left to right in double (float(n) converts exactly);
  // kT = etemp * ktoau (src/tblite.f90:133)
  if (r.etemp_on) {
    const double a = __dmul_rn(s.eimp, (double)(float)s.nstep);
    const double dum = __dsub_rn(s.eimp, __ddiv_rn(a, (double)(float)s.nadd));
    s.etemp = setetemp(s.nfrag, dum, r.ax, r.ieetemp);
    if (lane == 0) const_cast<MolDesc*>(bt.mol)[mol].kT = __dmul_rn(s.etemp, QCX_KTOAU);
  }
  const int nf = nfrag[mol];
  s.nfrag = nf;
  if (nf > 1) {
    // intenergy (src/md.f90:715-741) for the first 10 fragments (its arrays hold 10)
    double eint[10];
    int cnt[10];
    for (int j = 0; j < 10; ++j) {
      eint[j] = 0.0;
      cnt[j] = 0;
    }
    for (int i = 0; i < md.nat; ++i) {
      const int j = frag[md.atom_off + i] - 1;
      if (j < 0 || j >= 10) continue;
      const double* v = bt.vel + 3LL * (md.atom_off + i);
      const double v2 = __dadd_rn(__dadd_rn(__dmul_rn(v[0], v[0]), __dmul_rn(v[1], v[1])), __dmul_rn(v[2], v[2]));
      eint[j] = __dadd_rn(eint[j], __dmul_rn(__dmul_rn(0.5, bt.mass[md.atom_off + i]), v2));
      cnt[j] += 1;
    }
    for (int j = 0; j < nf && j < 10; ++j) s.fragT[j] = temp_of(eint[j], cnt[j]);
  }
  bool exit_now = false;
  if (nf > 6) {
    exit_now = true;  // "More than 6 fragments. Error?" (mdok stays 0)
  } else if (nf > r.nfragexit) {
    s.fragstate = 1;
    s.mdok = 1;
    exit_now = true;
  } else {
    s.fconst = nf >= 2 ? s.fconst + 1 : 0;
    if (s.fconst > 1000) {
      s.fragstate = 2;
      s.mdok = 1;
      exit_now = true;
    } else if (nf >= r.nfragexit) {
      s.morestep += 1;
      if (s.morestep > r.more) {
        s.fragstate = 1;
        s.mdok = 1;
        exit_now = true;
      }
    }
  }
  if (!exit_now && s.nstep >= r.max_steps) {
    s.fragstate = 1;
    s.mdok = 1;
    exit_now = true;
  }
  if (exit_now) {
    s.done = 1;
  } else {
    md_top(s, epot_of(bt, mol), bt.ekin[mol], md.nat, bt.xyz + 3LL * md.atom_off, avxyz + 3LL * md.atom_off, lane,
           32);
  }
  if (lane == 0) {
    if (s.done) bt.active[mol] = 0;
    st[mol] = s;
  }
}

void launch_md_begin(const DevBatch& bt, MdState* st, const double* heat, double* avxyz, const double* etemp0,
                     cudaStream_t stream) {
  k_md_begin<<<(bt.nmol + 127) / 128, 128, 0, stream>>>(bt, st, heat, avxyz, etemp0);
}

void launch_md_rules(const DevBatch& bt, MdState* st, const int* frag, const int* nfrag, const double* velof,
                     double* avxyz, const MdRules& r, cudaStream_t stream) {
  k_md_rules<<<(bt.nmol + kRulesWarps - 1) / kRulesWarps, 32 * kRulesWarps,
               sizeof(double) * kRulesWarps * r.max_nat, stream>>>(bt, st, frag, nfrag, velof, avxyz, r);
}

}  // namespace qcx
