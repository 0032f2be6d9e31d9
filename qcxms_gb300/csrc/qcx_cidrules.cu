// Stop rules of the collision MD (CID) on the device.
//
// The collision loop of QCxMS (src/cid.f90:739-1052) advances the ion plus one
// gas atom (the last atom) and, per step after leapfrog + egrad: ends on a
// failed energy call; takes the ion's centre-of-mass speed from its
// displacement (src/cid.f90:769-779), the ion's internal temperature and its
// running mean (src/cid.f90:783-793) and the collision energy in the centre of
// mass frame (calc_ECOM, src/cid.f90:1209-1215); counts the ion's fragments
// (fragment_structure on the ion's atoms, src/cid.f90:800); every 10 steps
// measures the gas atom's distance from the ion's centre of mass and, once it
// has grown for 5 checks in a row, marks the collision and ends the run
// 800 * (2 tstep in fs) steps later (src/cid.f90:955-985); after a
// fragmentation that follows the collision the end moves to add_steps after
// it (src/cid.f90:988-1001, add_steps from the ion size, src/cid.f90:276-278);
// and stops at that step (src/cid.f90:1030-1036). It also keeps the averaged
// structures that the fragment IPs take (src/cid.f90:743-746, 802-909, the
// result at 1095-1101). One thread per trajectory, the reference's operation
// order with explicit roundings. Not covered: the output files.
#include <cuda_runtime.h>

#include <cmath>

#include "qcx_consts.h"
#include "qcx_kernels.h"

namespace qcx {

namespace {

// src/xtb_mctc_convert.f90:27,55,63
constexpr double kAutoEV = 27.21138505;
constexpr double kAutoFs = 1.0 / QCX_FSTOAU;
constexpr double kMsToAu = 1.0 / 2.18769126364e6;

// center_of_mass (src/utility.f90:541-562) of the first nuc atoms
__device__ void com(const DevBatch& bt, const MolDesc& md, int nuc, double cm[3]) {
  double tm = 0.0;
  cm[0] = cm[1] = cm[2] = 0.0;
  for (int i = 0; i < nuc; ++i) {
    const long long a = md.atom_off + i;
    const double m = bt.mass[a];
    for (int d = 0; d < 3; ++d) cm[d] = __dadd_rn(cm[d], __dmul_rn(m, bt.xyz[3 * a + d]));
    tm = __dadd_rn(tm, m);
  }
  for (int d = 0; d < 3; ++d) cm[d] = __ddiv_rn(cm[d], tm);
}

__device__ double norm3(double x, double y, double z) {
  return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z)));
}

// distArCOM (src/cid.f90:1124-1139): the gas atom's distance from cm
__device__ double gas_distance(const DevBatch& bt, const MolDesc& md, const double cm[3]) {
  const double* g = bt.xyz + 3LL * (md.atom_off + md.nat - 1);
  return norm3(__dsub_rn(g[0], cm[0]), __dsub_rn(g[1], cm[1]), __dsub_rn(g[2], cm[2]));
}

// gradfail of egrad: a failed calculation or a result checkqc rejects in any of
// its three tests (src/iniqm.f90:650-654); cid.f90:763-766 stops the run on it
__device__ bool failed_eval(const DevBatch& bt, int mol) {
  return (bt.status[mol] & (kFailedEval | kCheckqcFailed)) != 0;
}

}  // namespace

__global__ void k_cid_begin(DevBatch bt, CidState* st, double* cav, CidRules r) {
  const int mol = blockIdx.x * blockDim.x + threadIdx.x;
  if (mol >= bt.nmol) return;
  const MolDesc md = bt.mol[mol];
  CidState s = {};
  s.total_steps = r.ntot;
  // avxyz = avxyz2 = 0 (src/cid.f90:244-245), check_fragmented = 1 (:265);
  // count_average starts .false. (its initialiser, :147); save_natf has no
  // initial value in the reference and starts at 0 here
  s.check_fragmented = 1;
  for (long long e = 9LL * md.atom_off; e < 9LL * (md.atom_off + md.nat); ++e) cav[e] = 0.0;
  const int nuc = md.nat - 1;
  for (int i = 0; i < nuc; ++i) s.summass = __dadd_rn(s.summass, bt.mass[md.atom_off + i]);
  double cm[3];
  com(bt, md, nuc, cm);
  for (int d = 0; d < 3; ++d) s.old_cm[d] = cm[d];
  const double d0 = gas_distance(bt, md, cm);
  s.lowest = d0;
  s.highest = d0;
  s.nfrag = 1;
  if (!bt.active[mol] || nuc < 1) {
    s.done = 1;
    s.failed = 1;
    bt.active[mol] = 0;
  }
  st[mol] = s;
}

__global__ void k_cid_rules(DevBatch bt, CidState* st, const int* frag, const int* nfrag, double* cav, CidRules r) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= bt.nmol) return;
  const int mol = bt.order ? bt.order[idx] : idx;
  CidState s = st[mol];
  if (s.done || scc_pending(bt, mol)) return;  // a pending SCC: the step has not happened yet
  const MolDesc md = bt.mol[mol];
  const int nuc = md.nat - 1;
  s.nstep += 1;
  double* av = cav + 9LL * md.atom_off;  // per ion atom: avxyz, avxyz2, store_avxyz
  // a new window of the averaged structure every dumpavg = 50 loop tops (src/cid.f90:743-746)
  if (s.xyzavg_dump == 50) {
    s.xyzavg_dump = 0;
    for (int i = 0; i < nuc; ++i)
      for (int d = 0; d < 3; ++d) av[9 * i + d] = 0.0;
  }
  s.ttime = __dadd_rn(s.ttime, __dmul_rn(r.tstep, kAutoFs));
  s.distance_dump += 1;
  s.xyzavg_dump += 1;
  if (failed_eval(bt, mol)) {
    s.done = 1;
    s.failed = 1;
    bt.active[mol] = 0;
    st[mol] = s;
    return;
  }
  double cm[3];
  com(bt, md, nuc, cm);
  const double cm_out =
      norm3(__dsub_rn(cm[0], s.old_cm[0]), __dsub_rn(cm[1], s.old_cm[1]), __dsub_rn(cm[2], s.old_cm[2]));
  for (int d = 0; d < 3; ++d) s.old_cm[d] = cm[d];
  const double new_velo = s.nstep != 1 ? __ddiv_rn(__ddiv_rn(cm_out, r.tstep), kMsToAu) : 0.0;
  // ekinet of the ion's atoms (src/mdinit.f90:57-76)
  double ek = 0.0;
  for (int i = 0; i < nuc; ++i) {
    const double* v = bt.vel + 3LL * (md.atom_off + i);
    const double v2 = __dadd_rn(__dadd_rn(__dmul_rn(v[0], v[0]), __dmul_rn(v[1], v[1])), __dmul_rn(v[2], v[2]));
    ek = __dadd_rn(ek, __dmul_rn(bt.mass[md.atom_off + i], v2));
  }
  ek = __dmul_rn(ek, 0.5);
  const double x = __dmul_rn(new_velo, kMsToAu);
  const double e_velo = __dmul_rn(__dmul_rn(0.5, s.summass), __dmul_rn(x, x));
  const double ekd = __dsub_rn(ek, e_velo);
  s.new_temp = __ddiv_rn(__dmul_rn(2.0, ekd), __dmul_rn(__dmul_rn(3.0, QCX_KTOAU), (double)nuc));
  if (s.nstep == 1) s.new_temp = r.tinit;
  s.tav = __dadd_rn(s.tav, s.new_temp);
  s.m += 1;
  s.avgT = __ddiv_rn(s.tav, (double)s.m);
  // beta = m_gas / (m_gas + m_ion) (src/cid.f90:347)
  const double mgas = bt.mass[md.atom_off + nuc];
  s.ecom = __dmul_rn(__dmul_rn(__ddiv_rn(mgas, __dadd_rn(mgas, s.summass)), e_velo), kAutoEV);
  s.nfrag = nfrag[mol];
  // averaged structures (src/cid.f90:802-909): avxyz sums every step of the
  // window; after the ion has fallen into more fragments, avxyz2 sums up to
  // cnt_steps = 50 steps as long as the fragments keep their atom counts
  {
    const int nf = s.nfrag;
    const double* x = bt.xyz + 3LL * md.atom_off;
    for (int i = 0; i < nuc; ++i)
      for (int d = 0; d < 3; ++d) av[9 * i + d] = __dadd_rn(av[9 * i + d], x[3 * i + d]);
    if (nf > s.check_fragmented) {
      s.count_average = 1;
      s.check_fragmented = nf;
    }
    if (nf < s.check_fragmented && s.count_average) {
      s.cnt = 0;
      for (int i = 0; i < nuc; ++i)
        for (int d = 3; d < 9; ++d) av[9 * i + d] = 0.0;
      s.count_average = 0;
      s.check_fragmented = 1;
    }
    if (s.count_average) {
      s.cnt += 1;
      for (int i = 0; i < nuc; ++i)
        for (int d = 0; d < 3; ++d) {
          av[9 * i + 3 + d] = __dadd_rn(av[9 * i + 3 + d], x[3 * i + d]);
          av[9 * i + 6 + d] = __ddiv_rn(av[9 * i + 3 + d], (double)s.cnt);
        }
      // avg_frag_struc (src/analyse.f90:452-502): the atom count of every
      // fragment (its arrays hold 10 fragments)
      int natf[10];
      for (int k = 0; k < 10; ++k) natf[k] = 0;
      const int* lab = frag + md.atom_off;
      for (int i = 0; i < nuc; ++i)
        if (lab[i] >= 1 && lab[i] <= 10) natf[lab[i] - 1] += 1;
      const int nchk = nf < 10 ? nf : 10;
      for (int k = 0; k < nchk; ++k) {
        if (s.cnt == 1) s.save_natf[k] = natf[k];
        if (natf[k] != s.save_natf[k]) {
          // a fragment changed: the count starts again (src/cid.f90:860-866)
          s.cnt = 0;
          for (int i = 0; i < nuc; ++i)
            for (int d = 3; d < 9; ++d) av[9 * i + d] = 0.0;
          break;
        }
      }
      if (s.cnt == 50) {
        for (int i = 0; i < nuc; ++i)
          for (int d = 0; d < 3; ++d) {
            av[9 * i + 6 + d] = __ddiv_rn(av[9 * i + 3 + d], (double)s.cnt);
            av[9 * i + 3 + d] = 0.0;
          }
        s.cnt = 0;
        s.count_average = 0;
      }
    }
  }
  if (s.distance_dump == 10) {
    s.distance_dump = 0;
    const double dist = gas_distance(bt, md, cm);
    if (dist > s.highest) s.highest = dist;
    if (dist < s.lowest) s.lowest = dist;
    s.step_counter = s.lowest < dist ? s.step_counter + 1 : 0;
    if (s.step_counter == 5) {
      s.collided = 1;
      s.total_steps = s.nstep + (int)llround(__dmul_rn(800.0, __dmul_rn(__dmul_rn(2.0, r.tstep), kAutoFs)));
      s.tav = 0.0;
      s.m = 0;
    }
  }
  if (s.nfrag > 1 && s.collided && !s.fragmented) {
    const int add_steps = nuc >= 40 ? (nuc / 10) * 1000 : (nuc > 10 ? (nuc / 10) * 500 : 0);
    s.total_steps = s.nstep + add_steps;
    s.fragmented = 1;
  }
  if (s.nstep >= s.total_steps) s.done = 1;
  if (s.done) bt.active[mol] = 0;
  st[mol] = s;
}

void launch_cid_begin(const DevBatch& bt, CidState* st, double* cav, const CidRules& r, cudaStream_t stream) {
  k_cid_begin<<<(bt.nmol + 127) / 128, 128, 0, stream>>>(bt, st, cav, r);
}

void launch_cid_rules(const DevBatch& bt, CidState* st, const int* frag, const int* nfrag, double* cav,
                      const CidRules& r, cudaStream_t stream) {
  k_cid_rules<<<(bt.nmol + 127) / 128, 128, 0, stream>>>(bt, st, frag, nfrag, cav, r);
}

}  // namespace qcx
