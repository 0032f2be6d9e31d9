"""Seeded synthetic molecules and initial velocities for the trajectory workloads.

No public dataset is involved: every structure is generated from a seed.
Heavy atoms form a random tree (or a chain) with 1.45 Angstrom bonds, hydrogens
are attached at 1.09 Angstrom, and every coordinate gets Gaussian jitter.
"""
import numpy as np

from . import constants
from .constants import AATOAU, KB_AU, MASS_AU

VALENCE = {1: 1, 6: 4, 7: 3, 8: 2, 9: 1, 15: 3, 16: 2, 17: 1, 14: 4, 5: 3}


def _place(rng, xyz, parent, bond, ntry=256):
    """Put a new atom at ``bond`` from ``parent``, as far as possible from all others."""
    v = rng.normal(size=(ntry, 3))
    v /= np.linalg.norm(v, axis=1)[:, None]
    cand = xyz[parent] + bond * v
    others = [k for k in range(len(xyz)) if k != parent]
    if not others:
        return cand[0]
    o = np.asarray([xyz[k] for k in others])
    dmin = np.min(np.linalg.norm(cand[:, None, :] - o[None, :, :], axis=2), axis=1)
    return cand[int(np.argmax(dmin))]


def build_molecule(heavy, n_h, rng, chain=False, bond_heavy=1.45, bond_h=1.09, jitter=0.05):
    """Return (Z, xyz[Bohr]) for the given heavy-atom list and hydrogen count."""
    Z = list(heavy)
    xyz = [np.zeros(3)]
    nbond = [0] * len(heavy)
    for i in range(1, len(heavy)):
        if chain:
            parent = i - 1
        else:
            free = [j for j in range(i) if nbond[j] < VALENCE.get(heavy[j], 4)]
            parent = int(rng.choice(free)) if free else int(rng.integers(0, i))
        xyz.append(_place(rng, xyz, parent, bond_heavy))
        nbond[parent] += 1
        nbond[i] += 1
    k = 0
    for _ in range(n_h):
        free = [j for j in range(len(heavy)) if nbond[j] < VALENCE.get(heavy[j], 4)]
        if free:
            parent = free[k % len(free)]
            k += 1
        else:
            parent = int(rng.integers(0, len(heavy)))
        xyz.append(_place(rng, xyz, parent, bond_h))
        nbond[parent] += 1
        Z.append(1)
    xyz = np.array(xyz) + rng.normal(scale=jitter, size=(len(Z), 3))
    return np.array(Z, dtype=np.int32), xyz * AATOAU


def c6h12o2(seed=1234):
    """The 20-atom C6H12O2 chain (6 C + 2 O heavy-atom chain, 12 H)."""
    rng = np.random.default_rng(seed)
    heavy = [6, 6, 6, 8, 6, 6, 8, 6]
    return build_molecule(heavy, 12, rng, chain=True)


def random_chno(nat, seed, fractions=((6, 0.35), (1, 0.5), (7, 0.05), (8, 0.1))):
    """Random C/H/N/O molecule with ``nat`` atoms and at least one heavy atom."""
    rng = np.random.default_rng(seed)
    elems = np.array([e for e, _ in fractions])
    p = np.array([f for _, f in fractions])
    p = p / p.sum()
    draw = rng.choice(elems, size=nat, p=p)
    heavy = [int(z) for z in draw if z != 1]
    if not heavy:
        heavy = [6]
    n_h = nat - len(heavy)
    return build_molecule(heavy, n_h, rng)


def masses(Z):
    return np.array([MASS_AU[int(z)] for z in Z])


def maxwell_boltzmann(Z, temp, seed):
    """Velocities (Bohr / au time) at temperature ``temp`` with no centre-of-mass motion."""
    rng = np.random.default_rng(seed + 7919)
    m = masses(Z)
    v = rng.normal(size=(len(Z), 3)) * np.sqrt(KB_AU * temp / m)[:, None]
    vcom = (m[:, None] * v).sum(0) / m.sum()
    return v - vcom


def batch_workload(ntraj, nmin, nmax, seed0=0, tmin=1000.0, tmax=4000.0):
    """ntraj random C/H/N/O cations with N ~ U{nmin..nmax} and T0 ~ U(tmin, tmax)."""
    mols = []
    for t in range(ntraj):
        rng = np.random.default_rng(100000 + seed0 + t)
        nat = int(rng.integers(nmin, nmax + 1))
        temp = float(rng.uniform(tmin, tmax))
        Z, xyz = random_chno(nat, seed0 + t)
        vel = maxwell_boltzmann(Z, temp, seed0 + t)
        mols.append({"Z": Z, "xyz": xyz, "vel": vel, "mass": masses(Z), "charge": 1, "temp": temp})
    return mols


def random_cho(nat, seed):
    """Random C/H/O molecule (C 0.35, H 0.55, O 0.10) with ``nat`` atoms."""
    return random_chno(nat, seed, fractions=((6, 0.35), (1, 0.55), (8, 0.10)))


AR_Z = 18
EVTOAU = 1.0 / 27.21138505  # src/xtb_mctc_convert.f90:28-29


def cid_workload(ntraj, nmin=10, nmax=80, seed0=0, e_lab_ev=40.0, bmax_aa=2.0, temp=500.0, gap_aa=4.0):
    """Collision-induced dissociation set-up: a C/H/N/O/S cation and one Ar atom.

    The ion (internal Maxwell-Boltzmann velocities at ``temp``) moves with lab-frame
    kinetic energy ``e_lab_ev`` towards an Ar atom at rest, offset sideways by an
    impact parameter b ~ U(0, bmax). As in the reference collision set-up
    (src/cid.f90:344-399, 512-620) the Ar atom is part of the electronic-structure
    system, so each trajectory is one molecule of N+1 atoms with charge +1.
    """
    mols = []
    for t in range(ntraj):
        rng = np.random.default_rng(700000 + seed0 + t)
        nat = int(rng.integers(nmin, nmax + 1))
        Z, xyz = random_chno(nat, 50000 + seed0 + t,
                             fractions=((6, 0.30), (1, 0.50), (7, 0.05), (8, 0.10), (16, 0.05)))
        m = masses(Z)
        com = (m[:, None] * xyz).sum(0) / m.sum()
        xyz = xyz - com
        rmax = np.linalg.norm(xyz, axis=1).max()
        u = rng.normal(size=3)
        u /= np.linalg.norm(u)
        w = rng.normal(size=3)
        w -= w.dot(u) * u
        w /= np.linalg.norm(w)
        b = rng.uniform(0.0, bmax_aa) * AATOAU
        ar = (rmax + gap_aa * AATOAU) * u + b * w
        vel = maxwell_boltzmann(Z, temp, seed0 + t)
        vion = np.sqrt(2.0 * e_lab_ev * EVTOAU / m.sum())
        vel = vel + vion * u
        Zc = np.concatenate([Z, [AR_Z]]).astype(np.int32)
        # the gas atom's mass is gas%mIatom (src/input.f90:531), placed at mass0(nuc0) (src/cid.f90:657)
        mols.append({"Z": Zc, "xyz": np.vstack([xyz, ar]), "vel": np.vstack([vel, np.zeros(3)]),
                     "mass": np.concatenate([m, [constants.gas_mass_au(AR_Z)]]), "charge": 1, "temp": temp,
                     "impact_parameter": b})
    return mols


def fragmented(seed, nparts, spacing=25.0):
    """A trajectory end that has fallen apart: nparts random C/H/N/O molecules
    (3-12 atoms; a quarter of the parts lone H atoms) ``spacing`` Bohr apart,
    atom order shuffled so that the fragments interleave. ``frag`` holds the
    fragment numbers that fragment_structure (src/fragments.f90:93-182) gives
    at rcut 3.0, at1 = 1: the first atom's part is fragment 1, the others
    follow in the order of their lowest-numbered atom."""
    rng = np.random.default_rng(seed)
    Zs, xs, part = [], [], []
    for k in range(nparts):
        if rng.random() < 0.25:
            Z, x = np.array([1]), np.zeros((1, 3))
        else:
            Z, x = random_chno(int(rng.integers(3, 13)), 1000 * seed + k)
            x = np.asarray(x, dtype=np.float64).reshape(-1, 3)
            x = x - x.mean(0)
        Zs.append(np.asarray(Z))
        xs.append(x + np.array([spacing * k, rng.normal() * 3.0, rng.normal() * 3.0]))
        part += [k] * len(Z)
    Z, xyz, part = np.concatenate(Zs), np.concatenate(xs), np.array(part)
    perm = rng.permutation(len(Z))
    Z, xyz, part = Z[perm], xyz[perm], part[perm]
    number = {}
    for p in part:
        if p not in number:
            number[p] = len(number) + 1
    frag = np.array([number[p] for p in part], dtype=np.int32)
    return {"Z": Z, "xyz": xyz, "frag": frag}
