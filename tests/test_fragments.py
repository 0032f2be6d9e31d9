"""Fragment assignment (src/fragments.f90:93-182, fragment_structure, called by
md.f90:450 every step with rcut = 3.0, at1 = 1, at2 = 0).

CPU: the oracle restatement on constructed cases with a known answer. GPU: the
CUDA kernel against the oracle, bit-exact, on dissociating geometries."""
import numpy as np
import pytest

import oracle
import qcxms_gb300 as qg
from qcxms_gb300 import molgen

AA = 1.0 / 0.52917726  # Angstrom -> Bohr, src/xtb_mctc_convert.f90:24-25


def _two_waters(sep_aa):
    Z = [8, 1, 1, 8, 1, 1]
    w = np.array([[0, 0, 0], [0.96, 0, 0], [-0.24, 0.93, 0]])
    xyz = np.concatenate([w, w + [sep_aa, 0, 0]]) * AA
    return np.array(Z), xyz


@pytest.fixture(scope="module")
def olib(oracle_lib):
    return oracle


def test_oracle_known_cases(oracle_lib):
    Z, xyz = _two_waters(10.0)
    frag, nf = oracle.fragments(Z, xyz)
    assert nf == 2 and list(frag) == [1, 1, 1, 2, 2, 2]
    # bonded at rcut 3 when close (H...O 1.34 A < 1.5 (0.32 + 0.64) A): one fragment
    Z, xyz = _two_waters(2.3)
    assert oracle.fragments(Z, xyz)[1] == 1
    # everything one fragment with at1 = at2 = 0
    Z, xyz = _two_waters(10.0)
    frag, nf = oracle.fragments(Z, xyz, at1=0, at2=0)
    assert nf == 1 and (frag == 1).all()
    # fragment 1 is at1's; the others follow their lowest atom
    frag, nf = oracle.fragments(Z, xyz, at1=4)
    assert list(frag) == [2, 2, 2, 1, 1, 1]
    # ignoring the only bond of a diatomic splits it
    Zd, xd = np.array([1, 1]), np.array([[0, 0, 0], [0.74 * AA, 0, 0]])
    assert oracle.fragments(Zd, xd)[1] == 1
    assert list(oracle.fragments(Zd, xd, at1=1, at2=2)[0]) == [1, 2]


def _dissociating(n, seed):
    Z, xyz = molgen.random_chno(n, seed)
    rng = np.random.default_rng(seed)
    xyz = np.asarray(xyz, dtype=np.float64).reshape(-1, 3).copy()
    # pull random subsets apart so that some bonds sit near the rcut threshold
    for _ in range(3):
        sel = rng.random(len(Z)) < 0.4
        xyz[sel] += rng.normal(0, 1, 3) / np.linalg.norm(rng.normal(0, 1, 3)) * rng.uniform(1.0, 8.0)
    return np.asarray(Z), xyz


@pytest.mark.gpu
def test_gpu_fragments_bit_exact(gpu, oracle_lib):
    mols = []
    for s in range(40):
        Z, xyz = _dissociating(5 + (s * 7) % 36, 500 + s)
        mols.append({"Z": Z, "xyz": xyz, "charge": 1})
    b = qg.Batch(mols)
    off = np.concatenate([[0], np.cumsum([len(m["Z"]) for m in mols])])
    for rcut, at1, at2 in [(3.0, 1, 0), (1.2, 1, 0), (1.5, 2, 0), (3.0, 1, 2), (1.0, 0, 0)]:
        frag, nfrag = b.fragments(rcut, at1, at2)
        multi = 0
        for i, m in enumerate(mols):
            ref, nref = oracle.fragments(m["Z"], m["xyz"], rcut, at1, at2)
            assert nfrag[i] == nref
            assert np.array_equal(frag[off[i]:off[i + 1]], ref)
            multi += nref > 1
        if rcut < 2.0 and at1:
            assert multi > 5  # the set really exercises several fragments
