"""Small fixed and seeded test structures (Bohr)."""
import numpy as np

from qcxms_gb300 import molgen
from qcxms_gb300.constants import AATOAU


def h2o_cation():
    return np.array([8, 1, 1]), np.array([[0.0, 0.0, 0.0], [0.0, 1.4, 1.1], [0.2, -1.5, 1.0]]), 1


def ch2o_cation():
    return (np.array([6, 1, 1, 8]), np.array([[0, 0, 0], [0, 1.9, 0.8], [0.2, -1.8, 1.0], [2.5, 0.1, 0.3]], float), 1)


def h2s_ch_cation():
    return (np.array([16, 1, 6, 1]), np.array([[0, 0, 0], [0, 2.4, 0.8], [3.2, -0.4, 0.4], [4.0, 1.4, 0.3]], float), 1)


def argon_h2o():
    Z, xyz, c = h2o_cation()
    return np.concatenate([Z, [18]]), np.concatenate([xyz, [[4.5, 0.3, -2.0]]]), c


def h2_cation():
    return np.array([1, 1]), np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 2.0]]), 1


def single_atom():
    return np.array([8]), np.zeros((1, 3)), 1


def c6h12o2():
    Z, xyz = molgen.c6h12o2()
    return Z, xyz, 1


def random_chno(nat, seed):
    Z, xyz = molgen.random_chno(nat, seed)
    return Z, xyz, 1


ALL_SMALL = {
    "h2o+": h2o_cation,
    "ch2o+": ch2o_cation,
    "h2s-ch+": h2s_ch_cation,
    "h2o+ar": argon_h2o,
    "h2+": h2_cation,
    "o+": single_atom,
}
