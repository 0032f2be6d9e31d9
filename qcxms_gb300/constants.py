"""Unit conversions, masses and radii used on the trajectory-step path.

Values follow QCxMS so that MD bookkeeping matches it bit for bit:
``src/xtb_mctc_convert.f90:24-54`` (unit conversions), ``src/xtb_mctc_constants.f90:35``
(kB), ``src/atomic_masses.f90:24-30`` (NIST standard atomic weights, Z <= 18),
``src/covalent_radii.f90:86-89`` (the ``Rad`` table used for fragment detection).
"""
AUTOAA = 0.52917726
AATOAU = 1.0 / AUTOAA
AUTOEV = 27.21138505
FSTOAU = 41.3413733365614
KB_AU = 3.166808578545117e-06  # Hartree per Kelvin
AMUTOKG = 1.660539040e-27
METOKG = 9.10938356e-31
AMUTOAU = AMUTOKG * (1.0 / METOKG)

# standard atomic weights (amu), Z = 1..18
_AMU = [0.0, 1.00794075, 4.00260193, 6.94003660, 9.01218307, 10.81102805, 12.01073590,
        14.00670321, 15.99940492, 18.99840316, 20.18004638, 22.98976928, 24.30505162,
        26.98153853, 28.08549871, 30.97376200, 32.06478741, 35.45293758, 39.94779856]
MASS_AU = [m * AMUTOAU for m in _AMU]

# Mass of the collision gas atom of the CID runs, gas%mIatom (src/input.f90:512-557).
# The reference writes it as a default-real literal times amutoau, e.g.
# `39.948 * amutoau` for Ar (src/input.f90:531): the literal is a single-precision
# number, promoted to double for the product (the build sets no -fdefault-real-8).
# It is not the standard atomic weight of MASS_AU. Keys: atomic number (N2 counts
# per atom, as cid.f90:660-666 places two N atoms of this mass).
_GAS_AMU_LITERAL = {2: 4.002, 7: 14.007, 10: 20.18, 18: 39.948}


def gas_mass_au(z):
    import numpy as np
    return float(np.float32(_GAS_AMU_LITERAL[z])) * AMUTOAU


# Rad (Angstrom) of QCxMS for Z = 1..18, bond criterion r < rcut * (Rad_i + Rad_j) / 2
_RAD_AA = [0.0, 0.32, 0.37, 1.30, 0.99, 0.84, 0.75, 0.71, 0.64, 0.60, 0.62,
           1.60, 1.40, 1.24, 1.14, 1.09, 1.04, 1.00, 1.01]
RAD_AU = [r * AATOAU for r in _RAD_AA]

SYMBOLS = ["", "H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne",
           "Na", "Mg", "Al", "Si", "P", "S", "Cl", "Ar"]
MAXZ = 18


def symbol_to_z(sym):
    s = sym.strip().capitalize()
    return SYMBOLS.index(s)
