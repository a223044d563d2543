"""Per-element Lennard-Jones parameters and species lookup.

The numeric table holds the per-element values (rmin [A], epsilon [eV], alpha) that the
reference ships as ppafm/defaults/atomtypes.ini (columns 1-5); parity of every force field
depends on using identical parameters.  `loadSpecies(path)` also reads a user file in the
same whitespace format, like ppafm/common.py:526-543.
"""

import os

import numpy as np

# (Z, symbol, rmin, epsilon, alpha)
_TABLE = [
    (1, "H", 1.4870, 0.000681, 1.80),
    (2, "He", 1.4815, 0.000945, 1.80),
    (3, "Li", 2.0000, 0.010000, 1.80),
    (4, "Be", 2.0000, 0.010000, 1.80),
    (5, "B", 2.0800, 0.003729, 1.80),
    (6, "C", 1.9080, 0.003729, 1.80),
    (7, "N", 1.7800, 0.007372, 1.80),
    (8, "O", 1.6612, 0.009106, 1.80),
    (9, "F", 1.7500, 0.002645, 1.80),
    (10, "Ne", 1.5435, 0.003643, 1.80),
    (11, "Na", 2.7700, 0.010000, 1.80),
    (12, "Mg", 2.4200, 0.010000, 1.80),
    (13, "Al", 2.4000, 0.010000, 1.80),
    (14, "Si", 1.9000, 0.025490, 1.80),
    (15, "P", 2.1000, 0.008673, 1.80),
    (16, "S", 2.0000, 0.010841, 1.80),
    (17, "Cl", 1.9480, 0.011491, 1.80),
    (18, "Ar", 1.8805, 0.012341, 1.80),
    (19, "K", 3.0200, 0.010000, 1.80),
    (20, "Ca", 2.7800, 0.010000, 1.80),
    (21, "Sc", 2.6200, 0.010000, 1.80),
    (22, "Ti", 2.4400, 0.010000, 1.80),
    (23, "V", 2.2700, 0.010000, 1.80),
    (24, "Cr", 2.2300, 0.010000, 1.80),
    (25, "Mn", 2.2500, 0.010000, 1.80),
    (26, "Fe", 2.2700, 0.010000, 1.80),
    (27, "Co", 2.2500, 0.010000, 1.80),
    (28, "Ni", 2.2300, 0.010000, 1.80),
    (29, "Cu", 2.2300, 0.010000, 1.80),
    (30, "Zn", 2.2400, 0.010000, 1.80),
    (31, "Ga", 2.4100, 0.010000, 1.80),
    (32, "Ge", 2.3200, 0.010000, 1.80),
    (33, "As", 2.2500, 0.010000, 1.80),
    (34, "Se", 2.1800, 0.010000, 1.80),
    (35, "Br", 2.2200, 0.013876, 1.80),
    (36, "Kr", 2.0000, 0.010000, 1.80),
    (37, "Rb", 3.1500, 0.010000, 1.80),
    (38, "Sr", 2.9400, 0.010000, 1.80),
    (39, "Y", 2.7100, 0.010000, 1.80),
    (40, "Zr", 2.5700, 0.010000, 1.80),
    (41, "Nb", 2.4600, 0.010000, 1.80),
    (42, "Mo", 2.3900, 0.010000, 1.80),
    (43, "Tc", 2.3700, 0.010000, 1.80),
    (44, "Ru", 2.3500, 0.010000, 1.80),
    (45, "Rh", 2.3200, 0.010000, 1.80),
    (46, "Pd", 2.3500, 0.010000, 1.80),
    (47, "Ag", 2.3700, 0.010000, 1.80),
    (48, "Cd", 2.3700, 0.010000, 1.80),
    (49, "In", 2.5300, 0.010000, 1.80),
    (50, "Sn", 2.4600, 0.010000, 1.80),
    (51, "Sb", 2.4100, 0.010000, 1.80),
    (52, "Te", 2.3600, 0.010000, 1.80),
    (53, "I", 2.3500, 0.017345, 1.80),
    (54, "Xe", 2.1815, 0.024344, 1.80),
    (55, "Cs", 3.3000, 0.010000, 1.80),
    (56, "Ba", 3.0500, 0.010000, 1.80),
    (57, "La", 2.8100, 0.010000, 1.80),
    (58, "Ce", 2.0000, 0.010000, 1.80),
    (59, "Pr", 2.0000, 0.010000, 1.80),
    (60, "Nd", 2.0000, 0.010000, 1.80),
    (61, "Pm", 2.0000, 0.010000, 1.80),
    (62, "Sm", 2.0000, 0.010000, 1.80),
    (63, "Eu", 2.0000, 0.010000, 1.80),
    (64, "Gd", 2.0000, 0.010000, 1.80),
    (65, "Tb", 2.0000, 0.010000, 1.80),
    (66, "Dy", 2.0000, 0.010000, 1.80),
    (67, "Ho", 2.0000, 0.010000, 1.80),
    (68, "Er", 2.0000, 0.010000, 1.80),
    (69, "Tm", 2.0000, 0.010000, 1.80),
    (70, "Yb", 2.0000, 0.010000, 1.80),
    (71, "Lu", 2.0000, 0.010000, 1.80),
    (72, "Hf", 2.5200, 0.010000, 1.80),
    (73, "Ta", 2.4200, 0.010000, 1.80),
    (74, "W", 2.3600, 0.010000, 1.80),
    (75, "Re", 2.3500, 0.010000, 1.80),
    (76, "Os", 2.3300, 0.010000, 1.80),
    (77, "Ir", 2.3400, 0.010000, 1.80),
    (78, "Pt", 2.3700, 0.010000, 1.80),
    (79, "Au", 2.4100, 0.010000, 1.80),
    (80, "Hg", 2.2500, 0.010000, 1.80),
    (81, "Tl", 2.5300, 0.010000, 1.80),
    (82, "Pb", 2.5300, 0.010000, 1.80),
    (83, "Bi", 3.5200, 0.010000, 1.80),
    (84, "Po", 2.0000, 0.010000, 1.80),
    (85, "At", 2.0000, 0.010000, 1.80),
    (86, "Rn", 2.0000, 0.010000, 1.80),]

SPECIES_DTYPE = [("rmin", np.float64), ("epsilon", np.float64), ("alpha", np.float64), ("atom", int), ("symbol", "|S10")]


def _default():
    return np.array([(r, e, a, z, s) for z, s, r, e, a in _TABLE], dtype=SPECIES_DTYPE)


def loadSpecies(fname=None):
    """Species table: the built-in one, or a file with rows 'rmin epsilon alpha Z symbol'."""
    if fname is None or not os.path.exists(fname):
        return _default()
    rows = []
    with open(fname) as f:
        for line in f:
            p = line.split()
            if len(p) >= 5:
                rows.append((float(p[0]), float(p[1]), float(p[2]), int(p[3]), p[4]))
    return np.array(rows, dtype=SPECIES_DTYPE)


def getFFdict(FFparams):
    """symbol (bytes) -> 1-based row index (common.py:806-811)."""
    return {ff[4]: i + 1 for i, ff in enumerate(FFparams)}


def atom2iZ(atm, elem_dict):
    """common.py:814-821."""
    try:
        return int(atm)
    except (TypeError, ValueError):
        key = atm.encode() if isinstance(atm, str) else atm
        if key in elem_dict:
            return elem_dict[key]
        raise ValueError(f"Did not find atomkind: {atm}")


def atoms2iZs(names, elem_dict):
    return np.array([atom2iZ(n, elem_dict) for n in names], dtype=np.int32)


SYMBOL_TO_Z = {s: z for z, s, *_ in _TABLE}
