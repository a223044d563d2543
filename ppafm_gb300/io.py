"""Molecule files: the xyz reader and writer of ppafm/io.py:19-110 (the format the ML
generator reads its molecules from).

An xyz file is: the atom count, a comment line, then one line per atom with the element
(symbol or atomic number), x, y, z and optional extra columns.  Charges are the first extra
column, or -- in ASE's extended format, whose comment line carries ``Properties=...`` -- the
column named ``charge`` or ``initial_charges`` (zeros when there is none).
"""

import re

import numpy as np

from .species import SYMBOL_TO_Z


def loadXYZ(fname):
    """(xyzs [N, 3] float64, Zs [N] int32, qs [N] float64, comment) of an xyz file."""
    xyzs, Zs, extra = [], [], []
    with open(fname) as f:
        line = f.readline().strip()
        try:
            N = int(line)
        except ValueError:
            raise ValueError(f"The first line of an xyz file should have the number of atoms, but got `{line}`")
        comment = f.readline().strip()
        for i, line in enumerate(f):
            if i >= N:
                break
            wds = line.split()
            try:
                Z = SYMBOL_TO_Z[wds[0]] if wds[0] in SYMBOL_TO_Z else int(wds[0])
                xyzs.append((float(wds[1]), float(wds[2]), float(wds[3])))
                Zs.append(Z)
                extra.append(wds[4:])
            except (ValueError, IndexError):
                raise ValueError(f"Could not interpret line in xyz file: `{line}`")
    xyzs = np.array(xyzs, dtype=np.float64).reshape(-1, 3)
    Zs = np.array(Zs, dtype=np.int32)
    qs = _charges(comment, extra) if extra and len(extra[0]) > 0 else np.zeros(len(Zs), dtype=np.float64)
    return xyzs, Zs, qs, comment


def _charges(comment, extra):
    m = re.match(r".*Properties=(\S*) ", comment)
    if not m:
        return np.array([float(e[0]) for e in extra], dtype=np.float64)
    # ASE: name:type:ncols triplets; the first two (species, pos) are not in the extra columns
    props = m.group(1).split(":")[6:]
    col = 0
    for name, size in zip(props[::3], props[2::3]):
        if name in ("charge", "initial_charges"):
            return np.array([float(e[col]) for e in extra], dtype=np.float64)
        col += int(size)
    return np.zeros(len(extra), dtype=np.float64)


def saveXYZ(fname, xyzs, Zs, qs=None, comment="", append=False):
    """Writes atoms (and charges as a fifth column) in the format loadXYZ reads."""
    Z_TO_SYMBOL = {z: s for s, z in SYMBOL_TO_Z.items()}
    xyzs = np.asarray(xyzs)
    with open(fname, "a" if append else "w") as f:
        f.write(f"{len(xyzs)}\n{comment}\n")
        for i in range(len(xyzs)):
            el = Z_TO_SYMBOL.get(int(Zs[i]), str(int(Zs[i])))
            line = f"{el} {xyzs[i][0]:10.6f} {xyzs[i][1]:10.6f} {xyzs[i][2]:10.6f}"
            if qs is not None:
                line += f" {qs[i]:10.6f}"
            f.write(line + "\n")
