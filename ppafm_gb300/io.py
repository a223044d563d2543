"""Files of the hot path's stages, restating ppafm/io.py: molecules (xyz, io.py:19-110) and
grids (XSF datagrids and npz, io.py:563-620, 716-880).

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


# Gaussian cube units (io.py:13-14)
bohrRadius2angstroem = 0.5291772109217
Hartree2eV = 27.211396132


def _cube_header(fname):
    with open(fname) as f:
        f.readline()
        f.readline()
        h = [f.readline().split() for _ in range(4)]
    return h


def loadCellCUBE(fname):
    """[origin, a, b, c] of a cube file in A (io.py:350-379): the voxel vectors times their
    counts, converted from bohr."""
    h = _cube_header(fname)
    b = bohrRadius2angstroem
    cell = [[float(v) * b for v in h[0][1:4]]]
    for k in (1, 2, 3):
        n = int(h[k][0])
        cell.append([float(v) * n * b for v in h[k][1:4]])
    return cell


def loadNCUBE(fname):
    """Voxel counts of a cube file (io.py:382-395)."""
    h = _cube_header(fname)
    return [int(h[1][0]), int(h[2][0]), int(h[3][0])]


def loadAtomsCUBE(fname):
    """[Zs, x, y, z, q] of a cube file's atoms, coordinates in A, charges 0 (io.py:291-320)."""
    e, x, y, z, q = [], [], [], [], []
    with open(fname) as f:
        f.readline()
        f.readline()
        natoms = int(f.readline().split()[0])
        for _ in range(3):
            f.readline()
        for _ in range(natoms):
            w = f.readline().split()
            e.append(int(w[0]))
            x.append(float(w[2]) * bohrRadius2angstroem)
            y.append(float(w[3]) * bohrRadius2angstroem)
            z.append(float(w[4]) * bohrRadius2angstroem)
            q.append(0.0)
    return [e, x, y, z, q]


def loadCUBE(fname, xyz_order=False):
    """(data, lvec [4, 3], grid size, header) of a Gaussian cube file (io.py:643-675): values
    converted from Hartree to eV (x slowest in the file); x, y, z order with xyz_order, else
    reversed like an XSF grid."""
    h = _cube_header(fname)
    nDim = np.array([int(h[1][0]), int(h[2][0]), int(h[3][0])])
    lvec = np.array(loadCellCUBE(fname), dtype=np.float64)
    natoms = abs(int(h[0][0]))
    with open(fname) as f:
        for _ in range(6 + natoms):
            f.readline()
        vals = np.array(f.read().split()[: int(np.prod(nDim))], dtype=np.float64)
    if vals.size != int(np.prod(nDim)):
        raise ValueError(f"{fname}: {vals.size} grid values, expected {int(np.prod(nDim))}")
    F = vals.reshape(nDim)
    if not xyz_order:
        F = F.transpose((2, 1, 0)).copy()
        nDim = [nDim[2], nDim[1], nDim[0]]
    F *= Hartree2eV
    head = ["BEGIN_BLOCK_DATAGRID_3D \n", "g98_3D_unknown \n", "DATAGRID_3D_g98Cube \n"]
    return F, lvec, nDim, head


def saveGeomXSF(fname, elems, xyzs, primvec, convvec=None, bTransposed=False):
    """An XSF geometry: CRYSTAL, PRIMVEC, CONVVEC (primvec when not given), PRIMCOORD atoms
    (io.py:203-226; xyzs [n, 3], or [3, n] with bTransposed)."""
    convvec = primvec if convvec is None else convvec
    xyzs = np.asarray(xyzs)
    if bTransposed:
        xyzs = xyzs.T
    with open(fname, "w") as f:
        f.write("CRYSTAL\nPRIMVEC\n")
        for v in primvec:
            f.write("".join(" %f " % x for x in v) + "\n")
        f.write("CONVVEC\n")
        for v in convvec:
            f.write("".join(" %f " % x for x in v) + "\n")
        f.write("PRIMCOORD\n%i %i\n" % (len(elems), 1))
        for i in range(len(elems)):
            f.write(f"{elems[i]} {xyzs[i][0]:10.10f} {xyzs[i][1]:10.10f} {xyzs[i][2]:10.10f}\n")
        f.write("\n")


def getFromHead_PRIMCOORD(head):
    """(Zs, Rs) of the PRIMCOORD block in a list of XSF header lines (io.py:623-637)."""
    Zs = Rs = None
    for i, line in enumerate(head):
        if "PRIMCOORD" in line:
            n = int(head[i + 1].split()[0])
            Zs = np.zeros(n, dtype="int32")
            Rs = np.zeros((n, 3))
            for j in range(n):
                w = head[i + j + 2].split()
                Zs[j] = int(w[0])
                Rs[j] = [float(w[1]), float(w[2]), float(w[3])]
    return Zs, Rs


def parseLvecASE(comment):
    """Lattice vectors of an ASE extended-xyz comment line (Lattice="ax ay az bx ... cz"),
    origin zero, as float32 values like io.py:506-525; None without them."""
    m = re.match('.*Lattice="\\s*((?:[+-]?(?:[0-9]*\\.)?[0-9]+\\s*){9})"', comment)
    if not m:
        return None
    lvec = np.zeros(12, dtype=np.float32)
    lvec[3:] = np.array([float(x) for x in m.group(1).split()], dtype=np.float32)
    return lvec.reshape(4, 3)


def loadPOSCAR(file_path):
    """(xyzs, Zs, lvec) of a VASP POSCAR/CONTCAR file (io.py:154-192): scale, lattice, element
    names and counts, optional selective-dynamics line, cartesian or direct coordinates."""
    with open(file_path) as f:
        f.readline()
        scale = float(f.readline())
        lvec = np.zeros((4, 3))
        for i in range(3):
            lvec[i + 1] = [float(v) for v in f.readline().split()[:3]]
        elems = [SYMBOL_TO_Z[e] for e in f.readline().split()]
        Zs = []
        for e, n in zip(elems, f.readline().split()):
            Zs += [e] * int(n)
        Zs = np.array(Zs, dtype=np.int32)
        line = f.readline()
        if line[0] in "Ss":
            line = f.readline()
        cartesian = line[0] in "CcKk"
        xyzs = np.array([[float(v) for v in f.readline().split()[:3]] for _ in range(len(Zs))])
        lvec *= scale
        if cartesian:
            xyzs *= scale
        else:
            xyzs = np.outer(xyzs[:, 0], lvec[1]) + np.outer(xyzs[:, 1], lvec[2]) + np.outer(xyzs[:, 2], lvec[3])
    return xyzs, Zs, lvec


def loadGeometryIN(fname):
    """(xyzs, Zs, lvec or None) of an FHI-aims geometry.in (io.py:126-151)."""
    Zs, xyzs, lvec = [], [], []
    with open(fname) as f:
        for line in f:
            ws = line.strip().split()
            if len(ws) == 0 or ws[0][0] == "#":
                continue
            if ws[0] == "atom":
                xyzs.append([float(ws[1]), float(ws[2]), float(ws[3])])
                Zs.append(SYMBOL_TO_Z[ws[4]])
            elif ws[0] == "lattice_vector":
                lvec.append([float(ws[1]), float(ws[2]), float(ws[3])])
            elif ws[0] == "atom_frac" and len(lvec) == 3:
                xyzs.append(np.array([float(ws[1]), float(ws[2]), float(ws[3])]) @ np.array(lvec))
                Zs.append(SYMBOL_TO_Z[ws[4]])
            elif ws[0] == "trust_radius":
                break
    lv = np.stack([[0.0, 0.0, 0.0]] + lvec, axis=0) if lvec else None
    return np.array(xyzs), np.array(Zs, dtype=np.int32), lv


def _geometry_format(fname):
    """The geometry format a file name implies, or None: POSCAR*/CONTCAR* by the base name, the
    others by suffix (.xyz, .xsf, .cube, .npy, FHI-aims .in and .in.next_step)."""
    base = fname.replace("\\", "/").rsplit("/", 1)[-1]
    if base.startswith(("POSCAR", "CONTCAR")):
        return "poscar"
    low = base.lower()
    if low.endswith((".in", ".in.next_step")):
        return "in"
    suffix = low.rsplit(".", 1)[-1] if "." in low else ""
    return suffix if suffix in ("xyz", "xsf", "cube", "npy") else None


def _atom_lists(xyzs, Zs, qs):
    """The [Zs, x, y, z, q] lists of the geometry readers (charges 0 when the file has none)."""
    qs = np.zeros(len(Zs)) if qs is None else qs
    return [list(Zs), list(xyzs[:, 0]), list(xyzs[:, 1]), list(xyzs[:, 2]), list(qs)]


def _geometry_from_file(fname, fmt, parameters):
    """(atom lists, grid size or None, lattice rows or None) of one file.  Files with a grid of
    their own (xsf, cube) give its size; atom-only formats take the parameters' grid size."""
    if fmt == "xsf":
        return loadXSFGeom(fname)
    if fmt == "cube":
        return loadAtomsCUBE(fname), loadNCUBE(fname), loadCellCUBE(fname)
    if fmt == "xyz":
        xyzs, Zs, qs, comment = loadXYZ(fname)
        lvec = parseLvecASE(comment)
    elif fmt == "poscar":
        (xyzs, Zs, lvec), qs = loadPOSCAR(fname), None
    elif fmt == "in":
        (xyzs, Zs, lvec), qs = loadGeometryIN(fname), None
    elif fmt == "npy":
        raise NotImplementedError("npy geometries are not read by this library")
    else:
        raise ValueError(f"unknown geometry format {fmt!r} of {fname}")
    return _atom_lists(xyzs, Zs, qs), np.array(parameters.gridN), lvec


def _full_lattice(lvec, parameters):
    """A [4, 3] lattice (origin + three vectors): rows the file lacks come from the
    parameters' grid (gridO when the file gives no lattice at all)."""
    defaults = [parameters.gridO, parameters.gridA, parameters.gridB, parameters.gridC]
    rows = [] if lvec is None else [list(v) for v in lvec]
    if not rows:
        rows = [list(defaults[0])]
    rows += [list(d) for d in defaults[len(rows) :]]
    return np.array(rows, dtype=np.float64)


def loadGeometry(fname=None, format=None, parameters=None):
    """(atoms [Zs, x, y, z, q] lists, grid size, lvec [4, 3]) of a geometry file: xyz (with an
    ASE lattice in the comment), xsf (PRIMCOORD), Gaussian cube, POSCAR/CONTCAR or FHI-aims
    .in; the behaviour of ppafm/io.py:398-503.  Lattice vectors the file lacks come from the
    parameters' grid.  A lattice vector that is zero is replaced by a box along its axis that
    holds the probe's path over the scan window (scanMin..scanMax shifted by r0Probe, z
    downwards) with 3 A to spare on each side, and periodic boundaries are switched off.  A
    grid size that is not positive becomes the lattice vector's length over a 0.1 A step.  The
    parameters' grid (gridO, gridA, gridB, gridC, gridN) is set to the result.  npy geometries
    are not read here."""
    if fname is None:
        raise ValueError("loadGeometry needs the name of a geometry file")
    if parameters is None:
        raise ValueError("loadGeometry needs the simulation parameters")
    fname = str(fname)
    fmt = format.lower() if format else _geometry_format(fname)
    if fmt is None:
        raise ValueError(f"cannot tell the geometry format of {fname} from its name; pass format=")
    atoms, nDim, lvec = _geometry_from_file(fname, fmt, parameters)
    nDim = np.array(nDim)
    lvec = _full_lattice(lvec, parameters)
    r0 = np.array(parameters.r0Probe, dtype=np.float64) * (1.0, 1.0, -1.0)
    path_lo = np.array(parameters.scanMin, dtype=np.float64) + r0
    path_hi = np.array(parameters.scanMax, dtype=np.float64) + r0
    pad, step = 3.0, 0.1  # A
    for axis in range(3):
        if np.allclose(lvec[axis + 1], 0):
            parameters.PBC = False
            lvec[axis + 1, axis] = path_hi[axis] - path_lo[axis] + 2 * pad
            lvec[0, axis] = path_lo[axis] - pad
        if not nDim[axis] > 0:
            nDim[axis] = round(np.linalg.norm(lvec[axis + 1]) / step)
    for name, row in zip(("gridO", "gridA", "gridB", "gridC"), lvec):
        grid = getattr(parameters, name)
        for k in range(3):
            grid[k] = row[k]
    parameters.gridN = nDim
    return atoms, nDim, lvec


def primcoords2Xsf(iZs, xyzs, lvec):
    """The XSF header (cell and PRIMCOORD atoms) the command-line stages write in front of their
    grids (io.py:323-346)."""
    lines = ["CRYSTAL", "PRIMVEC"]
    lines += [f"{lvec[k][0]:f} {lvec[k][1]:f} {lvec[k][2]:f}" for k in (1, 2, 3)]
    lines += ["CONVVEC"]
    lines += [f"{lvec[k][0]:f} {lvec[k][1]:f} {lvec[k][2]:f}" for k in (1, 2, 3)]
    lines += ["PRIMCOORD", "%i 1" % len(iZs)]
    lines += ["%i %5.6f %5.6f %5.6f" % (iZs[i], xyzs[0][i], xyzs[1][i], xyzs[2][i]) for i in range(len(iZs))]
    lines += ["", "BEGIN_BLOCK_DATAGRID_3D", "some_datagrid", "BEGIN_DATAGRID_3D_whatever"]
    return "\n".join(lines) + "\n"


# --------------------------------------------------------------------- grid files
# XSF datagrids and npz grids of ppafm/io.py:563-620, 716-880: the files the reference's
# command-line stages hand to each other (force fields, Fz and Δf stacks).  A datagrid has
# one more point than the data along each axis: the first plane is repeated as the last.

XSF_HEAD_DEFAULT = """
ATOMS
 1   0.0   0.0   0.0

BEGIN_BLOCK_DATAGRID_3D
   some_datagrid
   BEGIN_DATAGRID_3D_whatever
"""


def _ortho_lvec(sh, dd):
    return [[0, 0, 0], [sh[2] * dd[0], 0, 0], [0, sh[1] * dd[1], 0], [0, 0, sh[0] * dd[2]]]


def _row(vals):
    return " ".join(str(x) for x in vals) + "\n"


def saveXSFData(fname, data, lvec=None, dd=None, head=XSF_HEAD_DEFAULT, data_is_xyz_order=True):
    """Writes a scalar grid (x, y, z order unless data_is_xyz_order is False) as an XSF datagrid,
    values "%10.5e" with x fastest, the periodic edge repeated."""
    data = np.asarray(data)
    if data_is_xyz_order:
        data = data.transpose((2, 1, 0))
    if lvec is None:
        lvec = _ortho_lvec(data.shape, dd if dd is not None else [1.0, 1.0, 1.0])
    n = data.shape
    d2 = np.zeros(np.array(n) + 1)
    d2[:-1, :-1, :-1] = data
    d2[-1, :, :] = d2[0, :, :]
    d2[:, -1, :] = d2[:, 0, :]
    d2[:, :, -1] = d2[:, :, 0]
    with open(fname, "w") as f:
        for line in head:
            f.write(line)
        f.write(_row((n[2] + 1, n[1] + 1, n[0] + 1)))
        for vec in lvec:
            f.write(_row(vec))
        np.savetxt(f, d2.reshape(-1, 1), fmt="%10.5e")
        f.write("   END_DATAGRID_3D\n")
        f.write("END_BLOCK_DATAGRID_3D\n")


def loadXSFData(fname, xyz_order=True):
    """(data, lvec [4, 3], grid size, header lines) of an XSF datagrid; data in x, y, z order
    unless xyz_order is False, without the repeated edge."""
    head = []
    with open(fname) as f:
        while True:
            line = f.readline()
            head.append(line)
            if not line or "BEGIN_DATAGRID_3D" in line:
                break
        nDim = np.array([int(x) for x in f.readline().split()][::-1])
        lvec = np.array([[float(x) for x in f.readline().split()] for _ in range(4)])
        count = int(np.prod(nDim))
        vals = np.array(f.read().split()[:count], dtype=np.float64)
    if vals.size != count:
        raise ValueError(f"{fname}: {vals.size} grid values, expected {count}")
    F = vals.reshape(nDim)[:-1, :-1, :-1]
    if xyz_order:
        F = F.transpose((2, 1, 0))
        nDim = nDim[::-1].copy()
    return F.copy(), lvec, nDim - 1, head


def loadXSFGeom(fname):
    """([Zs, x, y, z, q], grid size, lvec) of an XSF file's PRIMCOORD atoms (atomic numbers)
    and datagrid header (io.py:229-267); ValueError without a PRIMCOORD block."""
    e, x, y, z, q = [], [], [], [], []
    with open(fname) as f:
        for line in f:
            if "PRIMCOORD" in line:
                break
        else:
            raise ValueError(f"{fname}: no PRIMCOORD block")
        n = int(f.readline().split()[0])
        for _ in range(n):
            ws = f.readline().split()
            e.append(int(ws[0]))
            x.append(float(ws[1]))
            y.append(float(ws[2]))
            z.append(float(ws[3]))
            q.append(0)
        for line in f:
            if "BEGIN_DATAGRID_3D" in line or "DATAGRID_3D_DENSITY" in line:
                break
        ws = f.readline().split()
        nDim = [int(ws[0]), int(ws[1]), int(ws[2])]
        lvec = [[float(w) for w in f.readline().split()[:3]] for _ in range(4)]
    return [e, x, y, z, q], (nDim[0] - 1, nDim[1] - 1, nDim[2] - 1), lvec


def packVecGrid(Fx, Fy, Fz, FF=None):
    if FF is None:
        FF = np.zeros(np.shape(Fx) + (3,))
    FF[..., 0] = Fx
    FF[..., 1] = Fy
    FF[..., 2] = Fz
    return FF


def unpackVecGrid(FF):
    return FF[..., 0].copy(), FF[..., 1].copy(), FF[..., 2].copy()


def limit_vec_field(FF, Fmax=100.0):
    """|F| <= Fmax in place, directions kept (io.py:766-778; on the GPU: ppgpu_clamp_grid)."""
    FR = np.sqrt(FF[..., 0] ** 2 + FF[..., 1] ** 2 + FF[..., 2] ** 2).ravel()
    mask = FR > Fmax
    for k in range(3):
        FF[..., k].flat[mask] *= Fmax / FR[mask]


def saveWSxM_2D(name_file, data, Xs, Ys):
    """One image as a WSxM ASCII XYZ file: header lines, then x, y, value per point
    (io.py:680-692)."""
    out = np.column_stack([np.asarray(Xs).ravel(), np.asarray(Ys).ravel(), np.asarray(data).ravel()])
    with open(name_file, "w") as f:
        f.write("WSxM file copyright Nanotec Electronica\nWSxM ASCII XYZ file\nX[A]  Y[A]  df[Hz]\n\n")
        np.savetxt(f, out)


def saveWSxM_3D(prefix, data, extent, slices=None):
    """The z slices of data [nx, ny, nz] as <prefix>_NNN.xyz WSxM files over extent
    (xmin, xmax, ymin, ymax) (io.py:695-706)."""
    nx, ny, nz = np.shape(data)
    Xs, Ys = np.meshgrid(np.linspace(extent[0], extent[1], nx), np.linspace(extent[2], extent[3], ny))
    for i in range(nz) if slices is None else slices:
        saveWSxM_2D(prefix + "_%03d.xyz" % i, data[:, :, i], Xs, Ys)


def saveNpy(fname, data, lvec, atomic_info):
    np.savez(fname + ".npz", data=data, lvec=lvec, atoms=atomic_info[0], lvec0=atomic_info[1])


def loadNpy(fname):
    d = np.load(fname + ".npz")
    return d["data"].copy(), d["lvec"], (d["atoms"], d["lvec0"])


def save_vec_field(fname, data, lvec, data_format="xsf", head=XSF_HEAD_DEFAULT, atomic_info=None):
    """fname_x/_y/_z.xsf, or fname.npz with keys FF, lvec, atoms, lvec0 (data [.., .., .., 3])."""
    if data_format == "xsf":
        for k, c in enumerate("xyz"):
            saveXSFData(f"{fname}_{c}.xsf", data[..., k], lvec, head=head)
    elif data_format == "npy":
        atomic_info = atomic_info if atomic_info is not None else (np.zeros((4, 1)), lvec)
        np.savez(fname + ".npz", FF=data, lvec=lvec, atoms=atomic_info[0], lvec0=atomic_info[1])
    else:
        raise ValueError(f"Cannot save vector field in format: {data_format}")


def load_vec_field(fname, data_format="xsf"):
    """(data [.., .., .., 3], lvec, grid size, header or (atoms, lvec0))."""
    if data_format == "xsf":
        comps = [loadXSFData(f"{fname}_{c}.xsf") for c in "xyz"]
        data = packVecGrid(comps[0][0], comps[1][0], comps[2][0])
        lvec, nDim, info = comps[2][1], comps[2][2], comps[2][3]
    elif data_format == "npy":
        d = np.load(fname + ".npz")
        data, lvec, info = d["FF"], d["lvec"], (d["atoms"], d["lvec0"])
        nDim = data.shape
    else:
        raise ValueError(f"Cannot load vector field in format: {data_format}")
    return data.copy(), lvec, nDim, info


def save_scal_field(fname, data, lvec, data_format="xsf", head=XSF_HEAD_DEFAULT, atomic_info=None):
    if data_format == "xsf":
        saveXSFData(fname + ".xsf", data, lvec, head=head)
    elif data_format == "npy":
        saveNpy(fname, data, lvec, atomic_info if atomic_info is not None else (np.zeros((4, 1)), lvec))
    else:
        raise ValueError(f"Cannot save scalar field in format: {data_format}")


def load_scal_field(fname, data_format="xsf"):
    if data_format == "xsf":
        data, lvec, nDim, info = loadXSFData(fname + ".xsf")
    elif data_format == "npy":
        data, lvec, info = loadNpy(fname)
        nDim = data.shape
    else:
        raise ValueError(f"Cannot load scalar field in format: {data_format}")
    return data.copy(), lvec, nDim, info
