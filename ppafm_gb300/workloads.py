"""Seeded synthetic inputs for the named workloads of the hot path.

The reference measures nothing on public data for this path, so every workload is a
seeded synthetic system with the stated shapes, sizes and value distributions:

  small_molecule   38-atom planar aromatic (24 C, 6 O, 8 H) on a jittered hexagonal
                   lattice, 20 A periodic cell, 200^3 grid, 160x160x30 scan
  slab_molecule    2000-atom FCC(111) metal slab (2.88 A in-plane spacing, q = 0) + 60-atom
                   C/N/O/H molecule 3 A above it, 40x40x25 A cell, 800x800x500 grid,
                   512x512x40 scan
  molecule_batch   256 molecules of 10-60 C/N/O/H/F/Cl atoms, cells 12-24 A per side at
                   0.125 A, 128x128x20 scan each
  density_overlap  40-atom molecule as Gaussian electron densities on a 256^3 grid of a
                   30 A cube (FFT route)

A workload is a dict of plain numpy arrays and scalars: atoms (Zs, Rs, Qs), lattice
``lvec`` (origin + 3 vectors), grid size, probe/tip parameters, FIRE settings, scan grid
and Δf settings.  ``scale`` shrinks grid and scan for quick tests with the same physics.
"""

import numpy as np

Z = dict(H=1, C=6, N=7, O=8, F=9, Cl=17, Au=79)

# Probe / relaxation / Δf settings shared by the workloads.
PROBE = dict(probeType=8, klat=0.25, krad=20.0, r0Probe=(0.0, 0.0, 4.0), charge=-0.05, tip="s")
FIRE = dict(dt=0.5, damping=0.1, convF2=1e-8, maxIters=300)
DF = dict(f0Cantilever=30000.0, kCantilever=1800.0, Amplitude=1.0)


def _neutralize(q):
    return q - q.mean()


def _honeycomb(extent, bond=1.4):
    """Honeycomb lattice sites (graphene-like) covering [-extent/2, extent/2]^2."""
    a = bond * np.sqrt(3.0)
    pts = []
    n = int(extent / a) + 3
    for i in range(-n, n + 1):
        for j in range(-n, n + 1):
            base = np.array([i * a + j * a / 2, j * a * np.sqrt(3) / 2])
            pts.append(base)
            pts.append(base + np.array([0.0, bond]))
    pts = np.array(pts)
    m = (np.abs(pts[:, 0]) <= extent / 2) & (np.abs(pts[:, 1]) <= extent / 2)
    return pts[m]


def _planar_molecule(rng, counts, extent, center, z, min_dist=1.1, jitter=0.0, lattice=False, zjitter=0.0):
    """Random planar molecule: atoms of the given element counts inside an extent x extent
    patch, either on a jittered honeycomb (lattice=True) or by rejection sampling."""
    symbols = [s for s, c in counts.items() for _ in range(c)]
    rng.shuffle(symbols)
    n = len(symbols)
    if lattice:
        sites = _honeycomb(extent)
        # a compact cluster: the n sites nearest to a random point near the centre
        c0 = rng.uniform(-1.0, 1.0, size=2)
        order = np.argsort(np.linalg.norm(sites - c0, axis=1))
        xy = sites[order[:n]] + rng.uniform(-jitter, jitter, size=(n, 2))
    else:
        xy = []
        tries = 0
        while len(xy) < n:
            p = rng.uniform(-extent / 2, extent / 2, size=2)
            tries += 1
            if tries > 200000:
                raise ValueError(f"cannot place {n} atoms {min_dist} A apart in a {extent} A patch")
            if all(np.linalg.norm(p - q) >= min_dist for q in xy):
                xy.append(p)
        xy = np.array(xy)
    R = np.zeros((n, 3))
    R[:, 0] = xy[:, 0] + center[0]
    R[:, 1] = xy[:, 1] + center[1]
    R[:, 2] = z + (rng.uniform(-zjitter, zjitter, size=n) if zjitter else 0.0)
    Zs = np.array([Z[s] for s in symbols], dtype=np.int32)
    return Zs, R


def _scan(cell_xy, npx, z0, nz, dz):
    step = (cell_xy[0] / npx[0], cell_xy[1] / npx[1])
    scanMin = (0.0, 0.0, z0)
    scanMax = (cell_xy[0] - step[0], cell_xy[1] - step[1], z0 + (nz - 1) * dz)
    return dict(scanMin=scanMin, scanMax=scanMax, scanStep=(step[0], step[1], dz))


def small_molecule(seed=0, scale=1.0):
    """38-atom planar molecule, 20 A cell, 0.1 A grid, 160x160x30 scan."""
    rng = np.random.default_rng(seed)
    L = 20.0
    Zs, R = _planar_molecule(rng, dict(C=24, O=6, H=8), 15.0, (L / 2, L / 2), 0.0, jitter=0.1, lattice=True)
    Qs = _neutralize(rng.uniform(-0.3, 0.3, size=len(Zs)))
    ng = max(8, int(round(200 * scale)))
    npx = max(4, int(round(160 * scale)))
    w = dict(name="small_molecule", seed=seed, Zs=Zs, Rs=R, Qs=Qs, lvec=np.array([[0.0, 0, 0], [L, 0, 0], [0, L, 0], [0, 0, L]]), gridN=(ng, ng, ng), PBC=True, nPBC=(1, 1, 1))
    w.update(PROBE)
    w.update(FIRE)
    w.update(DF)
    w.update(_scan((L, L), (npx, npx), 7.0, 30, 0.1))
    return w


def _fcc111_slab(natoms, cell_xy, spacing=2.88, nlayers=9, rng=None):
    """FCC(111) layers (ABC stacking) on a rectangular supercell strained to the cell,
    top layer at z = 0; the bottom layer is thinned at random to exactly natoms."""
    nrow_x = int(round(cell_xy[0] / spacing))
    nrow_y = int(round(cell_xy[1] / (spacing * np.sqrt(3) / 2)))
    nrow_y += nrow_y % 2
    ax = cell_xy[0] / nrow_x
    ay = cell_xy[1] / nrow_y
    dz = spacing * np.sqrt(2.0 / 3.0)  # (111) interlayer distance
    layers = []
    for L in range(nlayers):
        shift = [(0.0, 0.0), (ax / 2, ay / 3), (0.0, 2 * ay / 3)][L % 3]
        pts = []
        for j in range(nrow_y):
            for i in range(nrow_x):
                pts.append(((i + 0.5 * (j % 2)) * ax + shift[0], j * ay + shift[1], -L * dz))
        layers.append(np.array(pts))
    R = np.concatenate(layers)
    if len(R) < natoms:
        raise ValueError("slab too small")
    drop = len(R) - natoms
    nb = len(layers[-1])
    keep = np.ones(len(R), bool)
    keep[len(R) - nb + rng.choice(nb, size=drop, replace=False)] = False
    R = R[keep]
    R[:, 0] %= cell_xy[0]
    R[:, 1] %= cell_xy[1]
    return R


def slab_molecule(seed=0, scale=1.0):
    """2000-atom metal slab + 60-atom molecule, 40x40x25 A cell, 0.05 A grid (800x800x500),
    512x512x40 scan.  The slab is nine FCC(111) layers (2.88 A spacing, ABC), because two
    layers of a 40x40 A cell hold only ~450 atoms; the atom count (the cost driver) is kept."""
    rng = np.random.default_rng(seed)
    Lx, Ly, Lz = 40.0, 40.0, 25.0
    Rs_slab = _fcc111_slab(2000, (Lx, Ly), rng=rng)
    Zm, Rm = _planar_molecule(rng, dict(C=30, N=8, O=8, H=14), 14.0, (Lx / 2, Ly / 2), 3.0, min_dist=1.15)
    Qm = _neutralize(rng.uniform(-0.3, 0.3, size=len(Zm)))
    Zs = np.concatenate([np.full(len(Rs_slab), Z["Au"], np.int32), Zm])
    Rs = np.concatenate([Rs_slab, Rm])
    Qs = np.concatenate([np.zeros(len(Rs_slab)), Qm])
    n = (max(8, int(round(800 * scale))), max(8, int(round(800 * scale))), max(8, int(round(500 * scale))))
    npx = max(4, int(round(512 * scale)))
    origin = (0.0, 0.0, -14.5)
    w = dict(name="slab_molecule", seed=seed, Zs=Zs, Rs=Rs, Qs=Qs, lvec=np.array([origin, [Lx, 0, 0], [0, Ly, 0], [0, 0, Lz]]), gridN=n, PBC=True, nPBC=(1, 1, 1))
    w.update(PROBE)
    w.update(FIRE)
    w.update(DF)
    w.update(_scan((Lx, Ly), (npx, npx), 10.0, 40, 0.1))
    return w


def molecule_batch(seed=0, nmol=256, scale=1.0):
    """nmol molecules of 10-60 atoms, cells 12-24 A at 0.125 A, 128x128x20 scans."""
    rng = np.random.default_rng(seed)
    out = []
    elems = ["C", "N", "O", "H", "F", "Cl"]
    for m in range(nmol):
        na = int(rng.integers(10, 61))
        counts = dict(zip(elems, rng.multinomial(na, [0.4, 0.1, 0.1, 0.3, 0.05, 0.05])))
        counts = {k: int(v) for k, v in counts.items() if v > 0}
        # in-plane cell large enough for the molecule (a honeycomb blob of na atoms spans
        # about 2*sqrt(na*2.55/pi) A) plus 3 A, within 12-24 A; out of plane 12-24 A
        need = 2.0 * np.sqrt(na * 2.55 / np.pi) + 3.0
        lo = int(np.ceil(max(12.0, need) / 0.125))
        npts = np.array([rng.integers(lo, 193), rng.integers(lo, 193), rng.integers(96, 193)])
        cell = npts * 0.125
        Zs, R = _planar_molecule(rng, counts, 2 * need, (cell[0] / 2, cell[1] / 2), 0.0, jitter=0.15, lattice=True, zjitter=0.5)
        Qs = _neutralize(rng.uniform(-0.4, 0.4, size=len(Zs)))
        gN = tuple(max(8, int(round(int(k) * scale))) for k in npts)
        npx = max(4, int(round(128 * scale)))
        w = dict(name=f"batch_{m}", seed=seed, Zs=Zs, Rs=R, Qs=Qs, lvec=np.array([[0.0, 0, 0], [cell[0], 0, 0], [0, cell[1], 0], [0, 0, cell[2]]]), gridN=gN, PBC=True, nPBC=(1, 1, 1))
        w.update(PROBE)
        w.update(FIRE)
        w.update(DF)
        w.update(_scan((cell[0], cell[1]), (npx, npx), 7.5, 20, 0.1))
        out.append(w)
    return out


# Valence electrons and Gaussian widths (A) of the synthetic densities of density_overlap.
SIGMA_E = {1: 0.5, 6: 0.7, 7: 0.65, 8: 0.6, 9: 0.55, 17: 0.9}
VALENCE_Z = {1: 1, 6: 4, 7: 5, 8: 6, 9: 7, 17: 7}
SIGMA_CORE = 0.3


def density_overlap(seed=0, scale=1.0):
    """FFT density-overlap route: a 40-atom planar C/N/O/H molecule as Gaussian densities on a
    256^3 grid of a 30 A cube; tip = 6 electrons as two Gaussians on z, 1.15 A apart.

    Sample electron density: per atom a normalised Gaussian (sigma 0.5-0.9 A by element)
    holding (valence - q) electrons, q uniform +-0.3 e neutralised.  Sample charge density
    (for the Hartree potential): cores of +valence (sigma 0.3 A) minus the electron density,
    net charge 0.  Pauli: A = 12 eV A^3, B = 1.  Electrostatics: the Hartree potential
    correlated with the tip density normalised to one charge, times the probe charge Q.
    Scan: 160x160 pixels over the central 20x20 A, 30 z steps of 0.1 A."""
    rng = np.random.default_rng(seed)
    L = 30.0
    Zs, R = _planar_molecule(rng, dict(C=22, N=4, O=4, H=10), 14.0, (L / 2, L / 2), 0.0, jitter=0.1, lattice=True)
    Qs = _neutralize(rng.uniform(-0.3, 0.3, size=len(Zs)))
    origin = np.array([0.0, 0.0, -L / 2])
    rel = R - origin
    val = np.array([VALENCE_Z[int(z)] for z in Zs], dtype=np.float64)
    sig = np.array([SIGMA_E[int(z)] for z in Zs])
    rho_e_atoms = np.column_stack([rel, sig, val - Qs])
    core_atoms = np.column_stack([rel, np.full(len(Zs), SIGMA_CORE), val])
    tip_atoms = np.array([[0.0, 0.0, 0.575, 0.7, 3.0], [0.0, 0.0, -0.575, 0.7, 3.0]])
    ng = max(16, int(round(256 * scale)))
    npx = max(4, int(round(160 * scale)))
    w = dict(name="density_overlap", seed=seed, Zs=Zs, Rs=R, Qs=Qs, lvec=np.array([origin, [L, 0, 0], [0, L, 0], [0, 0, L]]), gridN=(ng, ng, ng), rho_e_atoms=rho_e_atoms, core_atoms=core_atoms, tip_atoms=tip_atoms, tip_electrons=6.0, Apauli=12.0, Bpauli=1.0)
    w.update(PROBE)
    w.update(FIRE)
    w.update(DF)
    scan = _scan((20.0, 20.0), (npx, npx), 7.0, 30, 0.1)
    scan["scanMin"] = (5.0, 5.0, scan["scanMin"][2])
    scan["scanMax"] = (5.0 + scan["scanMax"][0], 5.0 + scan["scanMax"][1], scan["scanMax"][2])
    w.update(scan)
    return w
