"""Training-data generators over the GPU AFMulator: the public interface of
ppafm/ml/Generator.py (``InverseAFMtrainer``, ``GeneratorAFMtrainer`` and the rotation
helpers), organised around where the work waits on a GPU.

Both generators produce batches of Δf image stacks.  In the reference every image is one
blocking ``afmulator(...)`` call that ends with a device-to-host copy.  Here an image is
queued on the CUDA stream -- force field, relaxation and Δf written into its slot of one
device buffer per batch (``_ImageBatch``) -- and the whole batch goes to the host in one
copy.  The host prepares the next molecule (placement, pair parameters, atom records) while
the GPU works on the previous ones, and the AFMulator runs in its overlap mode, so each
image's force field runs beside the previous image's relaxation.  The only synchronisation
per image left is the one a user asks for by overriding ``InverseAFMtrainer.on_afm_end``,
which sees the image as a host array in ``self.Xs``.

Behaviour kept from the reference (by the same public names, arguments, callbacks and
attributes): molecules read from xyz files or taken from a sample iterator; the molecule
(InverseAFMtrainer) or the scan window (GeneratorAFMtrainer) placed so that the probe's van
der Waals sphere starts ``distAbove`` above the molecule's van der Waals surface; the
augmentation and randomisation methods with the same random draws from ``np.random`` and
``random``; the callbacks ``on_batch_start``, ``on_sample_start``, ``on_afm_start`` and
``on_afm_end``.

Aux maps are host callables (the reference's AuxMap classes are OpenCL programs):
``aux_map(xyzqs, Zs) -> [nx, ny]`` for InverseAFMtrainer and
``aux_map(xyzqs, Zs, pot, rot) -> [nx, ny]`` for GeneratorAFMtrainer, where an aux map with
a ``scan_window`` attribute is told the lateral scan window of each sample.
"""

import random
import time

import numpy as np
import torch

from .. import common as PPU
from .. import io
from ..AFMulator import HartreePotential

# ------------------------------------------------------------------ host-side geometry


def _molecule_record(xyzs, qs, Zs):
    """One molecule as an [n_atoms, 5] array: x, y, z, charge, element."""
    return np.column_stack([np.asarray(xyzs, dtype=np.float64), np.asarray(qs, dtype=np.float64), np.asarray(Zs, dtype=np.float64)])


def _vdw_clearance(zs, Rvdw, RvdwPP, gap):
    """Height of the probe's centre above the molecule's highest atom when the probe's van der
    Waals sphere (radius RvdwPP) is ``gap`` above the molecule's van der Waals surface.  The
    atom whose sphere reaches highest decides (ppafm/ml/Generator.py:176-184, 594-615)."""
    top = int(np.argmax(zs + Rvdw))
    return gap + Rvdw[top] + RvdwPP - (zs.max() - zs[top])


def _probe_vdw_radius(afm):
    return afm.typeParams[afm.iZPP - 1][0]


def getRandomUniformDisk():
    """A point drawn uniformly from the unit disk (radius sqrt(u), angle 2 pi v, from one
    np.random.rand(2) draw)."""
    u, v = np.random.rand(2)
    radius, angle = np.sqrt(u), 2.0 * np.pi * v
    return radius * np.cos(angle), radius * np.sin(angle)


def rotate(xyzs, rotations):
    """The coordinates under each rotation matrix (rows of the result: R @ r)."""
    xyzs = np.asarray(xyzs)
    return [xyzs @ np.asarray(rot).T for rot in rotations]


def sortRotationsByEntropy(xyzs, rotations):
    """Rotations ordered by decreasing spread of the atoms' heights along the rotated z axis
    (the entropy term of common.maxAlongDirEntropy); ties keep their order."""

    def spread(rot):
        return PPU.maxAlongDirEntropy(xyzs, np.asarray(rot)[2].ravel().copy())[2]

    return sorted(rotations, key=lambda rot: -spread(rot))


# ------------------------------------------------------------------ device image batch


class _ImageBatch:
    """Device buffer of one batch's Δf stacks.  ``slot(...)`` is the view one evalAFM call
    writes; ``to_host(n)`` copies the first n entries of the leading axis (all by default)
    in one transfer."""

    def __init__(self, shape):
        self.images = torch.empty(shape, dtype=torch.float32, device="cuda")

    def slot(self, *index):
        return self.images[index]

    def to_host(self, n=None):
        return (self.images if n is None else self.images[:n]).cpu().numpy()


class _TrainerBase:
    """What both generators share: the AFMulator, the tips, the probe-to-surface distance and
    its randomisation, the callbacks, and the per-image call into the AFMulator."""

    def _init_common(self, afmulator, aux_maps, batch_size, distAbove, iZPPs):
        # images queued back to back: each image's force field runs beside the previous
        # image's relaxation (AFMulator.set_overlap); the host copies join the streams first
        afmulator.set_overlap(True)
        self.afmulator = afmulator
        self.aux_maps = aux_maps
        self.batch_size = batch_size
        self.distAbove = distAbove
        self.distAboveActive = distAbove
        self.iZPPs = iZPPs
        self.last_timing = {}

    def _tips(self):
        return zip(self.iZPPs, self.Qs, self.QZs)

    def _select_tip(self, iZPP, Q, QZ):
        afm = self.afmulator
        afm.iZPP = iZPP
        afm.setQs(Q, QZ)

    def _pair_parameters(self, Zs):
        afm = self.afmulator
        return PPU.getAtomsREA(afm.iZPP, Zs, afm.typeParams, alphaFac=-1.0)

    # randomisation shared by both generators
    def randomize_tip(self, max_tilt=0.5):
        """Moves the tip's rest position laterally to a random point of a disk of radius max_tilt."""
        self.afmulator.tipR0[:2] = max_tilt * np.array(getRandomUniformDisk())

    def randomize_distance(self, delta=0.25):
        """Draws the probe-to-surface distance uniformly from distAbove +- delta."""
        self.distAboveActive = np.random.uniform(self.distAbove - delta, self.distAbove + delta)

    # callbacks
    def on_batch_start(self):
        """Runs at the start of each batch."""

    def on_sample_start(self):
        """Runs when a sample (molecule) has been placed, before its first image."""

    def on_afm_start(self):
        """Runs before every image."""


# ------------------------------------------------------------------ InverseAFMtrainer


class InverseAFMtrainer(_TrainerBase):
    """Batches ``(Xs, Ys, mols)`` of molecules read from xyz files (ppafm/ml/Generator.py:
    14-238): Xs a list with one [n_batch, nx, ny, nz_out] array per tip, Ys one
    [n_batch, nx, ny] array per aux map, mols the [n_atoms, 5] arrays (x, y, z, charge,
    element) of the batch.  Each molecule is centred laterally in the scan window and lowered
    so the probe starts distAboveActive above its van der Waals surface."""

    def __init__(self, afmulator, aux_maps, paths, batch_size=30, distAbove=5.3, iZPPs=[8], Qs=[[-10, 20, -10, 0]], QZs=[[0.1, 0, -0.1, 0]]):
        assert len(iZPPs) == len(Qs) == len(QZs), "one charge set per tip"
        self._init_common(afmulator, aux_maps, batch_size, distAbove, iZPPs)
        self.paths = paths
        self.Qs = Qs
        self.QZs = QZs
        self.read_xyzs()
        self.counter = 0

    # --------------------------------------------------------------- molecules
    def read_xyzs(self):
        """Loads every path into ``self.molecules``."""
        self.molecules = []
        for path in self.paths:
            xyzs, Zs, qs, _ = io.loadXYZ(path)
            self.molecules.append(_molecule_record(xyzs, qs, Zs))

    def shuffle_molecules(self):
        random.shuffle(self.molecules)

    def _rotated_copies(self, mol, rotations):
        return [_molecule_record(xyz, mol[:, 3], mol[:, 4]) for xyz in rotate(mol[:, :3], rotations)]

    def augment_with_rotations(self, rotations):
        """Replaces every molecule by its copies under each rotation."""
        self.molecules = [copy for mol in self.molecules for copy in self._rotated_copies(mol, rotations)]

    def augment_with_rotations_entropy(self, rotations, n_best_rotations=30):
        """Like augment_with_rotations with each molecule's n_best_rotations rotations of
        largest height spread."""
        self.molecules = [copy for mol in self.molecules for copy in self._rotated_copies(mol, sortRotationsByEntropy(mol[:, :3], rotations)[:n_best_rotations])]

    def randomize_mol_parameters(self, rndQmax=0.0, rndRmax=0.0, rndEmax=0.0, rndAlphaMax=0.0):
        """Random changes of the current molecule's charges (added, +-rndQmax/2), van der Waals
        radii (added, +-rndRmax/2), well depths and alphas (scaled by 1 +- max/2)."""
        n = len(self.qs)

        def jitter(scale):
            return scale * (np.random.rand(n) - 0.5)

        if rndQmax > 0:
            self.qs[:] += jitter(rndQmax)
        if rndRmax > 0:
            self.REAs[:, 0] += jitter(rndRmax)
        if rndEmax > 0:
            self.REAs[:, 1] *= 1 + jitter(rndEmax)
        if rndAlphaMax > 0:
            self.REAs[:, 2] *= 1 + jitter(rndAlphaMax)

    # --------------------------------------------------------------- placement
    def handle_positions(self):
        """Moves the current molecule's lateral centre onto the scan window's centre."""
        (x0, y0, _), (x1, y1, _) = self.afmulator.scan_window
        self.xyzs[:, :2] += np.array([x1 + x0, y1 + y0]) / 2 - self.xyzs[:, :2].mean(axis=0)

    def handle_distance(self):
        """Shifts the current molecule in z so the top of the scan window is distAboveActive
        (plus the van der Waals radii) above its van der Waals surface."""
        afm = self.afmulator
        RvdwPP = _probe_vdw_radius(afm)
        zs = self.xyzs[:, 2]
        clearance = _vdw_clearance(zs, self.REAs[:, 0] - RvdwPP, RvdwPP, self.distAboveActive)
        self.xyzs[:, 2] += afm.scan_window[1][2] - clearance - zs.max()

    # --------------------------------------------------------------- iteration
    def _host_image_each(self):
        """True when a subclass overrides on_afm_end: it gets each image on the host."""
        return type(self).on_afm_end is not InverseAFMtrainer.on_afm_end

    def _load_molecule(self, mol):
        self.xyzs = mol[:, :3]
        self.qs = mol[:, 3]
        self.Zs = mol[:, 4].astype(np.int32)

    def __iter__(self):
        self.counter = 0
        return self

    def __len__(self):
        """Number of whole batches of the current molecules."""
        return len(self.molecules) // self.batch_size

    def __next__(self):
        remaining = len(self.molecules) - self.counter
        if remaining <= 0:
            raise StopIteration
        self.on_batch_start()
        t0 = time.perf_counter()
        afm = self.afmulator
        n = min(self.batch_size, remaining)
        nx, ny, nz = afm.scan_dim
        batch = _ImageBatch((len(self.iZPPs), n, nx, ny, nz - len(afm.dfWeight) + 1))
        host_each = self._host_image_each()
        aux = [[] for _ in self.aux_maps]
        mols = self.molecules[self.counter : self.counter + n]
        for s, mol in enumerate(mols):
            self._load_molecule(mol)
            self.handle_positions()
            self.on_sample_start()
            for t, tip in enumerate(self._tips()):
                self._select_tip(*tip)
                self.REAs = self._pair_parameters(self.Zs)
                self.handle_distance()
                self.on_afm_start()
                afm.prepareFF(self.xyzs, self.Zs, self.qs, REAs=self.REAs)
                image = batch.slot(t, s)
                afm.evalAFM(out=image)
                if host_each:
                    afm.join()
                self.Xs = image.cpu().numpy() if host_each else image
                self.on_afm_end()
            xyzqs = np.column_stack([self.xyzs, self.qs])
            for store, aux_map in zip(aux, self.aux_maps):
                store.append(aux_map(xyzqs, self.Zs))
            self.counter += 1
        afm.join()
        host = batch.to_host()  # [tips, n, ...]: one copy per batch
        self.last_timing["batch"] = time.perf_counter() - t0
        return list(host), [np.stack(store) for store in aux], mols

    def on_afm_end(self):
        """Runs after every image (``self.Xs`` holds it; a host array when overridden)."""


# ------------------------------------------------------------------ GeneratorAFMtrainer


def _charges_lj(sample):
    sample["qs"] = np.zeros(len(sample["Zs"]), dtype=np.float32)


def _charges_point(sample):
    if not isinstance(sample.get("qs"), np.ndarray):
        raise ValueError("an LJ+PC sample needs point charges: 'qs' must be a numpy array")


def _charges_hartree(sample):
    if not isinstance(sample.get("qs"), HartreePotential):
        raise ValueError("an LJ+Hartree sample needs its potential: 'qs' must be a HartreePotential")


# per simulation type: how a sample's 'qs' is checked or filled in
_SIM_TYPES = {"lj": _charges_lj, "lj+pc": _charges_point, "lj+hartree": _charges_hartree}


class GeneratorAFMtrainer(_TrainerBase):
    """Batches ``(Xs, Ys, mols, sws)`` from an iterator of sample dicts (ppafm/ml/Generator.py:
    240-663): Xs [n_batch, n_tip, nx, ny, nz_out], Ys [n_batch, n_aux, nx, ny], mols the
    [n_atoms, 5] arrays of the rotated molecules, sws [n_batch, n_tip, 2, 3] the scan windows.
    A sample holds AFMulator.eval's arguments (at least xyzs and Zs; qs, rot, sample_lvec,
    rot_center).  The molecule stays where it is; the scan window follows it laterally and
    starts distAboveActive above its van der Waals surface.  Simulation types: 'LJ', 'LJ+PC'
    (point charges qs, tip charges Qs/QZs) and 'LJ+Hartree' (qs a HartreePotential; rhos one
    tip density per tip -- a multipole dict or a TipDensity -- or None for the point-charge
    tip); 'FDBM' is not provided."""

    def __init__(self, afmulator, aux_maps, sample_generator, sim_type="LJ", batch_size=30, distAbove=5.3, iZPPs=[8], Qs=None, QZs=None, rhos=None, rho_deltas=None, ignore_elements=[], density_cutoff=None):
        kind = sim_type.lower()
        if kind == "fdbm" or rho_deltas is not None:
            raise NotImplementedError("the FDBM simulation type is not provided")
        if kind not in _SIM_TYPES:
            raise ValueError(f"Unknown simulation type `{sim_type}`")
        if rhos is not None and len(rhos) != len(iZPPs):
            raise ValueError(f"{len(rhos)} tip densities for {len(iZPPs)} tips")
        self._init_common(afmulator, aux_maps, batch_size, distAbove, iZPPs)
        self.sample_generator = sample_generator
        self.sim_type = kind
        self.rhos = list(rhos) if rhos is not None else [None] * len(iZPPs)
        self.ignore_elements = ignore_elements
        self.density_cutoff = None
        if Qs is None or QZs is None:
            if kind == "lj+pc":
                raise ValueError("point-charge electrostatics needs both Qs and QZs")
            self.Qs = self.QZs = [[0, 0, 0, 0] for _ in iZPPs]
        else:
            assert len(Qs) == len(QZs) == len(iZPPs), "one charge set per tip"
            self.Qs, self.QZs = Qs, QZs
        sw = afmulator.scan_window
        self.scan_window = sw
        self.scan_size = tuple(sw[1][k] - sw[0][k] for k in range(3))
        self.scan_dim = afmulator.scan_dim
        self.df_steps = afmulator.df_steps
        self.z_size = self.scan_dim[2] - self.df_steps + 1

    # --------------------------------------------------------------- samples
    def _load_next_sample(self):
        sample = next(self.sample_iterator)
        _SIM_TYPES[self.sim_type](sample)
        sample["rho_sample"] = None
        sample.setdefault("rot", np.eye(3))
        return sample

    def __len__(self):
        if not hasattr(self.sample_generator, "__len__"):
            raise RuntimeError("the sample generator has no length, so the number of batches is unknown")
        return len(self.sample_generator) // self.batch_size

    def _kept_atoms(self):
        """Mask of the atoms whose elements are not in ignore_elements."""
        return ~np.isin(self.sample_dict["Zs"], self.ignore_elements)

    # --------------------------------------------------------------- placement
    def handle_positions(self):
        """Centres the scan window laterally on the (kept) atoms of the rotated molecule."""
        xyzs = self.xyzs_rot[self._kept_atoms()] if self.ignore_elements else self.xyzs_rot
        cx, cy = xyzs[:, :2].mean(axis=0)
        hx, hy = self.scan_size[0] / 2, self.scan_size[1] / 2
        (_, _, z0), (_, _, z1) = self.scan_window
        self.scan_window = ((cx - hx, cy - hy, z0), (cx + hx, cy + hy, z1))
        for aux_map in self.aux_maps:
            if hasattr(aux_map, "scan_window"):
                aux_map.scan_window = ((cx - hx, cy - hy), (cx + hx, cy + hy))

    def handle_distance(self):
        """Raises or lowers the scan window so its bottom is distAboveActive (plus the van der
        Waals radii) above the molecule's van der Waals surface."""
        afm = self.afmulator
        RvdwPP = _probe_vdw_radius(afm)
        zs = self.xyzs_rot[:, 2]
        Rvdw = self.sample_dict["REAs"][:, 0] - RvdwPP
        if self.ignore_elements:
            keep = self._kept_atoms()
            zs, Rvdw = zs[keep], Rvdw[keep]
        z_min = zs.max() + _vdw_clearance(zs, Rvdw, RvdwPP, self.distAboveActive)
        (x0, y0, _), (x1, y1, _) = self.scan_window
        self.scan_window = ((x0, y0, z_min), (x1, y1, z_min + self.scan_size[2]))

    # --------------------------------------------------------------- randomisation
    def set_fdbm_parameters(self, A_pauli, B_pauli):
        """FDBM Pauli parameters (ppafm/ml/Generator.py:617-635): the reference uses them only
        for the FDBM simulation type, which this library does not provide."""

    def randomize_df_steps(self, minimum=4, maximum=20):
        """A random number of Δf steps in [minimum, maximum]; the output z size and the z step
        stay, so the scan grows or shrinks in z."""
        self.df_steps = np.random.randint(minimum, maximum + 1)
        nz = self.z_size + self.df_steps - 1
        self.scan_dim = (self.scan_dim[0], self.scan_dim[1], nz)
        self.scan_size = (self.scan_size[0], self.scan_size[1], self.afmulator.dz * nz)

    # --------------------------------------------------------------- iteration
    def __iter__(self):
        self.sample_dict = {}
        self.sample_iterator = iter(self.sample_generator)
        self.iteration_done = False
        return self

    def _image(self, batch, s, t, tip, rho):
        """Queues the image of tip t for the current sample into batch slot (s, t)."""
        afm = self.afmulator
        self._select_tip(*tip)
        if rho is not None:
            afm.setRho(rho, sigma=afm.sigma, B_pauli=afm.B_pauli)
        d = self.sample_dict
        d["REAs"] = self._pair_parameters(d["Zs"])
        self.handle_distance()
        afm.setScanWindow(self.scan_window, self.scan_dim, df_steps=self.df_steps)
        afm.setLvec()
        self.on_afm_start()
        afm.prepareFF(d["xyzs"], d["Zs"], d["qs"], rho_sample=d.get("rho_sample"), sample_lvec=d.get("sample_lvec"), rot=d["rot"], rot_center=d.get("rot_center"), REAs=d["REAs"])
        afm.evalAFM(out=batch.slot(s, t))
        return np.array(self.scan_window)

    def __next__(self):
        if self.iteration_done:
            raise StopIteration
        self.on_batch_start()
        t0 = time.perf_counter()
        batch = _ImageBatch((self.batch_size, len(self.iZPPs), self.scan_dim[0], self.scan_dim[1], self.z_size))
        mols, windows, aux = [], [], []
        for s in range(self.batch_size):
            try:
                self.sample_dict = self._load_next_sample()
            except StopIteration:
                self.sample_dict = None
                self.iteration_done = True
                break
            d = self.sample_dict
            xyzs, Zs, rot = d["xyzs"], d["Zs"], d["rot"]
            pot = d["qs"] if isinstance(d["qs"], HartreePotential) else None
            qs = np.zeros(len(Zs)) if pot is not None else d["qs"]
            centre = xyzs.mean(axis=0)
            self.xyzs_rot = (xyzs - centre) @ rot.T + centre
            mols.append(_molecule_record(self.xyzs_rot, qs, Zs))
            self.handle_positions()
            self.on_sample_start()
            windows.append([self._image(batch, s, t, tip, rho) for t, (tip, rho) in enumerate(zip(self._tips(), self.rhos))])
            xyzqs = np.column_stack([xyzs, qs])
            aux.append([aux_map(xyzqs, Zs, pot, rot) for aux_map in self.aux_maps])
        if not mols:
            raise StopIteration
        self.afmulator.join()
        Xs = batch.to_host(len(mols))  # one copy per batch
        self.last_timing["batch"] = time.perf_counter() - t0
        return Xs, np.array(aux), mols, np.array(windows)
