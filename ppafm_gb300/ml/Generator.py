"""The ML training-data generator of ppafm/ml/Generator.py:14-286 on libppgpu.

``InverseAFMtrainer`` keeps the reference's constructor, iteration protocol, callbacks
(on_batch_start / on_sample_start / on_afm_start / on_afm_end), positioning
(handle_positions, handle_distance) and augmentation methods.  What changes is where the
work waits: the reference evaluates each sample with a blocking ``afmulator(...)`` call that
copies the image to the host; here every sample's force field and relaxation are queued on
the CUDA stream into one device buffer per tip, and the batch is copied to the host once.
Host-side preparation of the next sample (positions, Lennard-Jones parameters, atom packing)
overlaps with the GPU work of the previous ones.  A subclass that overrides on_afm_end sees
``self.Xs`` as a host array, as in the reference, at the price of one synchronisation per
image; otherwise ``self.Xs`` is the image's device tensor.

Aux maps are callables ``aux_map(xyzqs, Zs) -> [nx, ny] array`` (the reference's AuxMap
classes need OpenCL and are not part of this library).
"""

import random
import time

import numpy as np
import torch

from .. import common as PPU
from .. import io
from ..AFMulator import HartreePotential


class InverseAFMtrainer:
    """Batches (Xs, Ys, mols): Xs a list (one per tip) of [n_batch, nx, ny, nz_out] arrays,
    Ys a list (one per aux map) of [n_batch, nx, ny] arrays, mols the [n_atoms, 5] arrays
    (x, y, z, charge, element) of the batch's molecules."""

    def __init__(self, afmulator, aux_maps, paths, batch_size=30, distAbove=5.3, iZPPs=[8], Qs=[[-10, 20, -10, 0]], QZs=[[0.1, 0, -0.1, 0]]):
        assert len(iZPPs) == len(Qs) and len(Qs) == len(QZs)
        self.afmulator = afmulator
        self.aux_maps = aux_maps
        self.paths = paths
        self.batch_size = batch_size
        self.distAbove = distAbove
        self.distAboveActive = distAbove
        self.iZPPs = iZPPs
        self.Qs = Qs
        self.QZs = QZs
        self.read_xyzs()
        self.counter = 0
        self.last_timing = {}

    def _sync_each_image(self):
        return type(self).on_afm_end is not InverseAFMtrainer.on_afm_end

    def __next__(self):
        if self.counter >= len(self.molecules):
            raise StopIteration
        self.on_batch_start()
        t0 = time.perf_counter()
        afm = self.afmulator
        mols = []
        batch_size = min(self.batch_size, len(self.molecules) - self.counter)
        nx, ny, nz = afm.scan_dim
        nout = nz - len(afm.dfWeight) + 1
        Xd = [torch.empty((batch_size, nx, ny, nout), dtype=torch.float32, device="cuda") for _ in self.iZPPs]
        Ys = [[] for _ in self.aux_maps]
        sync_each = self._sync_each_image()
        for s in range(batch_size):
            mol = self.molecules[self.counter]
            mols.append(mol)
            self.xyzs = mol[:, :3]
            self.qs = mol[:, 3]
            self.Zs = mol[:, 4].astype(np.int32)
            self.handle_positions()
            self.on_sample_start()
            for i, (iZPP, Q, Qz) in enumerate(zip(self.iZPPs, self.Qs, self.QZs)):
                afm.iZPP = iZPP
                afm.setQs(Q, Qz)
                self.REAs = PPU.getAtomsREA(afm.iZPP, self.Zs, afm.typeParams, alphaFac=-1.0)
                self.handle_distance()
                self.on_afm_start()
                afm.prepareFF(self.xyzs, self.Zs, self.qs, REAs=self.REAs)
                afm.evalAFM(out=Xd[i][s])
                self.Xs = Xd[i][s].cpu().numpy() if sync_each else Xd[i][s]
                self.on_afm_end()
            for i, aux_map in enumerate(self.aux_maps):
                xyzqs = np.concatenate([self.xyzs, self.qs[:, None]], axis=1)
                Ys[i].append(aux_map(xyzqs, self.Zs))
            self.counter += 1
        Xs = [x.cpu().numpy() for x in Xd]  # one copy per tip per batch
        Ys = [np.stack(y, axis=0) for y in Ys]
        self.last_timing["batch"] = time.perf_counter() - t0
        return Xs, Ys, mols

    def __iter__(self):
        self.counter = 0
        return self

    def __len__(self):
        """Number of whole batches of the current molecules."""
        return int(np.floor(len(self.molecules) / self.batch_size))

    def read_xyzs(self):
        self.molecules = []
        for path in self.paths:
            xyzs, Zs, qs, _ = io.loadXYZ(path)
            self.molecules.append(np.concatenate([xyzs, qs[:, None], Zs[:, None]], axis=1))

    def handle_positions(self):
        """Centres the current molecule in the scan window (x, y)."""
        sw = self.afmulator.scan_window
        scan_center = np.array([sw[1][0] + sw[0][0], sw[1][1] + sw[0][1]]) / 2
        self.xyzs[:, :2] += scan_center - self.xyzs[:, :2].mean(axis=0)

    def handle_distance(self):
        """Puts the molecule's highest van der Waals surface distAboveActive below the scan's top."""
        RvdwPP = self.afmulator.typeParams[self.afmulator.iZPP - 1][0]
        Rvdw = self.REAs[:, 0] - RvdwPP
        zs = self.xyzs[:, 2]
        imax = np.argmax(zs + Rvdw)
        total_distance = self.distAboveActive + Rvdw[imax] + RvdwPP - (zs.max() - zs[imax])
        self.xyzs[:, 2] += (self.afmulator.scan_window[1][2] - total_distance) - zs.max()

    # ------------------------------------------------------------ augmentation

    def shuffle_molecules(self):
        random.shuffle(self.molecules)

    def augment_with_rotations(self, rotations):
        molecules = self.molecules
        self.molecules = []
        for mol in molecules:
            for xyzs_rot in rotate(mol[:, :3], rotations):
                self.molecules.append(np.concatenate([xyzs_rot, mol[:, 3:4], mol[:, 4:5]], axis=1))

    def augment_with_rotations_entropy(self, rotations, n_best_rotations=30):
        molecules = self.molecules
        self.molecules = []
        for mol in molecules:
            rots = sortRotationsByEntropy(mol[:, :3], rotations)[:n_best_rotations]
            for xyzs_rot in rotate(mol[:, :3], rots):
                self.molecules.append(np.concatenate([xyzs_rot, mol[:, 3:4], mol[:, 4:5]], axis=1))

    def randomize_tip(self, max_tilt=0.5):
        self.afmulator.tipR0[:2] = np.array(getRandomUniformDisk()) * max_tilt

    def randomize_distance(self, delta=0.25):
        self.distAboveActive = np.random.uniform(self.distAbove - delta, self.distAbove + delta)

    def randomize_mol_parameters(self, rndQmax=0.0, rndRmax=0.0, rndEmax=0.0, rndAlphaMax=0.0):
        n = len(self.qs)
        if rndQmax > 0:
            self.qs[:] += rndQmax * (np.random.rand(n) - 0.5)
        if rndRmax > 0:
            self.REAs[:, 0] += rndRmax * (np.random.rand(n) - 0.5)
        if rndEmax > 0:
            self.REAs[:, 1] *= 1 + rndEmax * (np.random.rand(n) - 0.5)
        if rndAlphaMax > 0:
            self.REAs[:, 2] *= 1 + rndAlphaMax * (np.random.rand(n) - 0.5)

    # ------------------------------------------------------------ callbacks

    def on_batch_start(self):
        """Run at the start of each batch."""

    def on_sample_start(self):
        """Run before the first image of each sample."""

    def on_afm_start(self):
        """Run before every image."""

    def on_afm_end(self):
        """Run after every image (self.Xs holds it)."""


class GeneratorAFMtrainer:
    """Batches (Xs, Ys, mols, sws) from sample dicts (ppafm/ml/Generator.py:240-663):
    Xs [n_batch, n_tip, nx, ny, nz_out], Ys [n_batch, n_aux, nx, ny], mols the
    [n_atoms, 5] arrays of the rotated molecules, sws [n_batch, n_tip, 2, 3] the scan windows.
    Each sample dict holds the AFMulator.eval arguments (at least xyzs and Zs).  Simulation
    types: ``'LJ'``, ``'LJ+PC'`` (point-charge tip) and ``'LJ+Hartree'`` (the sample's
    ``qs`` is a HartreePotential; ``rhos`` one tip density per tip -- a multipole dict or a
    TipDensity on the force-field grid -- or None for the point-charge tip Qs, QZs);
    ``'FDBM'`` is not supported.  Images are queued on
    the GPU and copied to the host once per batch, as in InverseAFMtrainer.  Aux maps are
    callables ``aux_map(xyzqs, Zs, pot, rot) -> [nx, ny]`` (pot the HartreePotential or None);
    one with a ``scan_window`` attribute follows the scan window."""

    def __init__(self, afmulator, aux_maps, sample_generator, sim_type="LJ", batch_size=30, distAbove=5.3, iZPPs=[8], Qs=None, QZs=None, rhos=None, rho_deltas=None, ignore_elements=[], density_cutoff=None):
        self.afmulator = afmulator
        self.aux_maps = aux_maps
        self.sample_generator = sample_generator
        self.sim_type = sim_type.lower()
        if self.sim_type == "fdbm" or rho_deltas is not None:
            raise NotImplementedError("the FDBM simulation type is not supported")
        if self.sim_type not in ("lj", "lj+pc", "lj+hartree"):
            raise ValueError(f"Unknown simulation type `{sim_type}`")
        if rhos is not None and len(rhos) != len(iZPPs):
            raise ValueError(f"The length of rhos ({len(rhos)}) does not match the length of iZPPs ({len(iZPPs)})")
        self.rhos = list(rhos) if rhos is not None else [None] * len(iZPPs)
        self.batch_size = batch_size
        self.distAbove = distAbove
        self.distAboveActive = distAbove
        self.iZPPs = iZPPs
        self.ignore_elements = ignore_elements
        self.density_cutoff = None
        if Qs is None or QZs is None:
            if self.sim_type == "lj+pc":
                raise ValueError("Both Qs and QZs should be specified when using point-charge electrostatics.")
            self.Qs = self.QZs = [[0, 0, 0, 0] for _ in range(len(iZPPs))]
        else:
            assert len(Qs) == len(QZs) == len(iZPPs), "Inconsistent lengths for tip charge arrays."
            self.Qs = Qs
            self.QZs = QZs
        sw = self.afmulator.scan_window
        self.scan_window = sw
        self.scan_size = (sw[1][0] - sw[0][0], sw[1][1] - sw[0][1], sw[1][2] - sw[0][2])
        self.scan_dim = self.afmulator.scan_dim
        self.df_steps = self.afmulator.df_steps
        self.z_size = self.scan_dim[2] - self.df_steps + 1
        self.last_timing = {}

    def __iter__(self):
        self.sample_dict = {}
        self.sample_iterator = iter(self.sample_generator)
        self.iteration_done = False
        return self

    def __next__(self):
        if self.iteration_done:
            raise StopIteration
        self.on_batch_start()
        t0 = time.perf_counter()
        afm = self.afmulator
        mols, sws, Ys = [], [], []
        ntip = len(self.iZPPs)
        Xd = torch.empty((self.batch_size, ntip, self.scan_dim[0], self.scan_dim[1], self.z_size), dtype=torch.float32, device="cuda")
        for s in range(self.batch_size):
            try:
                self.sample_dict = self._load_next_sample()
            except StopIteration:
                self.sample_dict = None
                self.iteration_done = True
                break
            rot = self.sample_dict["rot"]
            xyzs = self.sample_dict["xyzs"]
            Zs = self.sample_dict["Zs"]
            pot = self.sample_dict["qs"] if isinstance(self.sample_dict["qs"], HartreePotential) else None
            qs = np.zeros(len(Zs)) if pot is not None else self.sample_dict["qs"]
            xyz_center = xyzs.mean(axis=0)
            self.xyzs_rot = np.dot(xyzs - xyz_center, rot.T) + xyz_center
            mols.append(np.concatenate([self.xyzs_rot, qs[:, None], Zs[:, None]], axis=1))
            self.handle_positions()
            self.on_sample_start()
            sws_ = []
            for i, (iZPP, Q, Qz, rho) in enumerate(zip(self.iZPPs, self.Qs, self.QZs, self.rhos)):
                afm.iZPP = iZPP
                afm.setQs(Q, Qz)
                if rho is not None:
                    afm.setRho(rho, sigma=afm.sigma, B_pauli=afm.B_pauli)
                self.sample_dict["REAs"] = PPU.getAtomsREA(afm.iZPP, self.sample_dict["Zs"], afm.typeParams, alphaFac=-1.0)
                self.handle_distance()
                afm.setScanWindow(self.scan_window, self.scan_dim, df_steps=self.df_steps)
                afm.setLvec()
                self.on_afm_start()
                d = self.sample_dict
                afm.prepareFF(d["xyzs"], d["Zs"], d["qs"], rho_sample=d.get("rho_sample"), sample_lvec=d.get("sample_lvec"), rot=d["rot"], rot_center=d.get("rot_center"), REAs=d["REAs"])
                afm.evalAFM(out=Xd[s, i])
                sws_.append(np.array(self.scan_window))
            xyzqs = np.concatenate([xyzs, qs[:, None]], axis=1)
            Ys.append([aux_map(xyzqs, Zs, pot, rot) for aux_map in self.aux_maps])
            sws.append(sws_)
        if len(mols) == 0:
            raise StopIteration
        Xs = Xd[: len(mols)].cpu().numpy()  # one copy per batch
        Ys = np.array(Ys)
        sws = np.array(sws)
        self.last_timing["batch"] = time.perf_counter() - t0
        return Xs, Ys, mols, sws

    def _load_next_sample(self):
        sample_dict = next(self.sample_iterator)
        if self.sim_type == "lj":
            sample_dict["qs"] = np.zeros((len(sample_dict["Zs"]),), dtype=np.float32)
            sample_dict["rho_sample"] = None
        elif ("qs" not in sample_dict) or (sample_dict["qs"] is None):
            raise ValueError("Sample dict does not contain qs, which is required for a simulation with electrostatics")
        elif self.sim_type == "lj+pc":
            if not isinstance(sample_dict["qs"], np.ndarray):
                raise ValueError("qs in sample dict is not a numpy array, which is required for a LJ+PC simulation.")
            sample_dict["rho_sample"] = None
        else:
            if not isinstance(sample_dict["qs"], HartreePotential):
                raise ValueError("qs in sample dict is not a HartreePotential, which is required for a LJ+Hartree simulation.")
            sample_dict["rho_sample"] = None
        if "rot" not in sample_dict:
            sample_dict["rot"] = np.eye(3)
        return sample_dict

    def __len__(self):
        if not hasattr(self.sample_generator, "__len__"):
            raise RuntimeError("Cannot infer the number of batches because sample generator does not have length attribute.")
        return int(np.floor(len(self.sample_generator) / self.batch_size))

    def _mask(self):
        Zs = self.sample_dict["Zs"]
        return np.prod([Zs != elem for elem in self.ignore_elements], axis=0).astype(bool)

    def handle_positions(self):
        """Moves the scan window laterally onto the molecule's centre."""
        ss = self.scan_size
        sw = self.scan_window
        xyzs = self.xyzs_rot[self._mask()] if self.ignore_elements else self.xyzs_rot
        c = xyzs[:, :2].mean(axis=0)
        sw = ((c[0] - ss[0] / 2, c[1] - ss[1] / 2, sw[0][2]), (c[0] + ss[0] / 2, c[1] + ss[1] / 2, sw[1][2]))
        self.scan_window = sw
        for aux_map in self.aux_maps:
            if hasattr(aux_map, "scan_window"):
                aux_map.scan_window = ((sw[0][0], sw[0][1]), (sw[1][0], sw[1][1]))

    def handle_distance(self):
        """Puts the scan window's bottom distAboveActive above the molecule's van der Waals surface."""
        RvdwPP = self.afmulator.typeParams[self.afmulator.iZPP - 1][0]
        Rvdw = self.sample_dict["REAs"][:, 0] - RvdwPP
        zs = self.xyzs_rot[:, 2]
        if self.ignore_elements:
            m = self._mask()
            zs, Rvdw = zs[m], Rvdw[m]
        imax = np.argmax(zs + Rvdw)
        total_distance = self.distAboveActive + Rvdw[imax] + RvdwPP - (zs.max() - zs[imax])
        z_min = zs.max() + total_distance
        sw = self.scan_window
        self.scan_window = ((sw[0][0], sw[0][1], z_min), (sw[1][0], sw[1][1], z_min + self.scan_size[2]))

    def set_fdbm_parameters(self, A_pauli, B_pauli):
        """FDBM Pauli parameters (ppafm/ml/Generator.py:617-635); the reference does nothing
        unless the simulation type is FDBM, which this library does not provide."""

    def randomize_df_steps(self, minimum=4, maximum=20):
        """Random number of Δf steps, keeping the output z size and the z step."""
        self.df_steps = np.random.randint(minimum, maximum + 1)
        self.scan_dim = (self.scan_dim[0], self.scan_dim[1], self.z_size + self.df_steps - 1)
        self.scan_size = (self.scan_size[0], self.scan_size[1], self.afmulator.dz * self.scan_dim[2])

    def randomize_tip(self, max_tilt=0.5):
        self.afmulator.tipR0[:2] = max_tilt * np.array(getRandomUniformDisk())

    def randomize_distance(self, delta=0.25):
        self.distAboveActive = np.random.uniform(self.distAbove - delta, self.distAbove + delta)

    def on_batch_start(self):
        """Run at the start of each batch."""

    def on_sample_start(self):
        """Run after a new sample is loaded."""

    def on_afm_start(self):
        """Run before every image."""


def sortRotationsByEntropy(xyzs, rotations):
    scored = [(PPU.maxAlongDirEntropy(xyzs, np.asarray(rot)[2].ravel().copy())[2], rot) for rot in rotations]
    scored.sort(key=lambda item: -item[0])
    return [rot for _, rot in scored]


def rotate(xyzs, rotations):
    return [np.dot(xyzs, np.asarray(rot).T) for rot in rotations]


def getRandomUniformDisk():
    """A point uniformly distributed over the unit disk."""
    rnd = np.random.rand(2)
    rnd[0] = np.sqrt(rnd[0])
    rnd[1] *= 2.0 * np.pi
    return rnd[0] * np.cos(rnd[1]), rnd[0] * np.sin(rnd[1])
