"""Grid data of the AFMulator's Hartree route, restating the grid classes of ppafm/ocl/field.py
(DataGrid :115-573, HartreePotential :575, TipDensity :583-650, MultipoleTipDensity :653-704)
on libppgpu.

A grid's values live on the host (a float32 numpy array), in device memory (a float32 CUDA
tensor), or both; each side is made from the other on first use (``array`` downloads,
``device()`` uploads).  Operations run on the GPU and return grids that live in device memory,
like the reference's OpenCL buffers.  Shapes are 3-D (scalar grids) or 4-D with 4 components
(the output of ``grad``); the first axis runs along the first lattice vector.
"""

import warnings

import numpy as np
import torch

from . import io
from ._lib import check, dptr, iptr, lib, stream_handle, tptr


def _lvec4(lvec):
    lvec = np.array(lvec, dtype=np.float64)
    if lvec.shape == (3, 3):
        lvec = np.vstack([np.zeros(3), lvec])
    assert lvec.shape == (4, 3), f"lvec should have shape (4, 3), but has shape {lvec.shape}"
    return lvec


class DataGrid:
    """Values on a periodic grid.  array: numpy array or CUDA tensor, 3-D or 4-D; lvec [4, 3]:
    the origin, then the three lattice vectors spanning the cell."""

    def __init__(self, array, lvec, shape=None):
        self._array = None
        self._dev = None
        if isinstance(array, torch.Tensor) and array.is_cuda:
            t = array.detach()
            if shape is not None:
                t = t.reshape(-1)[: int(np.prod(shape))].view(tuple(int(x) for x in shape))
            self._dev = t.to(torch.float32).contiguous()
            self.shape = tuple(self._dev.shape)
        else:
            a = array.cpu().numpy() if isinstance(array, torch.Tensor) else array
            self._array = np.ascontiguousarray(a, dtype=np.float32)
            self.shape = tuple(self._array.shape)
        if len(self.shape) not in (3, 4):
            raise ValueError(f"Dimension of array should be 3 or 4, but got {len(self.shape)}")
        self.lvec = _lvec4(lvec)

    @property
    def origin(self):
        return self.lvec[0]

    @property
    def step(self):
        """Single steps along each lattice vector (rows)."""
        return np.stack([self.lvec[i + 1] / self.shape[i] for i in range(3)])

    @property
    def cell_vol(self):
        """Volume of one grid cell (A^3)."""
        a, b, c = self.step
        return abs(np.cross(a, b).dot(c))

    @property
    def array(self):
        """Host values (copied from the device on first use)."""
        if self._array is None:
            self._array = self._dev.cpu().numpy()
        return self._array

    def device(self):
        """Device values (copied to the device on first use)."""
        if self._dev is None:
            self._dev = torch.from_numpy(self._array).cuda()
        return self._dev

    @property
    def n(self):
        return int(np.prod(self.shape))

    def update_array(self, array, lvec):
        """New values and cell (the device copy is refreshed on next use)."""
        self.__init__(array, lvec)

    def release(self, keep_on_host=True):
        """Frees the device copy (after copying it to the host if keep_on_host)."""
        if self._dev is not None:
            if keep_on_host:
                self.array
            self._dev = None

    @classmethod
    def from_file(cls, file_path, scale=1.0):
        """(grid, xyzs, Zs) from a cube file or an XSF datagrid (io.py loadCUBE + loadAtomsCUBE,
        loadXSFData + loadXSFGeom); values times scale."""
        file_path = str(file_path)
        if file_path.endswith(".cube"):
            data, lvec, _, _ = io.loadCUBE(file_path, xyz_order=True)
            Zs, x, y, z, _ = io.loadAtomsCUBE(file_path)
        elif file_path.endswith(".xsf"):
            data, lvec, _, _ = io.loadXSFData(file_path, xyz_order=True)
            try:
                (Zs, x, y, z, _), _, _ = io.loadXSFGeom(file_path)
            except ValueError:
                warnings.warn(f"Could not read geometry from {file_path} in DataGrid.from_file.")
                Zs = np.zeros(1)
                x = y = z = np.zeros((1, 1))
        else:
            raise ValueError(f"Unsupported file format in file `{file_path}`")
        if not np.allclose(scale, 1.0):
            data = data * scale
        return cls(data, lvec), np.stack([np.asarray(x).ravel(), np.asarray(y).ravel(), np.asarray(z).ravel()], axis=1), np.array(Zs)

    def to_file(self, file_path, clamp=None):
        """Saves as .xsf or .npy (a 4-D grid as its vector part and the _w component)."""
        import os

        head, ext = os.path.splitext(str(file_path))
        if ext not in (".xsf", ".npy"):
            raise ValueError(f"Unsupported file extension `{ext}` for saving data grid.")
        fmt = ext[1:]
        a = self.array.copy()
        if len(self.shape) == 3:
            if clamp:
                a[a > clamp] = clamp
            io.save_scal_field(head, a, self.lvec, data_format=fmt)
        else:
            assert self.shape[3] == 4, "Wrong number of components"
            if clamp:
                io.limit_vec_field(a, Fmax=clamp)
                a[..., 3][a[..., 3] > clamp] = clamp
            io.save_vec_field(head, a[..., :3], self.lvec, data_format=fmt)
            io.save_scal_field(head + "_w", a[..., 3], self.lvec, data_format=fmt)

    # ------------------------------------------------------------ operations on the GPU

    def _out(self, in_place, shape=None):
        if in_place:
            self._array = None  # the host copy goes stale
            return self
        return type(self)(torch.empty(shape or self.shape, dtype=torch.float32, device="cuda"), self.lvec)

    def clamp(self, minimum=-np.inf, maximum=np.inf, clamp_type="hard", soft_clamp_width=1.0, in_place=True, stream=None):
        """Values clipped to [minimum, maximum] ('hard') or blended into the bounds by a
        sigmoid of width soft_clamp_width ('soft') (field.py:288-340)."""
        if clamp_type not in ("hard", "soft"):
            raise ValueError(f"Unsupported clamp type `{clamp_type}`")
        src = self.device()
        out = self._out(in_place)
        check(lib().ppgpu_scalar_clamp(tptr(src), tptr(out.device()), self.n, float(minimum), float(maximum), int(clamp_type == "soft"), float(soft_clamp_width), stream_handle(stream)))
        return out

    def add_mult(self, array, scale=1.0, in_place=True, stream=None):
        """self + scale * array (field.py:342-376)."""
        if tuple(array.shape) != self.shape:
            raise ValueError(f"grid shapes differ: {array.shape} and {self.shape}")
        src = self.device()
        out = self._out(in_place)
        check(lib().ppgpu_scalar_add_mult(tptr(src), tptr(array.device()), tptr(out.device()), self.n, float(scale), stream_handle(stream)))
        return out

    def _get_normalization_factor(self, stream=None):
        """sum of all values / sum of the positive values (field.py:431-452), float64 sums."""
        sums = torch.empty(2, dtype=torch.float64, device="cuda")
        check(lib().ppgpu_scalar_sums(tptr(self.device()), self.n, tptr(sums), stream_handle(stream)))
        s = sums.cpu().numpy()
        return s[0] / s[1] if s[1] != 0 else np.inf * np.sign(s[0])

    def power_positive(self, p=1.2, normalize=True, in_place=True, stream=None):
        """max(0, value)^p, times (sum / positive sum)^p when normalize (field.py:378-429)."""
        scale = 1.0
        if normalize:
            f = self._get_normalization_factor(stream)
            assert f > 0, "Normalizing scaling factor should be positive."
            scale = float(np.float32(f) ** np.float32(p))
        src = self.device()
        out = self._out(in_place)
        check(lib().ppgpu_scalar_power(tptr(src), tptr(out.device()), self.n, float(p), scale, stream_handle(stream)))
        return out

    def grad(self, scale=1.0, array_out=None, order="C", stream=None):
        """Periodic centred-difference gradient (field.py:454-513): a 4-D grid (d/dx, d/dy, d/dz,
        value) times scale (a number or 4 numbers).  Only C order is produced here."""
        if len(self.shape) == 4 and self.shape[3] > 1:
            raise RuntimeError("Can only take gradient of a datagrid with a single component.")
        if order != "C":
            raise NotImplementedError("the gradient is stored in C order")
        sc = np.full(4, float(scale)) if np.ndim(scale) == 0 else np.array(scale, dtype=np.float64)
        if len(sc) != 4:
            raise ValueError(f"Scale should have length 4, but got {len(sc)}.")
        st = self.step
        if (st != np.diag(np.diag(st))).any():
            raise NotImplementedError("the gradient needs a rectangular grid")
        shape_out = self.shape[:3] + (4,)
        out = array_out if array_out is not None else torch.empty(shape_out, dtype=torch.float32, device="cuda")
        check(lib().ppgpu_grad_fd(tptr(self.device()), iptr(np.array(self.shape[:3], dtype=np.int32)), dptr(np.ascontiguousarray(np.diag(st))), dptr(sc), tptr(out), 0, stream_handle(stream)))
        return DataGrid(out, self.lvec)

    def interp_at(self, lvec_new, shape_new, array_out=None, rot=np.eye(3), rot_center=np.zeros(3), stream=None):
        """Periodic trilinear interpolation onto the grid lvec_new / shape_new, the new grid's
        points rotated about rot_center by rot (field.py:515-572)."""
        if len(self.shape) == 4 and self.shape[3] > 1:
            raise NotImplementedError("Interpolation for 4D grids is not implemented.")
        lvec_new = _lvec4(lvec_new)
        shape_new = tuple(int(x) for x in shape_new[:3])
        out = array_out if array_out is not None else torch.empty(shape_new, dtype=torch.float32, device="cuda")
        step_out = np.ascontiguousarray(lvec_new[1:] / np.array(shape_new)[:, None])
        check(lib().ppgpu_interp_grid(tptr(self.device()), iptr(np.array(self.shape[:3], dtype=np.int32)), dptr(np.ascontiguousarray(self.origin)), dptr(np.ascontiguousarray(self.step)),
                                      tptr(out), iptr(np.array(shape_new, dtype=np.int32)), dptr(np.ascontiguousarray(lvec_new[0])), dptr(step_out),
                                      dptr(np.ascontiguousarray(rot, dtype=np.float64)), dptr(np.ascontiguousarray(rot_center, dtype=np.float64)), stream_handle(stream)))
        return type(self)(out, lvec_new)


class HartreePotential(DataGrid):
    """Sample Hartree potential (V)."""


class ElectronDensity(DataGrid):
    """Sample electron density (e/A^3)."""


class TipDensity(DataGrid):
    """Tip charge density (e/A^3), centred on the grid origin (wrapped periodically)."""

    def interp_at(self, lvec_new, shape_new, array_out=None, stream=None):
        """The density resampled onto another grid about the origin: the grids' origins are
        ignored, the middle of the grid grows or shrinks and the corners stay, points beyond half
        of this cell are zero (field.py:606-650)."""
        if len(self.shape) == 4 and self.shape[3] > 1:
            raise NotImplementedError("Interpolation for 4D grids is not implemented.")
        lvec_new = _lvec4(lvec_new)
        shape_new = tuple(int(x) for x in shape_new[:3])
        out = array_out if array_out is not None else torch.empty(shape_new, dtype=torch.float32, device="cuda")
        step_out = np.ascontiguousarray(lvec_new[1:] / np.array(shape_new)[:, None])
        check(lib().ppgpu_interp_tip_grid(tptr(self.device()), iptr(np.array(self.shape[:3], dtype=np.int32)), dptr(np.ascontiguousarray(self.step)), dptr(np.ascontiguousarray(self.lvec[1:])),
                                          tptr(out), iptr(np.array(shape_new, dtype=np.int32)), dptr(step_out), stream_handle(stream)))
        return TipDensity(out, lvec_new)


class MultipoleTipDensity(TipDensity):
    """Multipole tip density on a periodic grid (field.py:653-704): normalised Gaussian of width
    sigma times the multipole combination (dict of 's', 'px', 'py', 'pz', 'dz2', 'dy2', 'dx2',
    'dxy', 'dxz', 'dyz' weights), centred on the grid origin.  lvec [3, 3]: lattice vectors."""

    def __init__(self, lvec, shape, center=(0, 0, 0), sigma=0.71, multipole={"dz2": -0.1}, tilt=0.0):
        from .fieldFFT import FFTGrid

        if np.any(np.asarray(center) != 0) or tilt != 0.0:
            raise NotImplementedError("the multipole tip density is made centred on the origin and untilted")
        lvec = np.asarray(lvec, dtype=np.float64)
        shape = tuple(int(x) for x in shape[:3])
        rho = FFTGrid(shape).probe_density(np.vstack([np.zeros(3), lvec]), sigma, multipole)
        super().__init__(rho, np.vstack([np.zeros(3), lvec]))
