"""Host-side helpers of the hot path, mirroring ppafm/common.py.

Pure host arithmetic (Δf kernels, periodic images, LJ mixing, scan grids) lives here as
numpy; the per-column Fz -> Δf convolution runs on the GPU (``Fz2df``).
"""

import numpy as np

from . import species as _species
from ._lib import check, dptr, lib, stream_handle, tptr

# ppafm/common.py:20-21
eVA_Nm = 16.0217662
CoulombConst = 14.399645

loadSpecies = _species.loadSpecies
loadSpeciesLines = _species.loadSpeciesLines
getFFdict = _species.getFFdict
atom2iZ = _species.atom2iZ
atoms2iZs = _species.atoms2iZs


# ------------------------------------------------------------------ parameters

# Defaults of PpafmParameters (common.py:26-78), in the reference's order.
_PARAM_DEFAULTS = dict(
    PBC=True, nPBC=[1, 1, 1], gridN=[-1, -1, -1], gridO=[0.0, 0.0, 0.0], gridA=[20.0, 0.0, 0.0], gridB=[0.0, 20.0, 0.0], gridC=[0.0, 0.0, 20.0],
    FFgrid0=[-1.0, -1.0, -1.0], FFgridA=[-1.0, -1.0, -1.0], FFgridB=[-1.0, -1.0, -1.0], FFgridC=[-1.0, -1.0, -1.0], moleculeShift=[0.0, 0.0, 0.0],
    probeType="O", charge=0.00, Apauli=18.0, Bpauli=1.0, ffModel="LJ", Rcore=0.7, r0Probe=[0.00, 0.00, 4.00], stiffness=[-1.0, -1.0, -1.0],
    klat=0.5, krad=20.00, tip="s", sigma=0.7, scanStep=[0.10, 0.10, 0.10], scanMin=[0.0, 0.0, 5.0], scanMax=[20.0, 20.0, 8.0],
    scanTilt=[0.0, 0.0, -0.1], tiltedScan=False, kCantilever=1800.0, f0Cantilever=30300.0, Amplitude=1.0, plotSliceFrom=16, plotSliceTo=22,
    plotSliceBy=1, imageInterpolation="bicubic", colorscale="gray", colorscale_kpfm="seismic", ddisp=0.05, aMorse=-1.6, Rtip=30.0,
    permit=0.00552634959, vdWDampKind=2, Vbias=0.0,
)


class PpafmParameters:
    """Simulation parameters with the reference's names and defaults (common.py:26-160):
    attributes, ``from_file`` for params.ini (``load_ini``: one ``key value...`` per line,
    ``#`` comments, values typed like the defaults) and params.toml, ``to_file`` for toml.
    Every function here that takes ``parameters`` accepts this object or a dict."""

    def __init__(self, **kw):
        for k, v in _PARAM_DEFAULTS.items():
            setattr(self, k, list(v) if isinstance(v, list) else v)
        self.apply_options(kw)

    def __setattr__(self, key, value):
        if key not in _PARAM_DEFAULTS:
            raise AttributeError(f"Parameter {key} is not known")
        object.__setattr__(self, key, value)

    @classmethod
    def from_file(cls, file_path="params.ini"):
        from pathlib import Path

        file_path = Path(file_path)
        obj = cls()
        try:
            with open(file_path, "rb" if file_path.suffix == ".toml" else "r") as f:
                if file_path.suffix == ".ini":
                    obj.load_ini(f.readlines())
                elif file_path.suffix == ".toml":
                    import tomllib

                    obj.apply_options(tomllib.load(f))
                else:
                    raise ValueError(f"Unsupported file extension: {file_path.suffix}")
        except FileNotFoundError:
            raise ValueError(f"File {file_path} not found")
        return obj

    def apply_options(self, obj):
        for key, value in obj.items():
            if key in _PARAM_DEFAULTS and value is not None:
                setattr(self, key, value)

    def model_dump(self):
        return {k: getattr(self, k) for k in _PARAM_DEFAULTS}

    def __eq__(self, other):
        return isinstance(other, PpafmParameters) and self.model_dump() == other.model_dump()

    def __repr__(self):
        return "PpafmParameters(" + ", ".join(f"{k}={v!r}" for k, v in self.model_dump().items()) + ")"

    def to_file(self, file_path="params.toml"):
        """Writes the parameters as toml (flat keys; strings, numbers, booleans, lists)."""
        from pathlib import Path

        file_path = Path(file_path)
        if file_path.suffix != ".toml":
            raise ValueError(f"Unsupported file extension: {file_path.suffix}")

        def fmt(v):
            if isinstance(v, bool):
                return "true" if v else "false"
            if isinstance(v, str):
                return '"' + v.replace("\\", "\\\\").replace('"', '\\"') + '"'
            if isinstance(v, (list, tuple)):
                return "[" + ", ".join(fmt(x) for x in v) + "]"
            return repr(float(v)) if isinstance(v, float) else str(int(v))

        with open(file_path, "w") as f:
            for k, v in self.model_dump().items():
                f.write(f"{k} = {fmt(v)}\n")

    def load_ini(self, lines):
        """params.ini lines (common.py:119-160): bools by their first letter, lists of three
        numbers (a string and a number for a tip list), gridN from the cell when not given."""
        for line in lines:
            words = line.split("#")[0].strip().split()
            if len(words) < 2:
                continue
            key = words[0]
            if key not in _PARAM_DEFAULTS:
                raise ValueError(f"Parameter {key} is not known")
            val = getattr(self, key)
            try:
                if isinstance(val, bool):
                    setattr(self, key, words[1].strip()[0] in "Tt")
                elif isinstance(val, float):
                    setattr(self, key, float(words[1]))
                elif isinstance(val, int):
                    setattr(self, key, int(words[1]))
                elif isinstance(val, str):
                    setattr(self, key, words[1])
                elif isinstance(val, list):
                    if isinstance(val[0], float):
                        setattr(self, key, [float(words[1]), float(words[2]), float(words[3])])
                    elif isinstance(val[0], int):
                        setattr(self, key, [int(words[1]), int(words[2]), int(words[3])])
                    else:
                        setattr(self, key, [str(words[1]), float(words[2])])
            except (ValueError, IndexError):
                raise ValueError(f"Error parsing parameters on line: {line}") from None
        if self.gridN[0] <= 0:
            autoGridN(self)
        if isinstance(self.tip, str):
            self.tip = self.tip.replace('"', "").replace("'", "")


def autoGridN(parameters):
    """Grid size at 10 points per A of each cell vector (common.py:518-522)."""
    for k, v in enumerate((parameters.gridA, parameters.gridB, parameters.gridC)):
        parameters.gridN[k] = round(np.linalg.norm(v) * 10)
    return parameters.gridN


# ------------------------------------------------------------------ Δf weights


def get_df_weight(Amp, dz=0.1):
    """Discretised Giessibl convolution kernel for peak-to-peak amplitude Amp and step dz
    (common.py:333-392): linear interpolation of F between samples, integrated against
    t/sqrt(1-t^2); returned already reversed for np.convolve."""
    n = int(np.ceil(Amp / dz))
    t = np.linspace(-1 + 2 * n * dz / Amp, -1, n + 1)
    f = np.zeros(n + 1)
    f2 = np.zeros(n + 1)
    if n > 1:
        ti = t[1:-1]
        f[1:-1] = np.sqrt(1 - ti * ti)
        f2[1:-1] = (np.arccos(-ti) - ti * f[1:-1]) / 2.0
    f2[0] = np.pi / 2  # t >= 1 behaves like t = 1
    df = f[:-1] - f[1:]
    df2 = f2[:-1] - f2[1:]
    w = np.zeros(n + 1)
    w[1:] = t[:-1] * df + df2
    w[:-1] -= t[1:] * df + df2
    return w / (np.pi * dz)


def get_simple_df_weight(n=10, dz=0.1):
    """The simpler kernel the AFMulator uses (common.py:395-418)."""
    n = max(int(n), 2)
    t = np.linspace(-1 + 0.5 / n, 1 - 0.5 / n, n - 1)
    f = np.sqrt(1 - t * t)
    w = np.zeros(n)
    w[:-1] = f
    w[1:] -= f
    w0 = np.sum(np.linspace(-1, 1, n) * w)
    return w / (w0 * n * dz)


def Fz2df(F, dz, k0, f0, amplitude=1.0, units=16.0217656, out=None, stream=None):
    """Frequency shift from Fz along the last axis (common.py:421-430) on the GPU.

    F: numpy array (any float dtype; the result is float64 like the reference) or a CUDA
    float32 torch tensor (result stays on the device).  Same 'valid'-mode convolution with
    get_df_weight(amplitude, dz), scaled by units*f0/k0."""
    import torch

    W = get_df_weight(amplitude, dz=dz)
    scale = units * f0 / k0
    host = not (isinstance(F, torch.Tensor) and F.is_cuda)
    Ft = torch.as_tensor(np.ascontiguousarray(F, dtype=np.float32)).cuda() if host else F.contiguous().float()
    nz = Ft.shape[-1]
    nw = len(W)
    if nw > nz:
        raise ValueError(f"amplitude/dz needs {nw} z samples, F has {nz}")
    nout = nz - nw + 1
    ncol = Ft.numel() // nz
    o = torch.empty(Ft.shape[:-1] + (nout,), dtype=torch.float32, device=Ft.device)
    W = np.ascontiguousarray(W, dtype=np.float64)
    check(lib().ppgpu_fz2df(tptr(Ft), ncol, nz, nw, dptr(W), scale, tptr(o), stream_handle(stream)))
    if host:
        res = o.cpu().numpy().astype(np.float64)
        if out is not None:
            out[...] = res
            return out
        return res
    return o


def Fz2df_tilt(F, d, k0, f0, amplitude=1.0, units=16.0217656):
    """Frequency shift of a tilted scan (common.py:433-445): each force component of
    F [nx, ny, nz, 3] convolved along the scan with get_df_weight(amplitude, |d|) on the
    GPU, projected on the scan direction d, scaled by units*f0/k0 (float64 result)."""
    d = np.asarray(d, dtype=np.float64)
    dr = float(np.sqrt(d[0] ** 2 + d[1] ** 2 + d[2] ** 2))
    F = np.asarray(F)
    comps = [Fz2df(np.ascontiguousarray(F[..., k]), dz=dr, k0=1.0, f0=1.0, amplitude=amplitude, units=1.0) for k in range(3)]
    return (comps[0] * d[0] + comps[1] * d[1] + comps[2] * d[2]) * units * f0 / k0


# ------------------------------------------------------------------ rotations


def rotation_matrix(axis, theta):
    """Counterclockwise rotation by theta about axis (common.py:448-466), from the unit
    quaternion (cos(theta/2), -axis sin(theta/2)) in the reference's sign convention."""
    axis = np.asarray(axis, dtype=np.float64)
    axis = axis / np.sqrt(np.dot(axis, axis))
    a = np.cos(theta / 2.0)
    b, c, d = -axis * np.sin(theta / 2.0)
    return np.array(
        [
            [a * a + b * b - c * c - d * d, 2 * (b * c + a * d), 2 * (b * d - a * c)],
            [2 * (b * c - a * d), a * a + c * c - b * b - d * d, 2 * (c * d + a * b)],
            [2 * (b * d + a * c), 2 * (c * d - a * b), a * a + d * d - b * b - c * c],
        ]
    )


def makeRotJitter(n=10, maxAngle=0.3):
    """50 random small rotations, angle up to maxAngle about random axes (common.py:469-476;
    like the reference, n is not used)."""
    r = (np.random.rand(50, 4) - 0.5) * 2
    return [rotation_matrix(r[i, :3] / np.sqrt(np.dot(r[i, :3], r[i, :3])), r[i, 3] * maxAngle) for i in range(50)]


def genRotations(axis, thetas):
    return np.array([rotation_matrix(axis, t) for t in thetas])


def sphereTangentSpace(n=100):
    """n orthonormal frames whose third rows are a golden-angle spiral over the sphere, the
    first row horizontal (common.py:483-497)."""
    theta = np.pi * (3.0 - np.sqrt(5.0)) * np.arange(n)
    z = np.linspace(1.0 - 1.0 / n, 1.0 / n - 1.0, n)
    r = np.sqrt(1.0 - z * z)
    c, s_ = np.cos(theta), np.sin(theta)
    rots = np.zeros((n, 3, 3))
    rots[:, 2] = np.stack([r * c, r * s_, z], axis=-1)
    rots[:, 0, 0] = -s_
    rots[:, 0, 1] = c
    rots[:, 1, :] = np.cross(rots[:, 2, :], rots[:, 0, :])
    return rots


def maxAlongDir(atoms, hdir):
    """(index, height) of the atom highest along hdir (common.py:500-503)."""
    x = np.dot(atoms[:, :3], np.asarray(hdir)[:, None])
    i = np.argmax(x)
    return i, x[i][0]


def maxAlongDirEntropy(atoms, hdir, beta=1.0):
    """maxAlongDir plus sum exp(beta (x - x_max)) over the atoms (common.py:506-510)."""
    x = np.dot(atoms[:, :3], np.asarray(hdir)[:, None])
    i = np.argmax(x)
    return i, x[i][0], np.sum(np.exp(beta * (x - x[i])))


def multRot(Zs, Rs, Qs, cLJs, rots, cog=(0, 0, 0)):
    """The atoms once per rotation about cog, rotations outer (common.py:779-802)."""
    Rs = np.asarray(Rs, dtype=np.float64)
    cog = np.asarray(cog, dtype=np.float64)
    R = np.concatenate([(Rs - cog) @ np.asarray(rot, dtype=np.float64).T + cog for rot in rots])
    m = len(rots)
    return np.tile(np.asarray(Zs), m), R, np.tile(np.asarray(Qs), m), np.tile(np.asarray(cLJs), (m, 1))


def wrapAtomsCell(Rs, da, db, avec, bvec):
    """Wraps Rs in place into the in-plane cell (avec, bvec), shifted by (da, db) cell
    fractions (common.py:596-605)."""
    M = np.array((avec[:2], bvec[:2]), dtype=np.float64)
    AB = np.dot(Rs[:, :2], np.linalg.inv(M))
    AB[:, 0] = (AB[:, 0] + 10 + da) % 1.0
    AB[:, 1] = (AB[:, 1] + 10 + db) % 1.0
    Rs[:, :2] = np.dot(AB, M)


# ------------------------------------------------------------- atoms and LJ


def PBCAtoms(Zs, Rs, Qs, avec, bvec, na=None, nb=None, parameters=None):
    """In-plane periodic images (common.py:608-628): images ordered i (along a) outer,
    j (along b) inner, atoms innermost; z unchanged.  na, nb default to the parameters' nPBC
    (1, 1 without parameters)."""
    if na is None:
        na = parameters.nPBC[0] if parameters is not None else 1
    if nb is None:
        nb = parameters.nPBC[1] if parameters is not None else 1
    Rs = np.asarray(Rs, dtype=np.float64).reshape(-1, 3)
    i, j = np.meshgrid(np.arange(-na, na + 1), np.arange(-nb, nb + 1), indexing="ij")
    i, j = i.reshape(-1, 1).astype(np.float64), j.reshape(-1, 1).astype(np.float64)
    nimg = i.shape[0]
    Rs_ = np.empty((nimg, Rs.shape[0], 3))
    for k in range(2):  # x + i a_k + j b_k, added in that order for every image
        Rs_[..., k] = (Rs[None, :, k] + i * avec[k]) + j * bvec[k]
    Rs_[..., 2] = Rs[None, :, 2]
    return np.tile(np.asarray(Zs), nimg), Rs_.reshape(-1, 3), np.tile(np.asarray(Qs, dtype=np.float64), nimg)


def parseAtoms(atoms, elem_dict, PBC=True, autogeom=False, lvec=None, parameters=None):
    """(iZs, Rs [n, 3], Qs) of loadGeometry's atom lists (common.py:828-848), replicated in the
    plane when PBC (cell from lvec, else the parameters' gridA/gridB).  autogeom (the
    reference's re-centring of the cell on the atoms) is not provided."""
    if autogeom:
        raise NotImplementedError("autogeom is not provided")
    Rs = np.array([atoms[1], atoms[2], atoms[3]], dtype=np.float64).T.copy()
    iZs = np.zeros(len(atoms[0])) if elem_dict is None else atoms2iZs(atoms[0], elem_dict)
    Qs = np.array(atoms[4], dtype=np.float64)
    if PBC:
        avec, bvec = (lvec[1], lvec[2]) if lvec is not None else (parameters.gridA, parameters.gridB)
        iZs, Rs, Qs = PBCAtoms(iZs, Rs, Qs, avec=avec, bvec=bvec, parameters=parameters)
    return iZs, Rs, Qs


def PBCAtoms3D(Zs, Rs, Qs, cLJs, lvec, npbc=(1, 1, 1)):
    """3-D periodic images (common.py:631-664): the atoms, then every other image (a outer, c
    inner).  Like the reference, the returned cLJs hold the images only (not the home cell)."""
    Rs = np.asarray(Rs, dtype=np.float64)
    lvec = np.asarray(lvec, dtype=np.float64)
    shifts = [(a, b, c) for a in range(-npbc[0], npbc[0] + 1) for b in range(-npbc[1], npbc[1] + 1) for c in range(-npbc[2], npbc[2] + 1) if (a, b, c) != (0, 0, 0)]
    R = np.concatenate([Rs] + [Rs + (a * lvec[0] + b * lvec[1] + c * lvec[2]) for a, b, c in shifts])
    m = len(shifts)
    cl = np.tile(np.asarray(cLJs), (m, 1)) if m else np.zeros((0, np.shape(cLJs)[1]))
    return np.tile(np.asarray(Zs), m + 1), R, np.tile(np.asarray(Qs), m + 1), cl


def getSampleAtomsREA(iZs, FFparams):
    """(R, E, alpha) of every atom's species (common.py:895-896)."""
    return np.array([(FFparams[i - 1][0], FFparams[i - 1][1], FFparams[i - 1][2]) for i in iZs])


def getAtomsRE(iZprobe, iZs, FFparams):
    """(R_ij, sqrt(E_i E_j)) pair parameters of the Morse model (common.py:899-905)."""
    Rpp, Epp = FFparams[iZprobe - 1][0], FFparams[iZprobe - 1][1]
    REs = np.array([(Rpp + FFparams[z - 1][0], Epp * FFparams[z - 1][1]) for z in iZs])
    REs[:, 1] = np.sqrt(REs[:, 1])
    return REs


def PBCAtoms3D_np(Zs, Rs, Qs, cLJs, REAs, lvec, npbc=(1, 1, 1)):
    """3-D periodic images with the home cell first, float32 (common.py:728-776)."""
    lvec = np.asarray(lvec, dtype=np.float64)
    shifts = [(0, 0, 0)] + [(a, b, c) for a in range(-npbc[0], npbc[0] + 1) for b in range(-npbc[1], npbc[1] + 1) for c in range(-npbc[2], npbc[2] + 1) if (a, b, c) != (0, 0, 0)]
    Rs = np.asarray(Rs)
    xyz = np.concatenate([Rs + (a * lvec[0] + b * lvec[1] + c * lvec[2])[None, :] for a, b, c in shifts]).astype(np.float32)
    m = len(shifts)
    Zs_ = np.tile(np.asarray(Zs, dtype=np.int32), m)
    qs_ = np.tile(np.asarray(Qs), m).astype(np.float32)
    cLJs_ = None if cLJs is None else np.tile(np.asarray(cLJs), (m, 1)).astype(np.float32)
    REAs_ = None if REAs is None else np.tile(np.asarray(REAs), (m, 1)).astype(np.float32)
    return Zs_, xyz, qs_, cLJs_, REAs_


def get_C612(i, j, FFparams):
    """c6 = 2 eps R^6, c12 = eps R^12 with R = r_i + r_j, eps = sqrt(e_i e_j) (common.py:851-857)."""
    Rij = FFparams[i][0] + FFparams[j][0]
    Eij = np.sqrt(FFparams[i][1] * FFparams[j][1])
    return 2 * Eij * (Rij**6), Eij * (Rij**12)


def getAtomsLJ(iZprobe, iZs, FFparams):
    """(c6, c12) of every atom against the probe (common.py:860-868); evaluated once per
    element with the scalar expressions of get_C612, so every value is the reference's."""
    iZs = np.asarray(iZs, dtype=np.int64).reshape(-1)
    if iZs.size == 0:
        return np.zeros((0, 2))
    uniq, inv = np.unique(iZs, return_inverse=True)
    table = np.array([get_C612(iZprobe - 1, int(z) - 1, FFparams) for z in uniq], dtype=np.float64)
    return table[inv.reshape(-1)]


def getAtomsREA(iZprobe, iZs, FFparams, alphaFac=-1.0):
    """(R, E, alpha) pair parameters (common.py:880-892), once per element."""
    iZs = np.asarray(iZs, dtype=np.int64).reshape(-1)
    REAs = np.zeros((iZs.size, 4))
    if iZs.size == 0:
        return REAs
    i = iZprobe - 1
    uniq, inv = np.unique(iZs, return_inverse=True)
    table = np.zeros((len(uniq), 3))
    for k, z in enumerate(uniq):
        j = int(z) - 1
        table[k, 0] = FFparams[i][0] + FFparams[j][0]
        table[k, 1] = np.sqrt(FFparams[i][1] * FFparams[j][1])
        table[k, 2] = FFparams[j][2] * alphaFac
    REAs[:, :3] = table[inv.reshape(-1)]
    return REAs


def REA2LJ(cREAs, cLJs=None):
    """common.py:871-877."""
    if cLJs is None:
        cLJs = np.zeros((len(cREAs), 2))
    R6 = cREAs[:, 0] ** 6
    cLJs[:, 0] = 2 * cREAs[:, 1] * R6
    cLJs[:, 1] = cREAs[:, 1] * (R6**2)
    return cLJs


def prepareScanGrids(scanMin=None, scanMax=None, scanStep=None, r0Probe=None, parameters=None):
    """Tip positions and the scan-output lattice (common.py:922-946).  Called like the
    reference with the parameters object (``prepareScanGrids(parameters)`` or
    ``prepareScanGrids(parameters=p)``: its scanMin, scanMax, scanStep, r0Probe), or with the
    four values."""
    if parameters is None and scanMax is None and scanMin is not None and not np.ndim(scanMin):
        parameters, scanMin = scanMin, None  # prepareScanGrids(parameters)
    if parameters is not None:
        g = (lambda k: parameters[k]) if isinstance(parameters, dict) else (lambda k: getattr(parameters, k))
        scanMin, scanMax, scanStep, r0Probe = g("scanMin"), g("scanMax"), g("scanStep"), g("r0Probe")
    xTips = np.arange(scanMin[0], scanMax[0] + 0.5 * scanStep[0], scanStep[0])
    yTips = np.arange(scanMin[1], scanMax[1] + 0.5 * scanStep[1], scanStep[1])
    zTips = np.arange(scanMin[2], scanMax[2] + 0.5 * scanStep[2], scanStep[2])
    lvecScan = np.array(
        [
            [scanMin[0] + r0Probe[0], scanMin[1] + r0Probe[1], scanMin[2] - r0Probe[2]],
            [scanMax[0] - scanMin[0], 0.0, 0.0],
            [0.0, scanMax[1] - scanMin[1], 0.0],
            [0.0, 0.0, scanMax[2] - scanMin[2]],
        ]
    )
    return xTips, yTips, zTips, lvecScan


def lvec2params(parameters, lvec):
    """The cell vectors of lvec [4, 3] into the parameters' gridA/B/C (common.py:949-952)."""
    parameters.gridA = np.array(lvec[1, :], dtype=np.float64)
    parameters.gridB = np.array(lvec[2, :], dtype=np.float64)
    parameters.gridC = np.array(lvec[3, :], dtype=np.float64)


def params2lvec(parameters):
    """lvec [4, 3] with origin 0 and the parameters' gridA/B/C (common.py:955-964)."""
    return np.array([[0.0, 0.0, 0.0], parameters.gridA, parameters.gridB, parameters.gridC], dtype=np.float64)


def genFFSampling(lvec, pixPerAngstrome=10):
    """Grid size for a lattice at a given density (common.py:967-977)."""
    return np.array([int(round(pixPerAngstrome * np.sqrt(np.dot(lvec[k], lvec[k])))) for k in (1, 2, 3)], np.int32)
