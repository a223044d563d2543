"""Generates the golden fixtures in tests/golden/ by running the reference ppafm package.

Run where the reference checkout exists (it is read only); its root is the first argument,
else $PPAFM_REFERENCE, else /root/reference:

    python tests/golden/make_golden.py [REFERENCE_ROOT]           # all fixtures
    python tests/golden/make_golden.py REFERENCE_ROOT extras      # xsf/, tilt.npz, params/ only

The script copies the reference's ``ppafm`` package to a temporary directory, compiles
its two C++ modules there from their own sources with g++ (ProbeParticle, GridUtils; the
same flags as oracle/Makefile), stubs the unused ``toml`` import, and calls the
reference's own functions on small seeded inputs.  Inputs and outputs are stored as
float64 .npz files; the tests compare the oracle and the GPU path against them.
"""

import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def setup_reference(ref_root):
    tmp = tempfile.mkdtemp(prefix="ppafm_golden_")
    pkg = os.path.join(tmp, "ppafm")
    shutil.copytree(os.path.join(ref_root, "ppafm"), pkg, ignore=shutil.ignore_patterns("*.so", "*.o", "__pycache__"))
    cpp = os.path.join(pkg, "cpp")
    for mod in ("ProbeParticle", "GridUtils"):
        src = os.path.join(cpp, mod + ".cpp")
        out = os.path.join(cpp, mod + "_lib.so")
        subprocess.run(["g++", "-fPIC", "-std=c++11", "-O2", "-fopenmp", "-ffp-contract=off", "-shared", "-I", cpp, src, "-o", out], check=True)
    with open(os.path.join(tmp, "toml.py"), "w") as f:
        f.write("def load(*a, **k):\n    raise RuntimeError('toml unavailable')\n\ndef dump(*a, **k):\n    raise RuntimeError('toml unavailable')\n")
    sys.path.insert(0, tmp)
    return tmp


DEFAULT_REFERENCE = os.environ.get("PPAFM_REFERENCE", "/root/reference")


def main(ref_root=DEFAULT_REFERENCE, only=None):
    tmp = setup_reference(ref_root)
    if only == "extras":
        try:
            make_xsf(tmp)
            make_tilt(tmp)
            make_params(ref_root)
            make_stages(tmp)
            make_helpers(tmp)
            make_cube(tmp)
        finally:
            shutil.rmtree(tmp, ignore_errors=True)
        return
    try:
        import ppafm.common as PPU
        import ppafm.core as core
        import ppafm.fieldFFT as fFFT
        import ppafm.HighLevel as HL
        import ppafm.io as pio

        rng = np.random.default_rng(20241203)
        # setFF_Fpointer registers a finalizer that clears the core's global grid pointer
        # when the array dies (core.py:59-61); keep every grid alive so that rebinding a
        # name does not clear the pointer of the grid registered next.
        keep = []

        # ---- Δf kernels and Fz -> Δf (common.py:333-430)
        cases = [(0.1, 0.1), (1.0, 0.2), (1.0, 0.1), (0.5, 0.1), (2.0, 0.1), (1.0, 0.05), (0.3, 0.1), (1.7, 0.13)]
        dfw = {f"w_{i}": PPU.get_df_weight(a, dz=d) for i, (a, d) in enumerate(cases)}
        scases = [(5, 0.2), (10, 0.1), (2, 0.1), (1, 0.1), (7, 0.05)]
        sw = {f"s_{i}": PPU.get_simple_df_weight(n=n, dz=d) for i, (n, d) in enumerate(scases)}
        Fz = rng.normal(size=(4, 3, 30)) * 0.05
        df1 = PPU.Fz2df(Fz, dz=0.1, k0=1800.0, f0=30000.0, amplitude=1.0)
        df2 = PPU.Fz2df(Fz, dz=0.1, k0=1800.0, f0=30300.0, amplitude=0.5)
        np.savez_compressed(os.path.join(HERE, "df.npz"), cases=np.array(cases), scases=np.array(scases), Fz=Fz, df1=df1, df2=df2, **dfw, **sw)

        # ---- atoms: species, PBC images, LJ mixing, scan grids
        FFparams = PPU.loadSpecies()
        species = np.array([(f[0], f[1], f[2], f[3]) for f in FFparams])
        Zs = np.array([6, 6, 8, 1, 7, 9, 17, 1, 6, 8], dtype=np.int32)
        Rs = np.column_stack([rng.uniform(1, 7, 10), rng.uniform(1, 7, 10), rng.uniform(-0.4, 0.4, 10)])
        Qs = rng.uniform(-0.3, 0.3, 10)
        Qs -= Qs.mean()
        lvec = np.array([[0.0, 0.0, 0.0], [8.0, 0.0, 0.0], [0.7, 7.5, 0.0], [0.0, 0.0, 8.5]])

        class P:  # the attributes PBCAtoms reads from a parameters object
            nPBC = [1, 1, 1]

        iZ9, R9, Q9 = PPU.PBCAtoms(Zs, Rs, Qs, avec=lvec[1], bvec=lvec[2], parameters=P())
        cLJ9 = PPU.getAtomsLJ(8, iZ9, FFparams)
        REAs = PPU.getAtomsREA(8, Zs, FFparams, alphaFac=-1.0)
        cLJ_rea = PPU.REA2LJ(REAs)
        Z3, xyz3, q3, c3, rea3 = PPU.PBCAtoms3D_np(Zs, Rs, Qs, cLJ_rea, REAs, lvec[1:], npbc=[1, 1, 0])

        class S:
            scanMin = [0.0, 0.0, 5.0]
            scanMax = [7.5, 6.0, 7.9]
            scanStep = [0.25, 0.5, 0.1]
            r0Probe = [0.0, 0.0, 4.0]

        xT, yT, zT, lvecScan = PPU.prepareScanGrids(parameters=S())
        np.savez_compressed(os.path.join(HERE, "atoms.npz"), species=species, Zs=Zs, Rs=Rs, Qs=Qs, lvec=lvec, iZ9=iZ9, R9=R9, Q9=Q9, cLJ9=cLJ9, REAs=REAs, cLJ_rea=cLJ_rea, Z3=Z3, xyz3=xyz3, q3=q3, c3=c3, xT=xT, yT=yT, zT=zT, lvecScan=lvecScan)

        # ---- force-field grids (ProbeParticle.cpp:508-554) on a skewed cell
        n = np.array([16, 14, 12], dtype=np.int32)
        Rs0 = HL.shift_positions(R9, -lvec[0])
        out = {}
        FF, V = HL.setFF(None, True, n=n, lvec=lvec)
        keep += [FF, V]
        core.getLennardJonesFF(Rs0, cLJ9)
        out["F_lj"], out["E_lj"] = FF.copy(), V.copy()
        for kind in (0, 1, 2):
            FF, V = HL.setFF(None, True, n=n, lvec=lvec)
            keep += [FF, V]
            core.getCoulombFF(Rs0, Q9 * PPU.CoulombConst, kind=kind)
            out[f"F_el{kind}"], out[f"E_el{kind}"] = FF.copy(), V.copy()
        Fcl = out["F_lj"].copy()
        pio.limit_vec_field(Fcl, Fmax=0.5)
        np.savez_compressed(os.path.join(HERE, "ff.npz"), n=n, lvec=lvec, Rs0=Rs0, cLJs=cLJ9, kqq=Q9 * PPU.CoulombConst, F_clamped=Fcl, **out)

        # ---- relaxed scan (HighLevel.py:104-184, ProbeParticle.cpp:633-701)
        # orthogonal 10 A cell at 0.2 A; tip heights over a planar molecule
        lv = np.array([[0.0, 0.0, 0.0], [10.0, 0.0, 0.0], [0.0, 10.0, 0.0], [0.0, 0.0, 10.0]])
        nr = np.array([50, 50, 50], dtype=np.int32)
        Zm = np.array([6, 6, 6, 6, 8, 1, 1, 7], dtype=np.int32)
        ang = np.linspace(0, 2 * np.pi, 8, endpoint=False) + rng.uniform(-0.2, 0.2, 8)
        Rm = np.column_stack([5 + 1.6 * np.cos(ang), 5 + 1.6 * np.sin(ang), np.zeros(8)])
        Qm = rng.uniform(-0.25, 0.25, 8)
        Qm -= Qm.mean()
        iZr, Rr, Qr = PPU.PBCAtoms(Zm, Rm, Qm, avec=lv[1], bvec=lv[2], parameters=P())
        cLJr = PPU.getAtomsLJ(8, iZr, FFparams)
        FFLJ, _ = HL.setFF(None, False, n=nr, lvec=lv)
        keep.append(FFLJ)
        core.getLennardJonesFF(Rr, cLJr)
        pio.limit_vec_field(FFLJ, Fmax=10.0)
        FFLJ = FFLJ.copy()
        FFel, _ = HL.setFF(None, False, n=nr, lvec=lv)
        keep.append(FFel)
        core.getCoulombFF(Rr, Qr * PPU.CoulombConst, kind=0)
        pio.limit_vec_field(FFel, Fmax=10.0)
        FFel = FFel.copy()

        class R:
            charge = -0.05
            stiffness = [-1.0, -1.0, -1.0]
            klat = 0.25
            krad = 20.0
            r0Probe = [0.0, 0.0, 4.0]
            scanMin = [2.0, 2.5, 7.0]
            scanMax = [7.8, 7.5, 9.9]
            scanStep = [0.2, 0.25, 0.1]
            tiltedScan = False
            Apauli = 1.0
            Vbias = 0.0

        core.lib.setRelax(300, 1e-8, 0.5, 0.1)  # core.setRelax is broken (core.py:97-98)
        core.lib.setFIRE(1.1, 0.5, 0.99)
        fzs, PPpos, _, lvecScanR = HL.perform_relaxation(lv, FFLJ, FFel=FFel, parameters=R())
        # iteration counts of a few strokes (relaxTipStroke returns the stroke's sum)
        FF = FFLJ + FFel * R.charge
        keep.append(FF)
        HL.setFF(FF, lvec=lv)
        core.setTip(kSpring=np.array((0.25, 0.25, 0.0)) / -PPU.eVA_Nm, kRadial=20.0 / -PPU.eVA_Nm, parameters=R())
        xT, yT, zT, _ = PPU.prepareScanGrids(parameters=R())
        picks = [(0, 0), (5, 7), (14, 3), (29, 20)]
        itsum = []
        for ix, iy in picks:
            rT = np.zeros((len(zT), 3))
            rT[:, 0] = xT[ix]
            rT[:, 1] = yT[iy]
            rT[:, 2] = zT[::-1]
            itsum.append(core.relaxTipStroke(rT, np.zeros_like(rT), np.zeros_like(rT)))
        df = PPU.Fz2df(fzs, dz=0.1, k0=1800.0, f0=30000.0, amplitude=1.0)
        np.savez_compressed(os.path.join(HERE, "relax.npz"), n=nr, lvec=lv, Zm=Zm, Rm=Rm, Qm=Qm, charge=R.charge, klat=R.klat, krad=R.krad, r0Probe=R.r0Probe, scanMin=R.scanMin, scanMax=R.scanMax, scanStep=R.scanStep, fzs=fzs, PPpos=PPpos, lvecScan=lvecScanR, picks=np.array(picks), itsum=np.array(itsum), df=df)

        # ---- FFT route (fieldFFT.py:268-319)
        fft = {}
        for tag, dims, lvf in (
            ("ortho", (24, 20, 16), np.array([[0.0, 0, 0], [6.0, 0, 0], [0, 5.0, 0], [0, 0, 4.0]])),
            ("skew_odd", (15, 16, 17), np.array([[0.0, 0, 0], [6.0, 0, 0], [1.2, 5.5, 0], [0, 0.4, 4.3]])),
        ):
            V = rng.normal(size=dims)
            rho = np.abs(rng.normal(size=dims))
            fx, fy, fz, e = fFFT.potential2forces_mem(V.copy(), lvf, np.array(dims), rho=rho.copy(), doForce=True, doPot=True, deleteV=False)
            fft.update({f"{tag}_V": V, f"{tag}_rho": rho, f"{tag}_lvec": lvf, f"{tag}_Fx": fx, f"{tag}_Fy": fy, f"{tag}_Fz": fz, f"{tag}_E": e})
            cwd = os.getcwd()
            os.chdir(tmp)  # potential2forces_mem writes rhoTip.xsf when it builds the tip density
            try:
                fx2, fy2, fz2, e2 = fFFT.potential2forces_mem(V.copy(), lvf, np.array(dims), sigma=0.7, multipole={"s": 1.0, "dz2": -0.3}, doForce=True, doPot=True, deleteV=False)
            finally:
                os.chdir(cwd)
            fft.update({f"{tag}_mFx": fx2, f"{tag}_mFy": fy2, f"{tag}_mFz": fz2, f"{tag}_mE": e2})
        np.savez_compressed(os.path.join(HERE, "fft.npz"), **fft)

        # ---- clamp (io.py:766-778)
        G = rng.normal(size=(5, 4, 3, 3)) * 20
        Gc = G.copy()
        pio.limit_vec_field(Gc, Fmax=10.0)
        np.savez_compressed(os.path.join(HERE, "clamp.npz"), G=G, Gc=Gc)
        print("golden fixtures written to", HERE)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


def make_xsf(tmp):
    """Grid files written by the reference's io (io.py:575-598, 781-842): an XSF scalar field,
    an XSF vector field (three files) and the npz forms, under tests/golden/xsf/."""
    import ppafm.io as pio

    out = os.path.join(HERE, "xsf")
    os.makedirs(out, exist_ok=True)
    rng = np.random.default_rng(777)
    lvec = np.array([[0.5, -0.25, 1.0], [6.0, 0.0, 0.0], [1.5, 5.0, 0.0], [0.0, 0.0, 4.0]])
    S = rng.normal(size=(5, 4, 3))
    V = rng.normal(size=(5, 4, 3, 3))
    pio.saveXSFData(os.path.join(out, "scal.xsf"), S, lvec)
    pio.save_vec_field(os.path.join(out, "vec"), V, lvec, data_format="xsf")
    pio.save_vec_field(os.path.join(out, "vec"), V, lvec, data_format="npy")
    pio.save_scal_field(os.path.join(out, "scal"), S, lvec, data_format="npy")
    pio.saveXSFData(os.path.join(out, "ortho.xsf"), S[:, :, :2], dd=[0.1, 0.2, 0.3])
    np.savez(os.path.join(out, "inputs.npz"), S=S, V=V, lvec=lvec)
    print("xsf fixtures written to", out)


def make_tilt(tmp):
    """Fz2df_tilt of a tilted scan's force vectors (common.py:433-445) -> tests/golden/tilt.npz."""
    import ppafm.common as PPU

    rng = np.random.default_rng(4242)
    F = rng.normal(size=(4, 3, 30, 3)) * 0.05
    cases = {}
    for i, (d, amp) in enumerate((((0.02, -0.01, 0.1), 1.0), ((0.0, 0.0, 0.1), 0.5), ((0.05, 0.05, 0.08), 1.3))):
        cases[f"d_{i}"] = np.array(d)
        cases[f"amp_{i}"] = np.array(amp)
        cases[f"df_{i}"] = PPU.Fz2df_tilt(F, d, k0=1800.0, f0=30300.0, amplitude=amp)
    np.savez_compressed(os.path.join(HERE, "tilt.npz"), F=F, **cases)
    print("tilt fixture written")


def make_params(ref_root):
    """PpafmParameters (common.py:26-160) of the reference's own test file
    (tests/data/test_params.ini) and its defaults, parsed by the reference -> tests/golden/params/."""
    import json

    import ppafm.common as PPU

    out = os.path.join(HERE, "params")
    os.makedirs(out, exist_ok=True)
    shutil.copyfile(os.path.join(ref_root, "tests", "data", "test_params.ini"), os.path.join(out, "test_params.ini"))
    parsed = PPU.PpafmParameters.from_file(os.path.join(out, "test_params.ini")).model_dump()
    default = PPU.PpafmParameters().model_dump()
    with open(os.path.join(out, "parsed.json"), "w") as f:
        json.dump({"parsed": parsed, "default": default}, f, indent=1)
    sp = PPU.loadSpecies()  # the reference's default species table
    np.savez(os.path.join(out, "species.npz"), rmin=sp["rmin"], epsilon=sp["epsilon"], alpha=sp["alpha"], atom=sp["atom"], symbol=sp["symbol"])
    print("params fixtures written")


def make_stages(tmp):
    """The file-based force-field stages (HighLevel.computeLJ, computeELFF_pointCharge,
    io.loadGeometry) of the reference on small seeded inputs -> tests/golden/stages/: an xyz
    molecule with charges, a POSCAR and an FHI-aims geometry.in, the parameters, the grids the
    stages return and what loadGeometry parses."""
    import json

    import ppafm.common as PPU
    import ppafm.HighLevel as HL
    import ppafm.io as pio

    out = os.path.join(HERE, "stages")
    os.makedirs(out, exist_ok=True)
    rng = np.random.default_rng(31)
    n = 14
    xyz = np.column_stack([rng.uniform(2.5, 6.5, n), rng.uniform(2.5, 6.5, n), rng.uniform(-0.3, 0.3, n)])
    Zs = rng.choice([1, 6, 7, 8], n)
    q = rng.uniform(-0.3, 0.3, n)
    q -= q.mean()
    sym = {1: "H", 6: "C", 7: "N", 8: "O"}
    with open(os.path.join(out, "mol.xyz"), "w") as f:
        f.write(f"{n}\nseeded molecule\n")
        for i in range(n):
            f.write(f"{sym[int(Zs[i])]} {xyz[i,0]:.6f} {xyz[i,1]:.6f} {xyz[i,2]:.6f} {q[i]:.6f}\n")
    ini = "probeType 8\ncharge -0.05\ngridA 9.0 0.0 0.0\ngridB 0.0 9.6 0.0\ngridC 0.0 0.0 8.0\ngridO 0.0 0.0 -3.0\ngridN 24 26 20\nnPBC 1 1 0\nscanMin 1.0 1.0 5.0\nscanMax 8.0 8.0 7.0\n"
    with open(os.path.join(out, "params.ini"), "w") as f:
        f.write(ini)
    cwd = os.getcwd()
    os.chdir(tmp)
    try:
        p = PPU.PpafmParameters.from_file(os.path.join(out, "params.ini"))
        FF, V, nDim, lvec = HL.computeLJ(os.path.join(out, "mol.xyz"), None, computeVpot=True, parameters=p)
        FF, V = FF.copy(), V.copy()
        p = PPU.PpafmParameters.from_file(os.path.join(out, "params.ini"))
        FE, VE, _, _ = HL.computeELFF_pointCharge(os.path.join(out, "mol.xyz"), tip="dz2", computeVpot=True, parameters=p)
        FE, VE = FE.copy(), VE.copy()
    finally:
        os.chdir(cwd)
    f32 = np.float32  # the GPU grids are float32; float32 copies keep the fixture small
    np.savez_compressed(os.path.join(out, "grids.npz"), F_lj=FF.astype(f32), E_lj=V.astype(f32), F_el=FE.astype(f32), E_el=VE.astype(f32), nDim=np.array(nDim), lvec=np.array(lvec))
    # geometry files: POSCAR (direct coordinates) and geometry.in, parsed by the reference
    with open(os.path.join(out, "POSCAR"), "w") as f:
        f.write("seeded cell\n1.5\n4.0 0.0 0.0\n0.5 5.0 0.0\n0.0 0.0 6.0\nC O H\n2 1 1\nDirect\n")
        for r in rng.uniform(0, 1, (4, 3)):
            f.write(f"{r[0]:.6f} {r[1]:.6f} {r[2]:.6f}\n")
    with open(os.path.join(out, "geometry.in"), "w") as f:
        f.write("# seeded\nlattice_vector 7.0 0.0 0.0\nlattice_vector 0.0 8.0 0.0\nlattice_vector 0.0 0.0 9.0\n")
        f.write("atom 1.0 2.0 3.0 C\natom 2.5 2.0 3.0 O\natom_frac 0.5 0.25 0.1 N\n")
    parsed = {}
    for name in ("POSCAR", "geometry.in", "mol.xyz"):
        p = PPU.PpafmParameters.from_file(os.path.join(out, "params.ini"))
        atoms, nD, lv = pio.loadGeometry(os.path.join(out, name), format="poscar" if name == "POSCAR" else None, parameters=p)
        parsed[name] = {"atoms": [[float(x) for x in a] for a in atoms], "nDim": [int(x) for x in nD], "lvec": np.asarray(lv, dtype=np.float64).tolist(), "PBC": bool(p.PBC), "gridN": [int(x) for x in p.gridN]}
    with open(os.path.join(out, "geometry.json"), "w") as f:
        json.dump(parsed, f, indent=1)
    print("stage fixtures written")


def make_helpers(tmp):
    """Host helpers of ppafm/common.py (rotations, sphere frames, image replication, wrapping,
    pair parameters) on seeded inputs -> tests/golden/helpers.npz."""
    import ppafm.common as PPU

    rng = np.random.default_rng(55)
    n = 7
    Zs = rng.choice([1, 6, 7, 8, 17], n)
    Rs = rng.uniform(-3, 3, (n, 3))
    Qs = rng.uniform(-0.3, 0.3, n)
    FF = PPU.loadSpecies()
    cLJs = PPU.getAtomsLJ(8, Zs, FF)
    lvec3 = np.array([[5.0, 0.0, 0.0], [1.0, 6.0, 0.0], [0.0, 0.5, 7.0]])
    axis = np.array([0.3, -0.4, 0.8])
    thetas = np.array([0.1, 1.2, -2.5])
    rots = PPU.genRotations(axis, thetas)
    out = dict(Zs=Zs, Rs=Rs, Qs=Qs, cLJs=cLJs, lvec3=lvec3, axis=axis, thetas=thetas)
    out["rot"] = PPU.rotation_matrix(axis, 0.7)
    out["rots"] = rots
    out["sphere"] = PPU.sphereTangentSpace(11)
    hdir = np.array([0.1, 0.2, 0.97])
    out["hdir"] = hdir
    i, h = PPU.maxAlongDir(Rs, hdir)
    i2, h2, e2 = PPU.maxAlongDirEntropy(Rs, hdir, beta=0.7)
    out["maxdir"] = np.array([i, h, i2, h2, e2])
    z, r, q, c = PPU.multRot(Zs, Rs, Qs, cLJs, rots, cog=(0.5, -0.5, 0.2))
    out.update(mr_Z=z, mr_R=r, mr_Q=q, mr_c=c)
    z, r, q, c = PPU.PBCAtoms3D(Zs, Rs, Qs, cLJs, lvec3, npbc=[1, 1, 0])
    out.update(p3_Z=z, p3_R=r, p3_Q=q, p3_c=c)
    W = Rs.copy()
    PPU.wrapAtomsCell(W, 0.25, -0.1, lvec3[0], lvec3[1])
    out["wrapped"] = W
    out["sREA"] = PPU.getSampleAtomsREA(Zs, FF)
    out["RE"] = PPU.getAtomsRE(8, Zs, FF)
    np.savez(os.path.join(HERE, "helpers.npz"), **out)
    print("helper fixtures written")


def make_cube(tmp):
    """A small Gaussian cube file (skewed voxels, three atoms) and what the reference's readers
    make of it (io.loadCUBE in both orders, loadAtomsCUBE, loadCellCUBE, loadNCUBE, loadGeometry)
    -> tests/golden/cube/."""
    import ppafm.common as PPU
    import ppafm.io as pio

    out = os.path.join(HERE, "cube")
    os.makedirs(out, exist_ok=True)
    rng = np.random.default_rng(77)
    n = (5, 4, 6)
    vox = np.array([[0.4, 0.0, 0.0], [0.1, 0.45, 0.0], [0.0, 0.05, 0.5]])
    data = rng.normal(size=n)
    path = os.path.join(out, "dens.cube")
    with open(path, "w") as f:
        f.write("seeded cube\nsecond comment line\n")
        f.write("%5d %12.6f %12.6f %12.6f\n" % (3, -1.0, 0.5, 2.0))
        for k in range(3):
            f.write("%5d %12.6f %12.6f %12.6f\n" % (n[k], *vox[k]))
        for Z, p in ((6, (1.0, 1.5, 2.0)), (8, (2.2, 0.3, -0.4)), (1, (0.0, 0.0, 0.0))):
            f.write("%5d %12.6f %12.6f %12.6f %12.6f\n" % (Z, 0.0, *p))
        vals = data.ravel()
        for i in range(0, vals.size, 6):
            f.write(" ".join("%13.5e" % v for v in vals[i : i + 6]) + "\n")
    F, lvec, nD, _ = pio.loadCUBE(path)
    Fx, _, nDx, _ = pio.loadCUBE(path, xyz_order=True)
    atoms = pio.loadAtomsCUBE(path)
    p = PPU.PpafmParameters()
    g_atoms, g_n, g_lvec = pio.loadGeometry(path, parameters=p)
    np.savez(os.path.join(out, "parsed.npz"), F=F, lvec=lvec, nD=np.array(nD), Fx=Fx, nDx=np.array(nDx), atoms=np.array(atoms, dtype=np.float64),
             cell=np.array(pio.loadCellCUBE(path)), ncube=np.array(pio.loadNCUBE(path)), g_atoms=np.array(g_atoms, dtype=np.float64), g_n=np.array(g_n), g_lvec=np.array(g_lvec))
    print("cube fixtures written")


if __name__ == "__main__":
    main(*sys.argv[1:])
