"""Host-side logic of the product (no GPU): Δf weights, species, atoms, scan grids, atom
packing, workloads, and that libppgpu.so exports every symbol include/ppgpu.h declares."""

import os
import re

import numpy as np
import pytest

from ppafm_gb300 import common, species, workloads

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_df_weights_match_reference_vectors(golden):
    assert np.allclose(common.get_df_weight(0.1), np.array([-5.0, 5.0]))
    assert np.allclose(common.get_df_weight(1.0, dz=0.2), np.array([-0.35594622, -0.22193265, -0.05447093, 0.05447093, 0.22193265, 0.35594622]))
    assert np.allclose(common.get_simple_df_weight(n=5, dz=0.2), np.array([-0.31362841, -0.37274317, 0, 0.37274317, 0.31362841]))
    g = golden("df")
    for i, (a, d) in enumerate(g["cases"]):
        assert np.array_equal(common.get_df_weight(a, dz=d), g[f"w_{i}"])
    for i, (n, d) in enumerate(g["scases"]):
        assert np.array_equal(common.get_simple_df_weight(n=int(n), dz=d), g[f"s_{i}"])


def test_species_table_matches_reference(golden):
    g = golden("atoms")
    t = species.loadSpecies()
    ref = g["species"]
    for row in t:
        z = int(row[3])
        r = ref[ref[:, 3] == z][0]
        assert (row[0], row[1], row[2]) == (r[0], r[1], r[2])
    d = species.getFFdict(t)
    assert species.atom2iZ("O", d) == 8 and species.atom2iZ(79, d) == 79
    with pytest.raises(ValueError):
        species.atom2iZ("Xx", d)


def test_atoms_and_scan_grids(golden):
    g = golden("atoms")
    FFp = species.loadSpecies()
    iZ, R, Q = common.PBCAtoms(g["Zs"], g["Rs"], g["Qs"], g["lvec"][1], g["lvec"][2])
    assert np.array_equal(iZ, g["iZ9"]) and np.array_equal(R, g["R9"]) and np.array_equal(Q, g["Q9"])
    assert np.array_equal(common.getAtomsLJ(8, iZ, FFp), g["cLJ9"])
    REAs = common.getAtomsREA(8, g["Zs"], FFp)
    assert np.array_equal(REAs, g["REAs"])
    assert np.array_equal(common.REA2LJ(REAs), g["cLJ_rea"])
    Z3, xyz3, q3, c3, _ = common.PBCAtoms3D_np(g["Zs"], g["Rs"], g["Qs"], g["cLJ_rea"], REAs, g["lvec"][1:], npbc=(1, 1, 0))
    assert np.array_equal(Z3, g["Z3"]) and np.array_equal(xyz3, g["xyz3"]) and np.array_equal(q3, g["q3"]) and np.array_equal(c3, g["c3"])
    xT, yT, zT, lv = common.prepareScanGrids([0.0, 0.0, 5.0], [7.5, 6.0, 7.9], [0.25, 0.5, 0.1], [0.0, 0.0, 4.0])
    for a, b in ((xT, "xT"), (yT, "yT"), (zT, "zT"), (lv, "lvecScan")):
        assert np.array_equal(a, g[b])


def test_pack_atoms_layout():
    """ppgpu_pack_atoms is host code: records, charged-first order, hi/lo split."""
    import ctypes

    from ppafm_gb300 import _lib

    L = _lib.load()
    rng = np.random.default_rng(3)
    n = 9
    R = rng.uniform(-30, 30, (n, 3))
    cLJ = rng.uniform(1, 100, (n, 2))
    kqq = np.array([0.0, 1.5, 0.0, -2.0, 0.0, 0.0, 0.3, 0.0, 0.0])
    out = np.zeros((n, 12), np.float32)
    nch = np.zeros(1, np.int32)
    _lib.check(L.ppgpu_pack_atoms(n, _lib.dptr(R), _lib.dptr(cLJ), _lib.dptr(kqq), out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), _lib.iptr(nch)))
    assert nch[0] == 3
    order = [1, 3, 6, 0, 2, 4, 5, 7, 8]
    for r, i in enumerate(order):
        hi = -out[r, [0, 1, 4]].astype(np.float64)
        lo = -out[r, [2, 3, 5]].astype(np.float64)
        assert np.allclose(hi + lo, R[i], rtol=0, atol=1e-12)
        assert out[r, 10] == np.float32(kqq[i])
        assert out[r, 8] == np.float32(-cLJ[i, 0]) and out[r, 9] == np.float32(cLJ[i, 1])
        assert out[r, 6] == np.float32(-6 * cLJ[i, 0]) and out[r, 7] == np.float32(12 * cLJ[i, 1])
    # argument errors are reported, not crashed on
    assert L.ppgpu_pack_atoms(-1, None, None, None, None, None) == _lib.PPGPU_ERR_ARG
    assert "bad arguments" in _lib.last_error()


def _header_functions():
    txt = open(os.path.join(ROOT, "include", "ppgpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\([^;{]*\)\s*;", txt)
    return sorted(set(n for n in names if n not in ("if", "while", "return")))


def test_library_exports_every_declared_symbol():
    from ppafm_gb300 import _lib, build

    build.build()
    import ctypes

    L = ctypes.CDLL(_lib.LIB_PATH)
    decl = _header_functions()
    assert len(decl) >= 30
    for name in decl:
        assert hasattr(L, name), name
    assert set(decl) == set(_lib.SIGNATURES), set(decl) ^ set(_lib.SIGNATURES)
    _lib.load()  # binds argtypes for every symbol


def test_workload_shapes():
    w = workloads.small_molecule(0)
    assert len(w["Zs"]) == 38 and tuple(w["gridN"]) == (200, 200, 200)
    assert sorted(np.bincount(w["Zs"])[[1, 6, 8]]) == [6, 8, 24]
    assert abs(w["Qs"].sum()) < 1e-12 and np.abs(w["Qs"]).max() <= 0.4  # U(-0.3,0.3) shifted to zero sum
    xT, yT, zT, _ = common.prepareScanGrids(w["scanMin"], w["scanMax"], w["scanStep"], w["r0Probe"])
    assert (len(xT), len(yT), len(zT)) == (160, 160, 30)
    s = workloads.slab_molecule(0, scale=0.05)
    assert len(s["Zs"]) == 2060 and (s["Qs"][:2000] == 0).all() and abs(s["Qs"].sum()) < 1e-9
    d = np.linalg.norm(s["Rs"][:2000, None, :2] - s["Rs"][None, :2000, :2], axis=-1)
    same_layer = np.abs(s["Rs"][:2000, None, 2] - s["Rs"][None, :2000, 2]) < 1e-9
    np.fill_diagonal(d, 1e9)
    assert d[same_layer].min() > 2.5
    full = workloads.slab_molecule(0)
    xT, yT, zT, _ = common.prepareScanGrids(full["scanMin"], full["scanMax"], full["scanStep"], full["r0Probe"])
    assert (len(xT), len(yT), len(zT)) == (512, 512, 40) and tuple(full["gridN"]) == (800, 800, 500)
    b = workloads.molecule_batch(0, nmol=16)
    assert all(10 <= len(m["Zs"]) <= 60 for m in b)
    assert all(96 <= n <= 192 for m in b for n in m["gridN"])
