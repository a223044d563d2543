"""Known answers for the AFMulator kernels (no OpenCL runtime here, so their parity with
relax.cl / FF.cl is pinned by cases whose answer follows from the physics, not from a
restatement of the kernels).

relax_afm_kernel (relaxStrokesTilted + update_FIRE + tipForce, relax.cl:37-41, 105-126,
391-464), called through the C ABI:
  * a linear force field -K (r - c) (reproduced exactly by trilinear interpolation) plus
    the lateral tip springs: the fixed point of every height is analytic, FIRE must stop
    within |F|/k of it (|F| < 1e-4 eV/A), with the warm start carried over the heights;
  * a uniform field plus the radial and lateral springs: the equilibrium solved by Newton's
    method in float64;
  * the 128-iteration cap: a constant field and no springs never converges; from rest the
    probe moves by n(n+1)/2 F dt^2 in n moves with v parallel to F, so after the cap it is at
    pos0 + 8256 F dt^2, every height reports 128 iterations, the next height starts there
    moved by the tip step, and the z convolution is Fz times the sum of the weights;
  * a zero field and no springs: F2SAFE keeps the mixing term finite (0/(0 + 1e-8)), the
    first evaluation converges, nothing moves.
evalLJC_QZs_noPos (FF.cl:366-423): the force field of a single charged atom against the
negative gradient of its pair energies (LJ c12/r^12 - c6/r^6 and Coulomb k q Q_k /|p + QZ_k z
- R| with R2SAFE added to r^2), taken by central differences in float64."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EVA_NM = 16.0217662
NPARAM = 28


def _afm_prm(dt=0.5, damp=0.1, stiff=(0.0, 0.0, 0.0, 0.0), dpos0=(0.0, 0.0, -4.0, 4.0), zstep=0.1, surf=0.0):
    """prm_afm of ppgpu_relax_afm: relax params, stiffness (already over -eVA_Nm), dpos0, tip
    rows (identity rotation, C[3] = -zstep: the tip moves down by zstep per height), surfFF."""
    p = np.zeros(NPARAM)
    p[0:4] = [dt, damp, 0.0, 0.0]
    p[4:8] = stiff
    p[8:12] = dpos0
    p[12:24] = [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, -zstep]
    p[24] = surf
    return p


def _grid(field, n=(64, 64, 64), L=16.0):
    """float4 grid [n0][n1][n2] of field(r) -> (F [..., 3], E) at the nodes r = i L / n."""
    import torch

    ax = [np.arange(k) * (L / k) for k in n]
    X, Y, Z = np.meshgrid(*ax, indexing="ij")
    r = np.stack([X, Y, Z], axis=-1)
    F, E = field(r)
    FE = np.concatenate([F, E[..., None]], axis=-1).astype(np.float32)
    return torch.from_numpy(FE).cuda().contiguous(), np.array(n, np.int32), np.eye(3) * L


def _run(FE, n, cell, prm, points, nz, W=None):
    """relax_afm_kernel through the C ABI; returns FEs, paths [npix, nz, 4], iters [npix, nz], X."""
    import torch

    from ppafm_gb300 import _lib

    L = _lib.lib()
    npix = len(points)
    pts = torch.from_numpy(np.ascontiguousarray(points, dtype=np.float32)).cuda()
    FEs = torch.empty((npix, nz, 4), dtype=torch.float32, device="cuda")
    paths = torch.empty_like(FEs)
    iters = torch.empty((npix, nz), dtype=torch.int32, device="cuda")
    nw = 0 if W is None else len(W)
    X = torch.empty((npix, nz - nw + 1), dtype=torch.float32, device="cuda") if W is not None else None
    inv_cell = np.ascontiguousarray(np.linalg.inv(cell).T, dtype=np.float64)
    Wd = None if W is None else np.ascontiguousarray(W, dtype=np.float64)
    _lib.check(L.ppgpu_relax_afm(_lib.tptr(FE), _lib.iptr(n), _lib.dptr(inv_cell), _lib.dptr(np.ascontiguousarray(prm)), npix, _lib.tptr(pts), nz, _lib.tptr(FEs), _lib.tptr(paths), _lib.tptr(iters), nw, _lib.dptr(Wd), _lib.tptr(X), None, _lib.stream_handle()))
    _lib.check(L.ppgpu_device_status(_lib.stream_handle()))
    return FEs.cpu().numpy(), paths.cpu().numpy(), iters.cpu().numpy(), (None if X is None else X.cpu().numpy())


def _tips(nx=6, ny=5, x0=6.0, y0=6.5, z=12.0, step=0.6):
    xs, ys = np.meshgrid(x0 + step * np.arange(nx), y0 + step * np.arange(ny), indexing="ij")
    return np.column_stack([xs.ravel(), ys.ravel(), np.full(xs.size, z), np.zeros(xs.size)])


def test_afm_relax_linear_field_fixed_point(gpulib):
    K = np.array([0.3, 0.2, 0.6])  # eV/A^2
    c = np.array([8.0, 7.5, 8.0])
    ks = 0.05  # lateral and vertical tip springs, eV/A^2 (stiffness -ks)
    d0 = np.array([0.1, -0.2, -3.0])
    FE, n, cell = _grid(lambda r: (-(r - c) * K, -0.5 * ((r - c) ** 2 * K).sum(-1)))
    prm = _afm_prm(stiff=(-ks, -ks, -ks, 0.0), dpos0=(*d0, 3.0))
    pts = _tips()
    nz, zstep = 6, 0.1
    FEs, paths, iters, _ = _run(FE, n, cell, prm, pts, nz)
    assert (iters < 128).all() and (iters >= 0).all()
    for iz in range(nz):
        tip = pts[:, :3] - np.array([0, 0, zstep * iz])
        fixed = (K * c + ks * (tip + d0)) / (K + ks)  # -K (r - c) - ks (r - tip - d0) = 0
        # the recorded force is the grid's at the point where |F| < 1e-4 eV/A was seen (before
        # the last move), so that point is -FEs/K + c: each component within 1e-4/(K + ks) of
        # the fixed point (plus the float32 rounding of the grid values)
        seen = c - FEs[:, iz, :3] / K
        err = np.abs(seen - fixed)
        assert (err <= 1e-4 / (K + ks) + 1e-5).all(), (iz, err.max(0))
        # the reported position is after that last move, a small one near the fixed point
        assert np.linalg.norm(paths[:, iz, :3] - seen, axis=-1).max() < 1e-3


def test_afm_relax_radial_spring_uniform_field(gpulib):
    F0 = np.array([0.05, -0.03, 0.4])
    kl, kr, l0 = 0.5, 30.0 / EVA_NM, 4.0
    d0 = np.array([0.0, 0.0, -l0])
    FE, n, cell = _grid(lambda r: (np.broadcast_to(F0, r.shape).copy(), np.zeros(r.shape[:-1])))
    prm = _afm_prm(stiff=(-kl, -kl, 0.0, -kr), dpos0=(*d0, l0))
    pts = _tips(nx=3, ny=3)
    FEs, paths, iters, _ = _run(FE, n, cell, prm, pts, 3)

    def force(dq):  # F0 + tipForce at displacement dq = pos - tip
        r = np.linalg.norm(dq)
        return F0 + (dq - d0) * np.array([-kl, -kl, 0.0]) + dq * (-kr) * (r - l0) / r

    dq = d0.copy()
    for _ in range(50):  # Newton with a central-difference Jacobian, float64
        J = np.column_stack([(force(dq + h) - force(dq - h)) / 2e-6 for h in np.eye(3) * 1e-6])
        dq = dq - np.linalg.solve(J, force(dq))
    assert np.abs(force(dq)).max() < 1e-12
    kmin = np.abs(np.linalg.eigvals(J)).min()
    for iz in range(3):
        tip = pts[:, :3] - np.array([0, 0, 0.1 * iz])
        err = np.linalg.norm(paths[:, iz, :3] - (tip + dq), axis=-1)
        # within |F|/k_min of the equilibrium where |F| < 1e-4 eV/A was seen, plus the last move
        assert (err <= 1e-4 / kmin + 1e-4).all(), (iz, err.max(), 1e-4 / kmin)
    assert (iters < 128).all()


def test_afm_relax_iteration_cap(gpulib):
    F0 = np.array([0.3, -0.2, 0.5])
    dt = 3e-3
    FE, n, cell = _grid(lambda r: (np.broadcast_to(F0, r.shape).copy(), np.full(r.shape[:-1], 0.25)))
    prm = _afm_prm(dt=dt, stiff=(0.0, 0.0, 0.0, 0.0), dpos0=(0.0, 0.0, -3.0, 3.0), zstep=0.1)
    # small coordinates keep the float32 rounding of 128 position updates below 3e-5 A, while
    # 127 instead of 128 moves would be 128 F dt^2 ~ 6e-4 A short
    pts = _tips(nx=2, ny=2, x0=2.0, y0=2.5, z=5.0)
    nz = 4
    W = np.array([0.5, -1.0, 0.25])
    FEs, paths, iters, X = _run(FE, n, cell, prm, pts, nz, W=W)
    assert (iters == 128).all()
    start = pts[:, :3] + np.array([0.0, 0.0, -3.0])
    for iz in range(nz):
        end = start + 128 * 129 / 2 * F0 * dt * dt
        np.testing.assert_allclose(paths[:, iz, :3], end, rtol=0, atol=3e-5)
        start = end + np.array([0.0, 0.0, -0.1])  # the next height: moved with the tip, from rest
    np.testing.assert_allclose(FEs[..., :3], np.broadcast_to(F0, FEs[..., :3].shape), rtol=1e-6)
    np.testing.assert_allclose(FEs[..., 3], 0.25, rtol=1e-6)
    np.testing.assert_allclose(X, F0[2] * W.sum(), rtol=1e-6)


def test_afm_relax_zero_force(gpulib):
    FE, n, cell = _grid(lambda r: (np.zeros(r.shape), np.zeros(r.shape[:-1])))
    prm = _afm_prm(stiff=(0.0, 0.0, 0.0, 0.0), dpos0=(0.2, 0.1, -3.0, 3.0))
    pts = _tips(nx=2, ny=3)
    FEs, paths, iters, _ = _run(FE, n, cell, prm, pts, 3)
    assert np.isfinite(paths).all() and np.isfinite(FEs).all()
    assert (iters == 0).all()
    for iz in range(3):
        np.testing.assert_allclose(paths[:, iz, :3], pts[:, :3] + np.array([0.2, 0.1, -3.0 - 0.1 * iz]), rtol=0, atol=2e-6)


def test_qzs_single_atom_against_energy_gradient(gpulib):
    """The AFMulator force field of one charged atom: F = -grad U, U = c12/r^12 - c6/r^6 +
    sum_k k_e q Q_k / |p + QZ_k z - R| (r^2 + R2SAFE in every distance), central differences."""
    from ppafm_gb300 import device as D

    R = np.array([3.3, 2.9, 4.1])
    c6, c12, q = 25.0, 4.5e4, 0.35
    Qs, QZs = [-10.0, 20.0, -10.0, 0.0], [0.1, 0.0, -0.1, 0.0]
    ke, r2safe = 14.399644, 1e-6
    n = np.array([24, 20, 32], np.int32)
    lvec = np.array([[0.0, 0.0, 0.0], [6.0, 0, 0], [0, 5.0, 0], [0, 0, 8.0]])
    ff = D.DeviceFF(n, lvec)
    atoms, na, nch = D.pack_atoms(R[None, :], np.array([[c6, c12]]), np.array([q]))
    g = ff.compute(atoms, na, nch, D.FF_QZS, Qs=Qs, QZs=QZs, with_E=True).grid4.cpu().numpy().astype(np.float64)

    def U(p):
        d = p - R
        r2 = (d * d).sum(-1) + r2safe
        u = c12 / r2**6 - c6 / r2**3
        for Q, z in zip(Qs, QZs):
            dq = d + np.array([0.0, 0.0, z])
            u = u + ke * q * np.float64(np.float32(Q)) / np.sqrt((dq * dq).sum(-1) + r2safe)
        return u

    ax = [np.arange(k) * (lvec[1 + i, i] / k) for i, k in enumerate(n)]
    P = np.stack(np.meshgrid(*ax, indexing="ij"), axis=-1)
    h = 1e-5
    F = np.stack([-(U(P + e) - U(P - e)) / (2 * h) for e in np.eye(3) * h], axis=-1)
    dist = np.linalg.norm(P - R, axis=-1)
    ok = dist > 1.0  # away from the repulsive core (where -grad U is huge and ill-posed for differences)
    scale = np.maximum(np.linalg.norm(F, axis=-1), 1e-2)
    err = np.linalg.norm(g[..., :3] - F, axis=-1) / scale
    assert err[ok].max() < 5e-5, err[ok].max()
    Eerr = np.abs(g[..., 3] - U(P)) / np.maximum(np.abs(U(P)), 1e-2)
    assert Eerr[ok].max() < 1e-4, Eerr[ok].max()


@pytest.mark.parametrize("tip", ["s", "pz"])
def test_hartree_tip_density_plane_waves(gpulib, tip):
    """The Hartree route with a tip density, no atoms: the potential V = cos(Gx x + Gz z) +
    0.5 sin(Gy y) on the force-field grid cross-correlated with a Gaussian tip density of width
    s (calc_force_hartree, field.py:1446-1504).  An s density of charge c multiplies each wave
    by c exp(-s^2 |G|^2 / 2); a pz density c (z / s) g(r) turns cos(G.r) into
    -c s Gz exp(-s^2 |G|^2 / 2) sin(G.r) (the sign fixes correlation against convolution).
    F = -grad E by periodic centred differences: a wave A cos(phase) gives A sin(phase)
    sin(G_k h) / h along axis k."""
    from ppafm_gb300.AFMulator import AFMulator, HartreePotential

    n = (16, 16, 20)
    lv = np.array([[0.0, 0, 0], [8.0, 0, 0], [0, 8.0, 0], [0, 0, 10.0]])
    h, s = 0.5, 0.7
    x, y, z = [np.arange(k) * h for k in n]
    Gx, Gy, Gz = 2 * np.pi / 8, 2 * 2 * np.pi / 8, 2 * 2 * np.pi / 10
    ph = Gx * x[:, None, None] + Gz * z[None, None, :] + 0 * y[None, :, None]
    wy = y[None, :, None] + 0 * ph
    V = (np.cos(ph) + 0.5 * np.sin(Gy * wy)).astype(np.float32)
    c = -0.3 if tip == "s" else 0.2
    afm = AFMulator(pixPerAngstrome=2, lvec=lv, rho={tip: c}, sigma=s, npbc=(0, 0, 0))
    assert tuple(afm.nDim) == n
    afm.prepareFF(np.zeros((0, 3)), np.zeros(0, dtype=np.int32), HartreePotential(V, lv), rot_center=np.zeros(3), REAs=np.zeros((0, 4)))
    FE = afm.downloadFF().astype(np.float64)
    A = np.exp(-(s * s) * (Gx**2 + Gz**2) / 2)
    B = 0.5 * np.exp(-(s * s) * Gy**2 / 2)
    if tip == "s":
        E = c * (A * np.cos(ph) + B * np.sin(Gy * wy))
        F = [c * A * np.sin(ph) * np.sin(Gx * h) / h, -c * B * np.cos(Gy * wy) * np.sin(Gy * h) / h, c * A * np.sin(ph) * np.sin(Gz * h) / h]
    else:  # only the wave with a z component survives an odd-in-z density
        a = -c * s * Gz * A
        E = a * np.sin(ph)
        F = [-a * np.cos(ph) * np.sin(Gx * h) / h, 0 * ph, -a * np.cos(ph) * np.sin(Gz * h) / h]
    for k, ref in enumerate(F + [E]):
        assert np.abs(FE[..., k] - ref).max() < 5e-6, (k, np.abs(FE[..., k] - ref).max())


def test_hartree_point_charge_tip_known_answers(gpulib):
    """The Hartree route with the point-charge tip, no atoms (field.py:1168-1317): the
    potential's field sampled at the tip charges Qs placed QZs above each force-field node.
    Potential on the force-field grid itself: periodic centred differences of a plane wave.
    Potential on a larger grid of its own: a linear potential, whose field the differences at
    +-0.05 A of the interpolated potential give exactly; the energy samples V at the charges,
    periodic over the force-field cell."""
    from ppafm_gb300.AFMulator import AFMulator, HartreePotential

    n = (16, 12, 20)
    lv = np.array([[0.0, 0, 0], [8.0, 0, 0], [0, 6.0, 0], [0, 0, 10.0]])
    h = 0.5
    kx, kz = 2 * np.pi / 8.0, 2 * 2 * np.pi / 10.0
    x, y, z = [np.arange(k) * h for k in n]
    one = np.ones(n)
    V = (np.sin(kx * x)[:, None, None] + 0.5 * np.cos(kz * z)[None, None, :]) * one
    Qs, QZs = [1.0, -2.0, 0.0, 0.0], [0.0, 1.0, 0.0, 0.0]
    none = (np.zeros((0, 3)), np.zeros(0, dtype=np.int32))
    kw = dict(rot_center=np.zeros(3), REAs=np.zeros((0, 4)))
    afm = AFMulator(pixPerAngstrome=2, lvec=lv, Qs=Qs, QZs=QZs, npbc=(0, 0, 0))
    assert tuple(afm.nDim) == n
    afm.prepareFF(*none, HartreePotential(V.astype(np.float32), lv), **kw)
    FE = afm.downloadFF().astype(np.float64)

    def field(zs):  # (Ex, Ez, V) of the wave at heights zs by centred differences
        ex = -np.cos(kx * x)[:, None, None] * np.sin(kx * h) / h * one
        ez = 0.5 * np.sin(kz * zs)[None, None, :] * np.sin(kz * h) / h * one
        return ex, ez, (np.sin(kx * x)[:, None, None] + 0.5 * np.cos(kz * zs)[None, None, :]) * one

    e0, e1 = field(z), field(z + 1.0)  # QZ = 1 A is two steps, periodic in the cell
    assert np.abs(FE[..., 0] - (e0[0] - 2 * e1[0])).max() < 1e-5
    assert np.abs(FE[..., 1]).max() < 1e-5
    assert np.abs(FE[..., 2] - (e0[1] - 2 * e1[1])).max() < 1e-5
    assert np.abs(FE[..., 3] - (e0[2] - 2 * e1[2])).max() < 1e-5
    a, b, cz = 0.3, -0.2, 0.5
    lvp = np.array([[-1.0, -1.0, -2.0], [12.0, 0, 0], [0, 10.0, 0], [0, 0, 16.0]])
    npot = (24, 20, 32)
    gp = [lvp[0][k] + np.arange(npot[k]) * 0.5 for k in range(3)]
    Vp = (a * gp[0][:, None, None] + b * gp[1][None, :, None] + cz * gp[2][None, None, :]).astype(np.float32)
    afm.prepareFF(*none, HartreePotential(Vp, lvp), **kw)
    FE = afm.downloadFF().astype(np.float64)
    for k, f in enumerate((a, b, cz)):  # F = sum_k Q_k (-grad V) = (1 - 2)(-a, -b, -c)
        assert np.abs(FE[..., k] - f).max() < 2e-3, (k, np.abs(FE[..., k] - f).max())

    def Vff(zs):
        return a * x[:, None, None] + b * y[None, :, None] + cz * zs[None, None, :]

    assert np.abs(FE[..., 3] - (Vff(z) - 2 * Vff((z + 1.0) % 10.0))).max() < 1e-4
