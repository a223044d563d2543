"""Known answers for the oracle's restatement of the AFMulator relaxation (CPU, no GPU).

The GPU kernels of the AFMulator are pinned by cases whose answer follows from the physics
(tests/test_gpu_afm_known.py).  The oracle's C restatement of relaxStrokesTilted + update_FIRE
+ tipForce (relax.cl:37-41, 105-126, 391-464), oc_afm_relax_tilted, which the generator tests
compare the GPU images with, is held here to the same answers, so that it is pinned on its own
and not only by agreement with the GPU:
  * a linear force field -K (r - c) plus the tip springs: every height stops within |F|/k of
    the analytic fixed point, with the warm start carried over the heights;
  * a uniform field plus the radial and lateral springs: the equilibrium solved by Newton's
    method in float64;
  * the 128-iteration cap: with no springs and a constant field the probe moves n(n+1)/2 F dt^2
    in n moves from rest, so after the cap it is at pos0 + 8256 F dt^2 at every height;
  * a zero field: F2SAFE keeps the mixing term finite, the first evaluation converges.
The oracle samples an x-fastest float4 grid (the OpenCL image's layout) with the fractional
coordinates dot(r, row_k of inv(cell)^T) n_k."""

import ctypes

import numpy as np

EVA_NM = 16.0217662


def _grid(field, n=(64, 64, 64), L=16.0):
    """x-fastest float4 grid [nz][ny][nx][4] of field(r) -> (F [..., 3], E) at r = i L / n."""
    ax = [np.arange(k) * (L / k) for k in n]
    Z, Y, X = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    r = np.stack([X, Y, Z], axis=-1)
    F, E = field(r)
    FE = np.ascontiguousarray(np.concatenate([F, E[..., None]], axis=-1), dtype=np.float32)
    return FE, np.array(n, np.int32), np.eye(3) * L


def _tips(nx=6, ny=5, x0=6.0, y0=6.5, z=12.0, step=0.6):
    xs, ys = np.meshgrid(x0 + step * np.arange(nx), y0 + step * np.arange(ny), indexing="ij")
    return np.column_stack([xs.ravel(), ys.ravel(), np.full(xs.size, z), np.zeros(xs.size)])


def _run(oracle, FE, n, cell, points, nz, dt=0.5, damp=0.1, stiff=(0.0, 0.0, 0.0, 0.0), dpos0=(0.0, 0.0, -4.0, 4.0), zstep=0.1):
    """oc_afm_relax_tilted with an identity tip rotation moving down by zstep per height;
    returns FEs, paths [npix, nz, 4], iters [npix, nz]."""
    L = oracle.lib()
    f32 = lambda a: np.ascontiguousarray(a, dtype=np.float32)  # noqa: E731
    fp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))  # noqa: E731
    npix = len(points)
    dinv = f32(np.linalg.inv(cell).T)
    tip = f32([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, -zstep])
    pts, st, d0, rx, surf = f32(points), f32(stiff), f32(dpos0), f32([dt, damp, 0.0, 0.0]), f32(np.zeros(4))
    FEs = np.zeros((npix, nz, 4), np.float32)
    paths = np.zeros((npix, nz, 4), np.float32)
    iters = np.zeros((npix, nz), np.int32)
    FEc = f32(FE)
    L.oc_afm_relax_tilted(fp(FEc), n.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), fp(dinv), npix, fp(pts), nz, fp(tip), fp(st), fp(d0), fp(rx), fp(surf), fp(FEs), fp(paths), iters.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), 0)
    return FEs, paths, iters


def test_oracle_afm_linear_field_fixed_point(oracle):
    K = np.array([0.3, 0.2, 0.6])  # eV/A^2
    c = np.array([8.0, 7.5, 8.0])
    ks = 0.05  # lateral and vertical tip springs, eV/A^2 (stiffness -ks)
    d0 = np.array([0.1, -0.2, -3.0])
    FE, n, cell = _grid(lambda r: (-(r - c) * K, -0.5 * ((r - c) ** 2 * K).sum(-1)))
    pts = _tips()
    nz, zstep = 6, 0.1
    FEs, paths, iters = _run(oracle, FE, n, cell, pts, nz, stiff=(-ks, -ks, -ks, 0.0), dpos0=(*d0, 3.0), zstep=zstep)
    assert (iters < 128).all() and (iters >= 0).all()
    for iz in range(nz):
        tip = pts[:, :3] - np.array([0, 0, zstep * iz])
        fixed = (K * c + ks * (tip + d0)) / (K + ks)  # -K (r - c) - ks (r - tip - d0) = 0
        seen = c - FEs[:, iz, :3] / K  # where |F| < 1e-4 eV/A was seen (before the last move)
        err = np.abs(seen - fixed)
        assert (err <= 1e-4 / (K + ks) + 1e-5).all(), (iz, err.max(0))
        assert np.linalg.norm(paths[:, iz, :3] - seen, axis=-1).max() < 1e-3


def test_oracle_afm_radial_spring_uniform_field(oracle):
    F0 = np.array([0.05, -0.03, 0.4])
    kl, kr, l0 = 0.5, 30.0 / EVA_NM, 4.0
    d0 = np.array([0.0, 0.0, -l0])
    FE, n, cell = _grid(lambda r: (np.broadcast_to(F0, r.shape).copy(), np.zeros(r.shape[:-1])))
    pts = _tips(nx=3, ny=3)
    FEs, paths, iters = _run(oracle, FE, n, cell, pts, 3, stiff=(-kl, -kl, 0.0, -kr), dpos0=(*d0, l0))

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
        assert (err <= 1e-4 / kmin + 1e-4).all(), (iz, err.max(), 1e-4 / kmin)
    assert (iters < 128).all()


def test_oracle_afm_iteration_cap(oracle):
    F0 = np.array([0.3, -0.2, 0.5])
    dt = 3e-3
    FE, n, cell = _grid(lambda r: (np.broadcast_to(F0, r.shape).copy(), np.full(r.shape[:-1], 0.25)))
    pts = _tips(nx=2, ny=2, x0=2.0, y0=2.5, z=5.0)
    nz = 4
    FEs, paths, iters = _run(oracle, FE, n, cell, pts, nz, dt=dt, dpos0=(0.0, 0.0, -3.0, 3.0))
    assert (iters == 128).all()
    start = pts[:, :3] + np.array([0.0, 0.0, -3.0])
    for iz in range(nz):
        end = start + 128 * 129 / 2 * F0 * dt * dt
        np.testing.assert_allclose(paths[:, iz, :3], end, rtol=0, atol=3e-5)
        start = end + np.array([0.0, 0.0, -0.1])  # the next height: moved with the tip, from rest
    np.testing.assert_allclose(FEs[..., :3], np.broadcast_to(F0, FEs[..., :3].shape), rtol=1e-6)
    np.testing.assert_allclose(FEs[..., 3], 0.25, rtol=1e-6)


def test_oracle_afm_zero_force(oracle):
    FE, n, cell = _grid(lambda r: (np.zeros(r.shape), np.zeros(r.shape[:-1])))
    pts = _tips(nx=2, ny=3)
    FEs, paths, iters = _run(oracle, FE, n, cell, pts, 3, dpos0=(0.2, 0.1, -3.0, 3.0))
    assert np.isfinite(paths).all() and np.isfinite(FEs).all()
    assert (iters == 0).all()
    for iz in range(3):
        np.testing.assert_allclose(paths[:, iz, :3], pts[:, :3] + np.array([0.2, 0.1, -3.0 - 0.1 * iz]), rtol=0, atol=2e-6)


def test_oracle_afm_ff_single_atom_against_energy_gradient(oracle):
    """The oracle's evalLJC_QZs_noPos for one charged atom against F = -grad U with U =
    c12/r^12 - c6/r^6 + sum_k k_e q Q_k / |p + QZ_k z - R| (r^2 + R2SAFE in every distance), by
    central differences, and its energy channel against U: the float64 sum within 1e-6
    relative; the float32 form (FF.cl's, the GPU images' comparison), which adds the tip
    charges' terms one by one and so loses the significand they cancel (a neutral -10/+20/-10 e
    tip), within 2^-17 of the terms' summed magnitudes (128 float32 ulps: each term of FF.cl's
    float32 evaluation carries the roundings of r^2, its root and the products; measured 37 ulps
    at worst here, where a wrong sign, charge or offset would be off by O(1))."""
    R = np.array([3.3, 2.9, 4.1])
    c6, c12, q = 25.0, 4.5e4, 0.35
    Qs, QZs = np.array([-10.0, 20.0, -10.0, 0.0]), np.array([0.1, 0.0, -0.1, 0.0])
    ke, r2safe = 14.399644, 1e-6
    n = np.array([24, 20, 32])
    lvec = np.array([[0.0, 0.0, 0.0], [6.0, 0, 0], [0, 5.0, 0], [0, 0, 8.0]])
    FE32 = oracle.afm_ff_qzs(n, lvec, R[None, :], np.array([q]), np.array([[c6, c12]]), Qs, QZs).astype(np.float64)
    FE32 = FE32.transpose(2, 1, 0, 3)  # [nx, ny, nz, 4]
    FE64 = oracle.afm_ff_qzs64(n, lvec, R[None, :], np.array([q]), np.array([[c6, c12]]), Qs, QZs).reshape(*n, 4)

    ax = [np.arange(k) * (lvec[1 + i, i] / k) for i, k in enumerate(n)]
    P = np.stack(np.meshgrid(*ax, indexing="ij"), axis=-1)
    d = P - R

    def U(p):
        dd = p - R
        r2 = (dd * dd).sum(-1) + r2safe
        u = c12 / r2**6 - c6 / r2**3
        for Q, z in zip(Qs, QZs):
            dq = dd + np.array([0.0, 0.0, z])
            u = u + ke * q * np.float64(np.float32(Q)) / np.sqrt((dq * dq).sum(-1) + r2safe)
        return u

    h = 1e-5
    F = np.stack([-(U(P + e) - U(P - e)) / (2 * h) for e in np.eye(3) * h], axis=-1)
    ok = np.linalg.norm(d, axis=-1) > 1.0  # away from the repulsive core
    scale = np.maximum(np.linalg.norm(F, axis=-1), 1e-2)
    err = np.linalg.norm(FE64[..., :3] - F, axis=-1) / scale
    assert err[ok].max() < 1e-6, err[ok].max()
    Eerr = np.abs(FE64[..., 3] - U(P)) / np.maximum(np.abs(U(P)), 1e-2)
    assert Eerr[ok].max() < 1e-6, Eerr[ok].max()
    # magnitudes of the summed terms: the LJ force and each tip charge's Coulomb force
    r2 = (d * d).sum(-1) + r2safe
    S = np.abs(12 * c12 / r2**7 - 6 * c6 / r2**4) * np.sqrt(r2)
    SE = np.abs(c12 / r2**6) + np.abs(c6 / r2**3)
    for Q, z in zip(Qs, QZs):
        if Q != 0:
            rq2 = ((d + np.array([0.0, 0.0, z])) ** 2).sum(-1) + r2safe
            S = S + ke * abs(q * Q) / rq2
            SE = SE + ke * abs(q * Q) / np.sqrt(rq2)
    err32 = np.linalg.norm(FE32[..., :3] - F, axis=-1)
    assert (err32[ok] <= 2.0**-17 * S[ok] + 1e-6 * scale[ok]).all(), (err32[ok] / S[ok]).max()
    assert (np.abs(FE32[..., 3] - U(P))[ok] <= 2.0**-17 * SE[ok] + 1e-6).all()
