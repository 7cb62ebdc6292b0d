"""CPU checks of the oracle's multipole devices (MPSphereScatterDevice,
MPCylinderScatterDevice, multipole_scatter_device.cpp) and of the special functions they
need. The reference evaluates them with Boost (absent here); the oracle's own
implementations are pinned against scipy.special, and the two devices against the
physics they compute: with enough moments the sphere device equals the orientational
average over a dense near-uniform direction set, and for q perpendicular to the axis the
cylinder device equals the average over rotations of q about the axis."""
import numpy as np
import pytest

import oracle
from sassena_gb300 import synth

sp = pytest.importorskip("scipy.special")


def test_spherical_bessel_against_scipy():
    for L in (0, 1, 7, 20, 40):
        for x in np.concatenate([[1e-9, 1e-3, 0.3, 0.5, 1.0], np.linspace(0.6, 2 * L + 60, 53)]):
            j = oracle.sph_bessel(L, x)
            ref = sp.spherical_jn(np.arange(L + 1), x)
            assert np.abs(j - ref).max() <= 1e-13 * max(np.abs(ref).max(), 1e-300), (L, x)


def test_cylinder_bessel_against_scipy():
    for N in (0, 3, 40, 80):
        for x in np.concatenate([[1e-9, 1e-3, 0.5, 24.9, 25.0, 25.1], np.linspace(0.2, 220, 57)]):
            J = oracle.cyl_bessel(N, x)
            ref = sp.jv(np.arange(N + 1), x)
            assert np.abs(J - ref).max() <= 2e-13, (N, x, np.abs(J - ref).max())


def test_spherical_harmonics_against_scipy():
    rng = np.random.default_rng(0)
    L = 20
    for theta, phi in [(0.0, 0.0), (np.pi, 1.0), (np.pi / 2, 3 * np.pi / 2)] + \
            list(zip(rng.uniform(0, np.pi, 20), rng.uniform(0, 2 * np.pi, 20))):
        y = oracle.conj_ylm(L, theta, phi)
        ref = np.array([np.conj(sp.sph_harm_y(l, m, theta, phi))
                        for l in range(L + 1) for m in range(-l, l + 1)])
        assert np.abs(y - ref).max() <= 1e-12
        # addition theorem: sum_m |Y_lm|^2 = (2l+1)/(4 pi)
        k = 0
        for l in range(L + 1):
            assert abs(np.sum(np.abs(y[k:k + 2 * l + 1]) ** 2) - (2 * l + 1) / (4 * np.pi)) < 1e-12
            k += 2 * l + 1


def test_spherical_coordinates_as_staged():
    rng = np.random.default_rng(1)
    xyz = rng.normal(size=(500, 3)).astype(np.float32)
    xyz[:4] = [[0, 0, 0], [0, 2, 0], [0, -2, 1], [-1, 0, 0]]
    got = oracle.to_spherical(xyz)
    x, y, z = (xyz[:, k].astype(np.float64) for k in range(3))
    r = np.sqrt(x * x + y * y + z * z)
    theta = np.where(r > 0, np.arccos(np.where(r > 0, z / np.where(r > 0, r, 1), 1)), 0)
    phi = np.mod(np.arctan2(y, x), 2 * np.pi)
    assert np.allclose(got[:, 0], r.astype(np.float32), rtol=0, atol=1e-6)
    assert np.allclose(got[:, 2], theta.astype(np.float32), rtol=0, atol=1e-6)
    assert np.allclose(got[:, 1], phi.astype(np.float32), rtol=0, atol=1e-6)
    assert got[0].tolist() == [0, 0, 0] and abs(got[1, 1] - np.pi / 2) < 1e-6


def molecule(seed=1, na=12, nf=6):
    rng = np.random.default_rng(seed)
    r0 = rng.normal(size=(na, 3)) * 2.0
    coords = np.stack([r0 + rng.normal(size=(na, 3)) * 0.3 for _ in range(nf)]).astype(np.float32)
    return coords, rng.uniform(0.5, 2.0, na)


def test_sphere_device_equals_dense_orientational_average():
    coords, b = molecule()
    q = np.array([[0.3, -0.5, 0.8]])
    fm = oracle.mp_sphere(coords, q, b[None], oracle.sphere_moments(24))
    dirs = synth.fibonacci_sphere(20000)
    fv = oracle.all_vectors(coords, np.array([0, len(dirs)], np.uintp), np.linalg.norm(q) * dirs,
                            b[None])
    # fqt and fq are linear in the per-moment / per-direction power and must agree; fq2 sums
    # squared per-moment means and depends on the basis
    for a, v in zip(fm[:2], fv[:2]):
        assert np.abs(a - v).max() <= 3e-6 * np.abs(fv[0][0, 0]).max()


def test_cylinder_device_equals_rotational_average():
    coords, b = molecule(seed=2)
    qc = np.array([[0.9, 0.4, 0.0]])
    fc = oracle.mp_cylinder(coords, qc, b[None], oracle.cylinder_moments(24), [0, 0, 1.0])
    M = 720
    ph = np.arange(M) * 2 * np.pi / M
    rot = np.linalg.norm(qc) * np.stack([np.cos(ph), np.sin(ph), np.zeros(M)], 1)
    fr = oracle.all_vectors(coords, np.array([0, M], np.uintp), rot, b[None])
    for a, v in zip(fc[:2], fr[:2]):
        assert np.abs(a - v).max() <= 1e-7 * np.abs(fr[0][0, 0]).max()


def test_cylinder_phase_uses_absolute_z_qz():
    # the reference multiplies z q_z by its own sign (parallel_sign,
    # multipole_scatter_device.cpp:944-948): the result cannot tell z from -z
    coords, b = molecule(seed=3)
    mirrored = coords.copy()
    mirrored[..., 2] *= -1
    q = np.array([[0.5, 0.2, 0.7]])
    mom = oracle.cylinder_moments(6)
    a = oracle.mp_cylinder(coords, q, b[None], mom, [0, 0, 1.0])
    m = oracle.mp_cylinder(mirrored, q, b[None], mom, [0, 0, 1.0])
    assert np.allclose(a[0], m[0], rtol=1e-12, atol=1e-12)


def test_invalid_moments_rejected():
    coords, b = molecule()
    q = np.array([[0.3, 0.0, 0.0]])
    with pytest.raises(ValueError):
        oracle.mp_sphere(coords, q, b[None], [(2, 3)])
    with pytest.raises(ValueError):
        oracle.mp_cylinder(coords, q, b[None], [(1, 4)], [0, 0, 1.0])
    with pytest.raises(ValueError):
        oracle.mp_cylinder(coords, q, b[None], [(0, 1)], [0, 0, 1.0])
