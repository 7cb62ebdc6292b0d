"""The learned control variate: network gradients against the FP64 oracle, GPU training,
sphere quadrature, and what the trained network gains over plain Monte Carlo at an equal
direction budget on an anisotropic (layered) sample, with the estimate staying unbiased."""
import numpy as np
import pytest

import oracle.mlp_oracle as mo
from sassena_gb300 import abi, cv, synth

pytestmark = pytest.mark.gpu


def test_mlp_gradient_matches_oracle(native_lib):
    net = abi.MLP(seed=3)
    rng = np.random.default_rng(0)
    x = rng.normal(size=(777, 4)).astype(np.float32)
    t = rng.normal(size=777).astype(np.float32)
    master, bf = net.params()
    g, loss = net.gradient(x, t)
    gref, lref = mo.gradient(bf, x, t)  # the GPU computes with the BF16 weights
    assert abs(loss - lref) <= 1e-5 * abs(lref)
    err = np.abs(g - gref).max() / np.abs(gref).max()
    assert err <= 2e-5, err
    # and the forward pass. The 128 x 128 layer's operand h1 is rounded to BF16 on both
    # sides, but from the GPU's FP32 tanh and the oracle's FP64 tanh: where those straddle a
    # BF16 rounding boundary (a few of the 10^5 values here), h1 differs by one BF16 step
    # (2^-8 relative) and that sample's y by up to about 1e-3. All others agree to 1e-5.
    y = net.predict(x)
    yref, _ = mo.forward(bf, x)
    dev = np.abs(y - yref) / max(1.0, np.abs(yref).max())
    assert np.mean(dev <= 1e-5) >= 0.99 and dev.max() <= 2e-3, (np.mean(dev <= 1e-5), dev.max())


def test_mlp_training_is_reproducible(native_lib):
    """The gradient and the loss are summed over the CTAs in a fixed order (no floating-point
    atomics): two evaluations give the same bits, and two trainings from the same seed on
    the same data end with the same weights; so does the sphere quadrature."""
    rng = np.random.default_rng(7)
    x = rng.normal(size=(5000, 4)).astype(np.float32)
    t = rng.normal(size=5000).astype(np.float32)
    net = abi.MLP(seed=5)
    g1, l1 = net.gradient(x, t)
    g2, l2 = net.gradient(x, t)
    assert np.array_equal(g1, g2) and l1 == l2
    weights = []
    for _ in range(2):
        n = abi.MLP(seed=5)
        n.train(x, t, steps=50, batch=1024, lr=1e-3)
        weights.append(n.params()[0])
        q = np.array([0.3, 0.9])
        weights.append(n.sphere_mean(q, 50000))
    assert np.array_equal(weights[0], weights[2]) and np.array_equal(weights[1], weights[3])


def test_mlp_training_fits_a_smooth_function(native_lib):
    rng = np.random.default_rng(1)
    u = synth.sphere_directions(20000, 5)
    s = rng.uniform(-1, 1, 20000)
    x = np.concatenate([u, s[:, None]], axis=1).astype(np.float32)
    t = (np.sin(3 * u[:, 0]) + u[:, 2] ** 2 * (1 + s)).astype(np.float32)
    net = abi.MLP(seed=2)
    _, loss0 = net.gradient(x, t)
    net.train(x, t, steps=1500, batch=2048, lr=3e-3)
    _, loss1 = net.gradient(x, t)
    assert loss1 < 0.02 * loss0, (loss0, loss1)


def test_sphere_mean_matches_quadrature_in_numpy(native_lib):
    net = abi.MLP(seed=4)
    net.set_scaling(1.0, 0.5, 0.2, 0.7)
    q = np.array([0.6, 1.0, 1.4])
    got = net.sphere_mean(q, 4096)
    _, bf = net.params()
    P = 4096
    i = np.arange(P) + 0.5
    z = 1 - 2 * i / P
    r = np.sqrt(1 - z * z)
    phi = np.pi * (3 - np.sqrt(5)) * i
    u = np.stack([r * np.cos(phi), r * np.sin(phi), z], 1)
    for k, qq in enumerate(q):
        x = np.concatenate([u, np.full((P, 1), (qq - 1.0) / 0.5)], 1)
        y, _ = mo.forward(bf, x)
        ref = np.mean(np.exp(y * 0.7 + 0.2))
        assert abs(got[k] - ref) <= 1e-5 * ref


def _cv_errors(w, m, seeds, train_samples=20000, steps=2500):
    with abi.Plan(w.na, w.nf, len(w.class_names), "all", "autocorrelate", "fftw", "fp32") as p:
        p.stage(w.coords)
        p.set_classes(w.atom_class)
        x, t, sc = cv.training_set(p, w, train_samples, seed=1)
        net, _ = cv.fit(x, t, sc, steps=steps, batch=2048, lr=2e-3)
        # truth: a dense quasi-uniform direction set
        nd = 8192
        dense = synth.fibonacci_sphere(nd)
        offs = (np.arange(w.nq + 1) * nd).astype(np.uintp)
        sv = (w.shells[:, None, None] * dense[None]).reshape(-1, 3)
        truth, _, _ = p.compute(offs, sv, w.class_factors)
        e_cv, e_mc = [], []
        for seed in seeds:
            dirs = synth.sphere_directions(m, 100 + seed)
            fqt_cv, fqt_mc, _, _, _ = abi.compute_cv(p, net, w.shells, dirs, w.class_factors,
                                                      nquad=65536)
            e_cv.append((fqt_cv[:, :4] - truth[:, :4]).real / truth[:, :1].real)
            e_mc.append((fqt_mc[:, :4] - truth[:, :4]).real / truth[:, :1].real)
    return np.array(e_cv), np.array(e_mc)


def test_control_variate_gain_and_unbiased(native_lib):
    # aligned rods: a smooth, strongly anisotropic orientational dependence that the network
    # can learn; the control variate removes most of the Monte Carlo variance
    w = synth.aligned_rods(seed=6, nmol=300, per_mol=8, nf=32, nq=3)
    e_cv, e_mc = _cv_errors(w, m=32, seeds=range(24))
    rms_cv, rms_mc = np.sqrt(np.mean(e_cv ** 2)), np.sqrt(np.mean(e_mc ** 2))
    print("control variate: rms error %.4f vs plain MC %.4f (gain %.2fx, %.1fx fewer directions "
          "for equal error)" % (rms_cv, rms_mc, rms_mc / rms_cv, (rms_mc / rms_cv) ** 2))
    assert rms_cv < 0.6 * rms_mc, (rms_cv, rms_mc)
    # unbiased: the mean error over seeds is within 3 standard errors
    se = e_cv.std(axis=0) / np.sqrt(len(e_cv))
    assert np.all(np.abs(e_cv.mean(axis=0)) <= 3 * se + 1e-4), (e_cv.mean(axis=0), se)


def test_control_variate_on_speckle_dominated_sample_stays_unbiased(native_lib):
    # layered disordered box: variance dominated by speckle the network cannot learn; the
    # estimator must still be unbiased and not worse than plain Monte Carlo by much
    w = synth.layered(seed=8, na=3000, nf=16, box=24.0, period=6.0, amplitude=0.6, nq=3,
                      qmin=0.8, qmax=1.3, nm=8)
    e_cv, e_mc = _cv_errors(w, m=32, seeds=range(16))
    rms_cv, rms_mc = np.sqrt(np.mean(e_cv ** 2)), np.sqrt(np.mean(e_mc ** 2))
    assert rms_cv < 1.25 * rms_mc, (rms_cv, rms_mc)
    se = e_cv.std(axis=0) / np.sqrt(len(e_cv))
    assert np.all(np.abs(e_cv.mean(axis=0)) <= 3.5 * se + 1e-4), (e_cv.mean(axis=0), se)
