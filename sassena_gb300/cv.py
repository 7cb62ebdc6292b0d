"""Learned control variate workflow: training data from the library's own exact intensities,
GPU training of the network, and the control-variate orientational average.

The intensities used as training targets are |A(q u)|^2 averaged over the trajectory's frames,
computed by the phase-sum kernels (sass_amplitudes); the network and the estimator run in the
CUDA library (sass_mlp_*, sass_compute_cv)."""
from __future__ import annotations

import numpy as np

from . import abi, synth


def training_set(plan, w, n_samples, seed=0, frames=None):
    """(x [n][4] float32, target [n] float32, scaling) for workload `w` staged in `plan`.

    Samples are (u, |q|) with u uniform on the sphere and |q| uniform over the shells' range;
    the target is log(mean_t |A(q u, t)|^2 / NA), normalised to zero mean and unit variance."""
    rng = np.random.default_rng(seed)
    qmin, qmax = float(w.shells.min()), float(w.shells.max())
    q_mid, q_half = 0.5 * (qmin + qmax), max(0.5 * (qmax - qmin), 1e-6)
    # sample shells on a grid of 64 |q| values so amplitude groups stay full
    grid = np.linspace(qmin, qmax, 64)
    shell = np.sort(rng.integers(0, len(grid), n_samples))
    u = synth.sphere_directions(n_samples, seed + 17)
    sv = grid[shell, None] * u
    cf = np.tile(w.class_factors[:1], (len(grid), 1))
    amp = plan.amplitudes(sv, shell.astype(np.int32), cf)
    inten = np.mean(np.abs(amp) ** 2, axis=1) / w.na
    logi = np.log(np.maximum(inten, 1e-30))
    y_mean, y_std = float(logi.mean()), float(logi.std() or 1.0)
    x = np.concatenate([u, ((grid[shell] - q_mid) / q_half)[:, None]], axis=1).astype(np.float32)
    t = ((logi - y_mean) / y_std).astype(np.float32)
    perm = rng.permutation(n_samples)
    return x[perm], t[perm], dict(q_mid=q_mid, q_half=q_half, y_mean=y_mean + np.log(w.na),
                                  y_std=y_std)


def fit(x, t, scaling, steps=2000, batch=4096, lr=2e-3, seed=0, device=0):
    """Train a fresh network on the GPU; returns (net, final mini-batch loss)."""
    net = abi.MLP(device=device, seed=seed)
    net.set_scaling(scaling["q_mid"], scaling["q_half"], scaling["y_mean"], scaling["y_std"])
    loss = net.train(x, t, steps=steps, batch=batch, lr=lr)
    return net, loss
