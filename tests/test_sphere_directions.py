"""Orientations of vectors.type = sphere / cylinder (algorithm boost_uniform_on_sphere).

The reference draws them with boost::mt19937 seeded by vectors.seed and
boost::uniform_on_sphere<double>(3) (sphere) or (2) (cylinder) through a variate_generator
(parameters.cpp:945-959, :1001-1012). The host layer restates Boost.Random's published
algorithms; this file restates them a second time in Python from the published
descriptions (the Mersenne Twister of Matsumoto and Nishimura, Marsaglia's 1972 method
for points on a sphere, the Box-Muller transform) and compares the driver's orientations
bit for bit, for Boost 1.56 and later (the default) and for Boost 1.47 to 1.55.
"""
import json
import math
import subprocess

import numpy as np
import pytest

from sassena_gb300 import abi, synth


class MT19937:
    """The 32-bit Mersenne Twister with its standard seeding (init_genrand)."""

    def __init__(self, seed):
        mt = [seed & 0xFFFFFFFF]
        for i in range(1, 624):
            mt.append((1812433253 * (mt[-1] ^ (mt[-1] >> 30)) + i) & 0xFFFFFFFF)
        self.mt, self.i = mt, 624

    def __call__(self):
        mt = self.mt
        if self.i >= 624:
            for k in range(624):
                y = (mt[k] & 0x80000000) | (mt[(k + 1) % 624] & 0x7FFFFFFF)
                mt[k] = mt[(k + 397) % 624] ^ (y >> 1) ^ (0x9908B0DF if y & 1 else 0)
            self.i = 0
        y = mt[self.i]
        self.i += 1
        y ^= y >> 11
        y ^= (y << 7) & 0x9D2C5680
        y ^= (y << 15) & 0xEFC60000
        return y ^ (y >> 18)


def test_mt19937_known_answer():
    g = MT19937(5489)  # the C++ standard's check: the 10,000th draw of the default seed
    for _ in range(9999):
        g()
    assert g() == 4123659995


def marsaglia(seed, n, dim):
    """uniform_on_sphere<double>(dim), Boost 1.56 and later, dim 2 or 3."""
    g = MT19937(seed)
    u = lambda: g() * (1.0 / 4294967296.0)  # noqa: E731  uniform_01: x * 2^-32
    out = []
    for _ in range(n):
        while True:
            x = u() * 2 - 1
            y = u() * 2 - 1
            s = x * x + y * y
            if not ((dim == 2 and s == 0) or s > 1):
                break
        if dim == 3:
            m = 2 * math.sqrt(1 - s)
            out.append((x * m, y * m, 2 * s - 1))
        else:
            m = 1 / math.sqrt(s)
            out.append((x * m, y * m, 0.0))
    return np.array(out)


def box_muller(seed, n, dim):
    """uniform_on_sphere<double>(dim), Boost 1.47 to 1.55: normal variates by Box-Muller
    pairs (the second kept for the next call, across orientations), divided by the length."""
    g = MT19937(seed)
    u = lambda: g() * (1.0 / 4294967296.0)  # noqa: E731
    state = {"valid": False}

    def normal():
        if not state["valid"]:
            state["r1"] = u()
            r2 = u()
            state["rho"] = math.sqrt(-2.0 * math.log(1.0 - r2))
            state["valid"] = True
        else:
            state["valid"] = False
        pi = 3.14159265358979323846
        f = math.cos if state["valid"] else math.sin
        return state["rho"] * f(2.0 * pi * state["r1"]) * 1.0 + 0.0

    out = []
    for _ in range(n):
        v = [normal() for _ in range(dim)]
        s = 0.0
        for c in v:
            s += c * c
        l = math.sqrt(s)
        v = [c / l for c in v] + [0.0] * (3 - dim)
        out.append(v)
    return np.array(out)


def driver_orientations(tmp_path, vtype, seed, resolution, boost=None):
    w = synth.small("all", seed=2, na=5, nf=3, nq=1, nm=1)
    axis = "" if vtype == "sphere" else "<axis><x>0</x><y>0</y><z>1</z></axis>"
    average = ("<average><orientation><type>vectors</type>%s<vectors><type>%s</type>"
               "<algorithm>boost_uniform_on_sphere</algorithm><resolution>%d</resolution><seed>%d</seed>"
               "</vectors></orientation></average>" % (axis, vtype, resolution, seed))
    extra = "<gpu><boost_random>%s</boost_random></gpu>" % boost if boost else ""
    cfg = synth.write_files(str(tmp_path / "s"), w, average=average, extra=extra)
    out = str(tmp_path / "dry.json")
    r = subprocess.run([abi.DRIVER_PATH, "--config", cfg, "--dry-run", out], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return np.array(json.load(open(out))["orientations"])


@pytest.mark.parametrize("seed", [0, 7, 4294967301])  # the last one truncates to 5, as mt19937::seed does
@pytest.mark.parametrize("vtype,dim", [("sphere", 3), ("cylinder", 2)])
def test_driver_draws_boost_156_orientations(tmp_path, vtype, dim, seed):
    got = driver_orientations(tmp_path, vtype, seed, 50)
    want = marsaglia(seed, 50, dim)
    assert got.shape == (50, 3)
    assert np.array_equal(got, want)
    assert np.allclose(np.linalg.norm(got, axis=1), 1.0, atol=1e-15)


@pytest.mark.parametrize("vtype,dim", [("sphere", 3), ("cylinder", 2)])
def test_driver_draws_boost_147_orientations(tmp_path, vtype, dim):
    got = driver_orientations(tmp_path, vtype, 11, 40, boost="1.47")
    want = box_muller(11, 40, dim)
    # libm's log/sin/cos may differ from Python's in the last bit
    assert np.allclose(got, want, rtol=0, atol=4e-16)


def test_truncated_seed_gives_the_same_stream(tmp_path):
    a = driver_orientations(tmp_path / "a", "sphere", 5, 10)
    b = driver_orientations(tmp_path / "b", "sphere", 4294967301, 10)
    assert np.array_equal(a, b)
