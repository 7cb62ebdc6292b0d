"""CPU checks of bench.py's own arithmetic: the per-shell error metric, the roofline peaks and
the ncu traffic lookup (no GPU)."""
import json
import os

import numpy as np

import bench


def test_shell_errors_metric():
    # two shells, three frames; S(q,t) error relative to |S_ref(q,0)|, I(q) relative to itself
    ref_fqt = np.array([[4.0, 2.0, 1.0], [2.0 + 2.0j, 1.0, 0.5]])
    got_fqt = ref_fqt + np.array([[0.004, -0.008, 0.0], [0.0, 0.0, 0.001j]])
    ref_fq = np.array([2.0, 1.0 + 1.0j])
    got_fq = ref_fq * (1 + 1e-3)
    ref_fq2 = np.array([5.0, 2.0])
    got_fq2 = ref_fq2 + np.array([0.0, 2e-3])
    e = bench.shell_errors((got_fqt, got_fq, got_fq2), (ref_fqt, ref_fq, ref_fq2))
    np.testing.assert_allclose(e["sqt"], [0.008 / 4.0, 0.001 / abs(2 + 2j)])
    np.testing.assert_allclose(e["fq"], [1e-3, 1e-3])
    np.testing.assert_allclose(e["fq0"], [0.004 / 4.0, 0.0])
    np.testing.assert_allclose(e["fq2"], [0.0, 1e-3])


def test_hbm_peak_reads_the_measured_copy_bandwidth(tmp_path, monkeypatch):
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    peak, src = bench.hbm_peak()
    assert peak == 6800.0 and "fallback" in src
    (tmp_path / "MEASURED_PEAKS.json").write_text(json.dumps({"hbm_gbs": 6688.8}))
    peak, src = bench.hbm_peak()
    assert peak == 6688.8 and "measured" in src


def test_profile_traffic_lookup():
    # the committed captures of the dominant kernels
    assert bench.profile_traffic("phase_rec_kernel", "coherent_sqt") > 2e8
    assert bench.profile_traffic("reg2_fft_kernel", "incoherent_fqt") > 1e6
    assert bench.profile_traffic("phase_rec_kernel", "static_xray") > 2e8
    assert bench.profile_traffic("no_such_kernel", "coherent_sqt") is None
    for name in os.listdir(os.path.join(bench.ROOT, "profiles")):
        if name.endswith(".json"):
            with open(os.path.join(bench.ROOT, "profiles", name)) as f:
                d = json.load(f)
            assert "command" in d and ("dram_bytes_per_launch" in d or "fp64_pipe_inst_per_term" in d)
