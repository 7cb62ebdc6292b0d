"""CPU tests of the C++ host layer: configuration, database, PDB/DCD, staging,
scatter-factor classes, sub-vectors and the signal.h5 writer/reader (no GPU)."""
import json
import os
import subprocess

import numpy as np
import pytest

import oracle
from sassena_gb300 import abi, synth

import h5lite


def run_driver(*args):
    return subprocess.run([abi.DRIVER_PATH] + list(args), capture_output=True, text=True)


def dry(cfg, tmp_path, *extra):
    out = str(tmp_path / "dry.json")
    r = run_driver("--config", cfg, "--dry-run", out, *extra)
    assert r.returncode == 0, r.stderr
    return json.load(open(out))


# ---- signal.h5 ----------------------------------------------------------------------------
def test_signal_roundtrip_and_structure(tmp_path):
    rng = np.random.default_rng(0)
    nq, nf = 7, 13
    q = rng.normal(size=(nq, 3))
    fqt = rng.normal(size=(nq, nf)) + 1j * rng.normal(size=(nq, nf))
    fq = rng.normal(size=nq) + 1j * rng.normal(size=nq)
    fq2 = rng.normal(size=nq) + 0j
    path = str(tmp_path / "signal.h5")
    abi.write_signal(path, q, fqt, fqt[:, 0], fq, fq2, rawconfig="<root>cfg</root>",
                     database="<root>db</root>")
    # the host reader
    d = abi.read_signal(path)
    assert np.array_equal(d["qvectors"], q)
    assert np.array_equal(d["fqt"], fqt) and np.array_equal(d["fq2"], fq2)
    # an independent reader, with structural checks
    f = h5lite.File(path)
    assert sorted(f.root) == ["fq", "fq0", "fq2", "fqt", "meta", "qvectors"]
    assert np.array_equal(f.read("qvectors"), q)
    got = f.read("fqt")
    assert got.shape == (nq, nf, 2) and got.dtype == np.float64
    assert np.array_equal(got[..., 0] + 1j * got[..., 1], fqt)
    assert np.array_equal(f.read("fq0"), np.stack([fqt[:, 0].real, fqt[:, 0].imag], 1))
    assert f.read("meta/config") == b"<root>cfg</root>"
    assert f.read("meta/database") == b"<root>db</root>"
    raw = f.read("meta/rawconfig")
    assert raw.dtype == np.int8 and raw.tobytes() == b"<root>cfg</root>"


def test_signal_chunked_like_reference(tmp_path):
    # root datasets: chunked, unlimited first dimension, the reference's chunk shapes
    # (file_writer_service.cpp:68-159); /meta stays contiguous
    rng = np.random.default_rng(1)
    nq, nf = 5, 13
    q = rng.normal(size=(nq, 3))
    fqt = rng.normal(size=(nq, nf)) + 1j * rng.normal(size=(nq, nf))
    path = str(tmp_path / "c.h5")
    abi.write_signal(path, q, fqt, fqt[:, 0], fqt[:, 1], fqt[:, 2])
    f = h5lite.File(path)
    unlimited = 0xFFFFFFFFFFFFFFFF
    qi = f.info("qvectors")
    assert qi["layout"] == "chunked" and qi["chunk"] == (10000, 3, 8)
    assert qi["maxdims"] == (unlimited, 3) and qi["shape"] == (nq, 3)
    ti = f.info("fqt")
    assert ti["chunk"] == (10000 // nf, nf, 2, 8) and ti["maxdims"] == (unlimited, nf, 2)
    for n in ("fq0", "fq", "fq2"):
        assert f.info(n)["chunk"] == (10000, 2, 8)
    assert f.info("meta/rawconfig")["layout"] == "contiguous"
    got = f.read("fqt")
    assert np.array_equal(got[..., 0] + 1j * got[..., 1], fqt)


def test_signal_multilevel_chunk_index(tmp_path):
    # small chunks: 300 rows of qvectors in 75 chunks (two-level B-tree); fqt with NF above
    # the chunk size is chunked along frames too (1 x 4 x 2 chunks, 600 of them)
    rng = np.random.default_rng(2)
    nq, nf = 300, 5
    q = rng.normal(size=(nq, 3))
    fqt = rng.normal(size=(nq, nf)) + 1j * rng.normal(size=(nq, nf))
    fq = rng.normal(size=nq) + 1j * rng.normal(size=nq)
    path = str(tmp_path / "m.h5")
    abi.write_signal(path, q, fqt, fqt[:, 0], fq, fq, chunksize=4)
    f = h5lite.File(path)
    assert np.array_equal(f.read("qvectors"), q)
    assert f.tree_depth == 2
    got = f.read("fqt")
    assert f.info("fqt")["chunk"] == (1, 4, 2, 8) and f.tree_depth == 2
    assert np.array_equal(got[..., 0] + 1j * got[..., 1], fqt)
    d = abi.read_signal(path)
    assert np.array_equal(d["fqt"], fqt) and np.array_equal(d["fq"], fq)
    # zero rows: no chunk index at all
    empty = str(tmp_path / "e.h5")
    abi.write_signal(empty, np.zeros((0, 3)), np.zeros((0, nf), complex), np.zeros(0, complex),
                     np.zeros(0, complex), np.zeros(0, complex))
    assert h5lite.File(empty).read("fqt").shape == (0, nf, 2)
    assert abi.read_signal(empty)["qvectors"].shape == (0, 3)


def test_signal_optional_datasets(tmp_path):
    path = str(tmp_path / "s.h5")
    abi.write_signal(path, np.ones((2, 3)), fqt=None, fq0=None, fq=np.array([1 + 2j, 3]),
                     fq2=None)
    f = h5lite.File(path)
    assert sorted(f.root) == ["fq", "meta", "qvectors"]
    d = abi.read_signal(path)
    assert "fqt" not in d and np.allclose(d["fq"], [1 + 2j, 3])


def test_signal_reader_rejects_non_hdf5(tmp_path):
    p = tmp_path / "x.h5"
    p.write_bytes(b"not an hdf5 file" * 10)
    with pytest.raises(RuntimeError):
        abi.read_signal(str(p))


# ---- configuration, sample, staging ---------------------------------------------------------
@pytest.fixture
def small_files(tmp_path):
    w = synth.small("all", "autocorrelate", seed=21, na=23, nf=9, nq=3, nm=4)
    w.class_factors[:] = w.class_factors[:1]  # database type-0 constants
    cfg = synth.write_files(str(tmp_path / "run"), w)
    return w, cfg


def test_dry_run_matches_workload(small_files, tmp_path):
    w, cfg = small_files
    d = dry(cfg, tmp_path)
    assert d["nf"] == w.nf and d["na"] == w.na
    assert np.allclose(np.array(d["qvectors"])[:, 0], w.shells, rtol=0, atol=0)
    # orientations from a file are normalised (parameters.cpp:932-943)
    assert np.allclose(d["orientations"], w.directions, atol=1e-15)
    assert np.allclose(d["subvectors_q0"], w.shells[0] * w.directions, atol=1e-15)
    labels = d["class_labels"]
    cls = np.array(d["atom_class"])
    assert [labels[c] for c in cls] == [w.class_names[c] for c in w.atom_class]
    cf = np.array(d["class_factors"])
    order = [w.class_names.index(l) for l in labels]
    assert np.allclose(cf, w.class_factors[0][order][None, :].repeat(w.nq, 0))
    # DCD written in the reference's layout reads back bit-exactly (float32 staging)
    assert d["coord_sum"] == pytest.approx(float(w.coords.astype(np.float64).sum()), rel=1e-12)


def test_scans_follow_reference(tmp_path):
    w = synth.small("all", seed=2, na=5, nf=3, nq=1, nm=1)
    cfg = synth.write_files(str(tmp_path / "s"), w)
    txt = open(cfg).read().replace(
        "<vectors><type>file</type><file>qvectors.txt</file></vectors>",
        "<vectors><type>scans</type><scans><scan><base><x>0.3</x><y>0.4</y><z>1.2</z></base>"
        "<from>0.1</from><to>2.0</to><points>17</points><exponent>1.7</exponent></scan>"
        "</scans></vectors>")
    open(cfg, "w").write(txt)
    q = abi.config_qvectors(cfg)
    ref = oracle.scan([0.3, 0.4, 1.2], 0.1, 2.0, 17, 1.7)
    assert np.array_equal(q, ref)  # float powf reproduced bit for bit


def test_type2_form_factors_and_background(tmp_path):
    rng = np.random.default_rng(3)
    w = synth.small("all", "square", seed=4, na=11, nf=2, nq=4, nm=2)
    params = synth.xray_form_factor_params(rng, len(w.class_names))
    cfg = synth.write_files(str(tmp_path / "x"), w, sfactor_params=params)
    d = dry(cfg, tmp_path)
    labels = d["class_labels"]
    cf = np.array(d["class_factors"])
    for i, q in enumerate(w.shells):
        for c, l in enumerate(labels):
            v = params[w.class_names.index(l)]
            assert cf[i, c] == pytest.approx(oracle.sfactor(2, v, q), rel=1e-15)


def test_frameset_first_last_stride_clones(small_files, tmp_path):
    w, cfg = small_files
    txt = open(cfg).read().replace(
        "<frameset><file>sample.dcd</file><format>dcd</format></frameset>",
        "<frameset><file>sample.dcd</file><format>dcd</format><first>1</first><last>7</last>"
        "<stride>2</stride><clones>2</clones></frameset>")
    open(cfg, "w").write(txt)
    d = dry(cfg, tmp_path)
    # trim_index keeps i >= first, i <= last and i % stride == 0 (absolute index)
    keep = [i for i in range(w.nf) if i >= 1 and i <= 7 and i % 2 == 0]
    assert d["nf"] == 2 * len(keep)
    expect = 2 * w.coords[keep].astype(np.float64).sum()
    assert d["coord_sum"] == pytest.approx(expect, rel=1e-12)


def test_target_selection_range(small_files, tmp_path):
    w, cfg = small_files
    txt = open(cfg).read().replace(
        "</sample>",
        "<selections><selection><type>range</type><name>part</name><from>3</from><to>9</to>"
        "</selection></selections></sample><stager><target>part</target></stager>")
    open(cfg, "w").write(txt)
    d = dry(cfg, tmp_path)
    assert d["na"] == 7
    assert d["coord_sum"] == pytest.approx(float(w.coords[:, 3:10].astype(np.float64).sum()),
                                           rel=1e-12)


@pytest.mark.parametrize("edit,needle", [
    (("<type>autocorrelate</type>", "<type>bogus</type>"), "DSP type not understood"),
    (("sample.dcd</file>", "missing.dcd</file>"), "DCD"),
    (("<file>db.xml</file>", "<file>nodb.xml</file>"), "does not exist"),
    (("<type>vectors</type>", "<type>multipole</type>"), "multipole"),
])
def test_driver_errors(small_files, tmp_path, edit, needle):
    w, cfg = small_files
    txt = open(cfg).read().replace(*edit)
    open(cfg, "w").write(txt)
    r = run_driver("--config", cfg, "--dry-run", str(tmp_path / "o.json"))
    assert r.returncode == 1
    assert needle in r.stderr


def test_dcd_atom_count_mismatch(small_files, tmp_path):
    w, cfg = small_files
    synth.write_dcd(os.path.join(os.path.dirname(cfg), "sample.dcd"), w.coords[:, :-1])
    r = run_driver("--config", cfg, "--dry-run", str(tmp_path / "o.json"))
    assert r.returncode == 1 and "Atom number mismatch" in r.stderr


def test_truncated_dcd(small_files, tmp_path):
    w, cfg = small_files
    p = os.path.join(os.path.dirname(cfg), "sample.dcd")
    data = open(p, "rb").read()
    open(p, "wb").write(data[:-20])
    r = run_driver("--config", cfg, "--dry-run", str(tmp_path / "o.json"))
    assert r.returncode == 1 and "truncated" in r.stderr


def test_command_line_overrides(small_files, tmp_path):
    w, cfg = small_files
    d = dry(cfg, tmp_path, "--scattering.signal.file=other.h5", "--gpu.precision", "fp32")
    assert d["signal"].endswith("other.h5") and d["precision"] == "fp32"
    r = run_driver("--config", cfg, "--dry-run", str(tmp_path / "o.json"), "--no.such=1")
    assert r.returncode == 1 and "unknown option" in r.stderr


def multipole_xml(kind, moments_type="resolution", resolution=3, extra=""):
    return ("<average><orientation><type>multipole</type><multipole><type>%s</type><moments>"
            "<type>%s</type><resolution>%d</resolution><file>moments.txt</file></moments>"
            "</multipole>%s</orientation></average>" % (kind, moments_type, resolution, extra))


def test_multipole_moments_from_configuration(small_files, tmp_path):
    w, _ = small_files
    d = str(tmp_path / "mp")
    cfg = synth.write_files(d, w, average=multipole_xml("sphere", resolution=3))
    j = dry(cfg, tmp_path)
    assert j["orientation"] == "multipole" and j["multipole"] == "sphere"
    assert [tuple(m) for m in j["moments"]] == oracle.sphere_moments(3)
    cfg = synth.write_files(d, w, average=multipole_xml("cylinder", resolution=2))
    assert [tuple(m) for m in dry(cfg, tmp_path)["moments"]] == oracle.cylinder_moments(2)
    with open(os.path.join(d, "moments.txt"), "w") as f:
        f.write("0 0\n4 -3\n2 1\n")
    cfg = synth.write_files(d, w, average=multipole_xml("sphere", moments_type="file"))
    assert [tuple(m) for m in dry(cfg, tmp_path)["moments"]] == [(0, 0), (4, -3), (2, 1)]


@pytest.mark.parametrize("kind,lines,needle", [
    ("sphere", "2 3\n", "between -Major and +Major"),
    ("cylinder", "1 4\n", "between 0 and 3"),
    ("cylinder", "0 2\n", "must be 0 for Major 0"),
    ("sphere", "-1 0\n", "must be >= 0"),
])
def test_multipole_moment_checks(small_files, tmp_path, kind, lines, needle):
    d = str(tmp_path / "mp")
    cfg = synth.write_files(d, small_files[0], average=multipole_xml(kind, moments_type="file"))
    with open(os.path.join(d, "moments.txt"), "w") as f:
        f.write(lines)
    r = run_driver("--config", cfg, "--dry-run", str(tmp_path / "x.json"))
    assert r.returncode != 0 and needle in r.stderr, r.stderr


def test_stager_dump_writes_the_reference_dcd_layout(small_files, tmp_path):
    # stager.dump (data_stager.cpp:91-94): the staged frames as a DCD laid out like the
    # reference's DCDCoordinateWriter; without alignments the dry run stages on the host
    w, _ = small_files
    d = str(tmp_path / "dump")
    cfg = synth.write_files(d, w, extra="<stager><dump>true</dump><file>out.dcd</file></stager>")
    dry(cfg, tmp_path)
    ref = str(tmp_path / "ref.dcd")
    synth.write_dcd(ref, w.coords)
    assert open(os.path.join(d, "out.dcd"), "rb").read() == open(ref, "rb").read()
    # and the driver reads it back as a trajectory
    cfg2 = synth.write_files(str(tmp_path / "again"), w)
    import shutil
    shutil.copy(os.path.join(d, "out.dcd"), str(tmp_path / "again" / "sample.dcd"))
    j = dry(cfg2, tmp_path)
    assert j["coord_sum"] == pytest.approx(float(np.sum(w.coords, dtype=np.float64)), rel=0, abs=1e-6)


def test_stager_dump_unknown_format(small_files, tmp_path):
    w, _ = small_files
    cfg = synth.write_files(str(tmp_path / "x"), w, extra="<stager><mode>columns</mode></stager>")
    r = run_driver("--config", cfg, "--dry-run", str(tmp_path / "x.json"))
    assert r.returncode != 0 and "stager.mode" in r.stderr


def test_file_selections_ndx_and_pdb(small_files, tmp_path):
    # selection type "file" (parameters.cpp:148-176, atomselection_reader.cpp:33-120)
    w, _ = small_files
    d = str(tmp_path / "sel")
    os.makedirs(d, exist_ok=True)
    with open(os.path.join(d, "index.ndx"), "w") as f:
        f.write("[ System ]\n" + " ".join(str(i + 1) for i in range(w.na)) + "\n")
        f.write("[ Core ]\n3 1 5\n7\n[Tail]\n2 4\n")
    beta = [1.0 if i % 3 == 0 else 0.0 for i in range(w.na)]
    with open(os.path.join(d, "flags.pdb"), "w") as f:
        for i in range(w.na):
            f.write("ATOM  %5d C1   MOL A   1    %8.3f%8.3f%8.3f  1.00%6.2f      SEG%d\n"
                    % (i + 1, 0, 0, 0, beta[i], i % 2))
    sels = ("<selections>"
            "<selection><type>file</type><format>ndx</format><file>index.ndx</file>"
            "<expression>Core|Tail\\]</expression></selection>"
            "<selection><type>file</type><name>flagged</name><file>flags.pdb</file></selection>"
            "<selection><type>file</type><name>seg1</name><file>flags.pdb</file><selector>segid</selector>"
            "<expression>SEG1</expression></selection>"
            "</selections>")
    for target, want in (("Core", [2, 0, 4, 6]), ("Tail]", [1, 3]),
                         ("flagged", [i for i in range(w.na) if i % 3 == 0]),
                         ("seg1", [i for i in range(w.na) if i % 2 == 1])):
        cfg = synth.write_files(d, w, sample_extra=sels, extra="<stager><target>%s</target></stager>" % target)
        j = dry(cfg, tmp_path)
        assert j["na"] == len(want), target
        assert j["coord_sum"] == pytest.approx(float(w.coords[:, want].astype(np.float64).sum()), abs=1e-6)
    # the System group does not match the expression, so it is not a selection
    cfg = synth.write_files(d, w, sample_extra=sels, extra="<stager><target>System</target></stager>")
    r = run_driver("--config", cfg, "--dry-run", str(tmp_path / "x.json"))
    assert r.returncode != 0 and "unknown selection" in r.stderr


def test_dcdlist_frameset(small_files, tmp_path):
    # frameset format dcdlist (frames.cpp:71-85): the listed files, each `clones` times
    w, _ = small_files
    d = str(tmp_path / "list")
    cfg = synth.write_files(d, w)
    a, b = os.path.join(d, "a.dcd"), os.path.join(d, "b.dcd")
    synth.write_dcd(a, w.coords[:4])
    synth.write_dcd(b, w.coords[4:])
    with open(os.path.join(d, "frames.list"), "w") as f:
        f.write("%s\n#%s\n%s\n" % (a, b, b))
    xml = open(cfg).read().replace(
        "<framesets><frameset><file>sample.dcd</file><format>dcd</format></frameset></framesets>",
        "<framesets><frameset><file>frames.list</file><format>dcdlist</format><clones>2</clones>"
        "</frameset></framesets>")
    open(cfg, "w").write(xml)
    j = dry(cfg, tmp_path)
    want = np.concatenate([w.coords[:4], w.coords[:4], w.coords[4:], w.coords[4:]])
    assert j["nf"] == len(want)
    assert j["coord_sum"] == pytest.approx(float(want.astype(np.float64).sum()), abs=1e-6)
