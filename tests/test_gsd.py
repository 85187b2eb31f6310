"""GSD 1.0 frame files (include/cil_gsd.h): the library's file writer against the reference's
vendored gsd.c (byte-identical files for the same chunk sequence; golden file written by
tests/golden/make_gsd_golden.py), gsd.c reading the library's files, and the numpy reader
(cil_cuda_gb300/gsd.py) against gsd.c on the golden file and on the reference's own
shipped outputs. No GPU: the file layer makes no CUDA call."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, GOLDEN)

import gsd_sequence  # noqa: E402
from cil_cuda_gb300.gsd import GSDFile  # noqa: E402
from oracle import ref_gsd  # noqa: E402
from oracle.refdir import reference_path  # noqa: E402

REF_DIR = reference_path()
REF_OUTPUTS = ["cil.Last.gsd", "z0.001t3.16_v2.Last.gsd"]  # final-state files shipped with the reference


@pytest.fixture(scope="module")
def G():
    import cil_cuda_gb300 as G
    if not os.path.exists(G.LIB_PATH):
        from cil_cuda_gb300 import build
        build.build()
    G.lib()
    return G


@pytest.fixture(scope="module")
def ref():
    if not ref_gsd.available():
        import subprocess
        subprocess.run(["bash", os.path.join(ROOT, "oracle", "ref_build.sh")], check=False)
    if not ref_gsd.available():
        pytest.skip("reference gsd.c not built (reference tree absent)")
    return ref_gsd


def write_ours(G, path, seq, **kw):
    with G.GSDWriter(path, **kw) as w:
        for fr in seq:
            for name, typ, arr in fr:
                w.write_chunk(name, arr, typ)
            w.end_frame()
        assert w.nframes == len(seq)


def random_sequence(seed, nframes=30):
    rng = np.random.default_rng(seed)
    out = []
    for f in range(nframes):
        fr = []
        for k in range(int(rng.integers(1, 12))):
            typ = int(rng.integers(1, 11))
            n, m = int(rng.integers(1, 5000)), int(rng.integers(1, 4))
            a = rng.integers(0, 120, size=(n, m)).astype(gsd_sequence.TYPES[typ])
            fr.append((f"c{k}/t{typ}", typ, a))
        out.append(fr)
    return out


def test_writer_reproduces_golden_file_of_reference_gsd_c(G, tmp_path):
    p = str(tmp_path / "ours.gsd")
    write_ours(G, p, gsd_sequence.frames())
    ours = open(p, "rb").read()
    gold = open(os.path.join(GOLDEN, "gsd_ref_sequence.gsd"), "rb").read()
    assert len(ours) == len(gold)
    assert ours == gold
    f = GSDFile(p)
    assert f.header["index_allocated_entries"] == 512  # moved twice: 128 -> 256 -> 512
    assert len(f.names) == 128  # name list full; later names carry id 65535


@pytest.mark.parametrize("seed", [1, 2])
def test_writer_matches_reference_on_random_sequences(G, ref, tmp_path, seed):
    seq = random_sequence(seed)
    a, b = str(tmp_path / "ours.gsd"), str(tmp_path / "ref.gsd")
    write_ours(G, a, seq, application="app", schema="schema", schema_version=(3, 7))
    ref.write_sequence(b, seq, application="app", schema="schema", schema_version=(3, 7))
    assert open(a, "rb").read() == open(b, "rb").read()


def test_reference_reader_reads_library_file(G, ref, tmp_path):
    seq = gsd_sequence.frames()
    p = str(tmp_path / "ours.gsd")
    write_ours(G, p, seq)
    names = gsd_sequence.names(seq)
    got, nf = ref.read_all(p, names)
    assert nf == len(seq)
    stored = set(GSDFile(p).names)
    assert "many/110" in stored and "many/111" not in stored
    checked = 0
    for f, fr in enumerate(seq):
        for name, typ, arr in fr:
            key = (f, name)
            if name == gsd_sequence.LONG_NAME or name not in stored:
                assert key not in got  # gsd.c finds neither a truncated name nor one beyond the name list
                continue
            a = np.asarray(arr)
            exp = a.reshape(-1) if a.ndim < 2 or a.shape[1] == 1 else a
            np.testing.assert_array_equal(got[key], exp)
            assert got[key].dtype == exp.dtype
            checked += 1
    assert checked > 300


def test_numpy_reader_agrees_with_reference_reader(ref):
    p = os.path.join(GOLDEN, "gsd_ref_sequence.gsd")
    seq = gsd_sequence.frames()
    names = gsd_sequence.names(seq)
    got, nf = ref.read_all(p, names)
    f = GSDFile(p)
    assert f.nframes == nf == len(seq)
    for (fr, name), a in got.items():
        b = f.read(fr, name)
        np.testing.assert_array_equal(b, a)
        assert b.dtype == a.dtype
    # and nothing the reference cannot find is found
    for fr in range(nf):
        for name in names:
            if (fr, name) not in got:
                assert f.find(fr, name) is None


@pytest.mark.parametrize("name", REF_OUTPUTS)
def test_numpy_reader_reads_reference_outputs(ref, name):
    p = os.path.join(REF_DIR, name)
    if not os.path.exists(p):
        pytest.skip("reference outputs absent")
    f = GSDFile(p)
    names = f.names
    got, nf = ref.read_all(p, names)
    assert f.nframes == nf >= 1
    for (fr, nm), a in got.items():
        np.testing.assert_array_equal(f.read(fr, nm), a)
    # the chunk set and order outputGSDFrame writes (OutputWriter.cpp:505-644)
    assert f.chunk_names(0) == ["configuration/step", "configuration/dimensions", "configuration/box",
                                "particles/N", "particles/types", "particles/Z", "particles/diameter",
                                "particles/typeid", "particles/charge", "particles/position",
                                "particles/velocity", "particles/mass"]
    n = int(f.read(0, "particles/N")[0])
    assert f.read(0, "particles/position").shape == (n, 3)
    assert int(f.read(0, "configuration/dimensions")[0]) == 3
    assert (f.application, f.schema, f.schema_version) == ("CIL", "hoomd", (1 << 16) | 1)
    z = f.read(0, "particles/position")[:, 2]
    assert np.all(z.view(np.uint32) == np.float32(-0.0).view(np.uint32))  # single-element cells: zhack[0]


def test_unended_frame_stays_out_of_the_index(G, ref, tmp_path):
    p = str(tmp_path / "partial.gsd")
    w = G.GSDWriter(p)
    w.write_chunk("a", np.arange(4, dtype=np.int32))
    w.end_frame()
    w.write_chunk("a", np.arange(5, dtype=np.int32))  # never ended
    w.close()
    f = GSDFile(p)
    assert f.nframes == 1
    np.testing.assert_array_equal(f.read(0, "a"), np.arange(4))
    _, nf = ref.read_all(p, ["a"])
    assert nf == 1


def test_bad_chunks_and_paths_are_errors(G, tmp_path):
    w = G.GSDWriter(str(tmp_path / "x.gsd"))
    with pytest.raises(G.CilError) as e:
        w.write_chunk("empty", np.zeros(0, np.float32))
    assert e.value.status == 1  # CIL_ERR_CONFIG, as gsd.c's -2
    with pytest.raises(G.CilError):
        w.write_chunk("badtype", np.zeros(3, np.float32), 11)
    w.close()
    with pytest.raises(G.CilError) as e:
        G.GSDWriter(str(tmp_path / "no" / "such" / "dir.gsd"))
    assert e.value.status == 8  # CIL_ERR_IO


def test_reader_rejects_non_gsd(tmp_path):
    p = tmp_path / "bad.gsd"
    p.write_bytes(b"\0" * 512)
    with pytest.raises(ValueError):
        GSDFile(str(p))
