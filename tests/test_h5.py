"""HDF5 final-state files without libhdf5 (cil_cuda_gb300/csrc/cil_h5.cpp, include/cil_input.h).

The reader is pinned on the reference's own output: the final-state files its binary wrote
(`<name>.Last.h5`) hold SigmaCore, RHO, PR and Vel, whose FP32 values its `.Last.gsd` files
of the same runs hold too, as the diameter, charge, mass and velocity chunks (read with the GSD
reader pinned on the reference's gsd.c). The writer lays a file out as those files are laid
out, and INIT H5 (Input.cpp:610-726) restarts a run from one."""
import copy
import json
import os
import struct

import numpy as np
import pytest
from oracle.refdir import reference_path  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = reference_path()
SINGLE = os.path.join(ROOT, "tests", "golden", "input_single_element_2d.json")
TWO = os.path.join(ROOT, "tests", "golden", "input_two_element_2d.json")
RUNS = ("z0.001t3.16_v2", "cil")


@pytest.fixture(scope="module")
def G():
    import cil_cuda_gb300 as G
    G.lib()
    return G


@pytest.mark.parametrize("stem", RUNS)
def test_reader_matches_the_gsd_file_of_the_same_run(G, stem):
    h5, gsd = os.path.join(REF, stem + ".Last.h5"), os.path.join(REF, stem + ".Last.gsd")
    if not (os.path.exists(h5) and os.path.exists(gsd)):
        pytest.skip("reference outputs absent")
    from cil_cuda_gb300.gsd import GSDFile
    f = GSDFile(gsd)
    n = int(f.read(0, "particles/N")[0])
    R, S = G.h5_read(h5, "R"), G.h5_read(h5, "SigmaCore")
    assert R.shape == (n, 1, 2) and S.shape == (n, 1)
    f32 = lambda a: np.asarray(a).astype(np.float32).ravel()  # noqa: E731
    np.testing.assert_array_equal(f.read(0, "particles/diameter"), f32(S))
    np.testing.assert_array_equal(f.read(0, "particles/charge"), f32(G.h5_read(h5, "RHO")))
    np.testing.assert_array_equal(f.read(0, "particles/mass"), f32(G.h5_read(h5, "PR")))
    np.testing.assert_array_equal(f.read(0, "particles/velocity")[:, :2], G.h5_read(h5, "Vel").reshape(n, 2))
    box = f.read(0, "configuration/box")
    d = f.read(0, "particles/position")[:, :2].astype(np.float64) - (R.reshape(n, 2) - box[:2] / 2)
    assert np.abs(d).max() <= 4 * np.spacing(np.float32(box[0]))  # FP32(x - L/2) against FP32(x) - L/2
    assert np.all(G.h5_read(h5, "State") == 0) and G.h5_read(h5, "CpuTime").shape == (1,)


def random_state(rng, n, E, D):
    return dict(pos=rng.uniform(0, 50, size=(n, E, D)), sigma=rng.uniform(0.8, 1.2, size=(n, E)),
                vel=rng.normal(size=(n, E, D)), force=rng.normal(size=(n, E, D)), force_dis=rng.normal(size=(n, E, D)),
                force_ran=rng.normal(size=(n, E, D)), rho=rng.uniform(size=n), theta=rng.uniform(size=n),
                pressure=rng.normal(size=n), state=np.zeros(n, np.int32), t0=rng.integers(0, 10 ** 6, n), cpu_time=3.5)


@pytest.mark.parametrize("n,E,D", [(37, 1, 2), (500, 2, 3), (0, 1, 2)])
def test_writer_round_trip(G, tmp_path, n, E, D):
    rng = np.random.default_rng(n + E + D)
    st = random_state(rng, n, E, D)
    path = str(tmp_path / "x.Last.h5")
    G.h5_write_state(path, **st)
    f32 = lambda a: np.asarray(a, np.float64).astype(np.float32).astype(np.float64)  # noqa: E731
    for name, key in (("R", "pos"), ("Vel", "vel"), ("F", "force"), ("FD", "force_dis"), ("FR", "force_ran"),
                      ("SigmaCore", "sigma"), ("RHO", "rho"), ("Theta", "theta"), ("PR", "pressure")):
        a = G.h5_read(path, name)
        assert a.shape == np.shape(st[key]), name
        np.testing.assert_array_equal(a, f32(st[key]))
    np.testing.assert_array_equal(G.h5_read(path, "T0"), st["t0"])
    np.testing.assert_array_equal(G.h5_read(path, "CpuTime"), [3.5])


def header_layout(path):
    """Superblock fields and the object header message types of every dataset."""
    b = open(path, "rb").read()
    u = lambda f, o: struct.unpack_from("<" + f, b, o)  # noqa: E731
    sb = dict(version=b[8], sizes=(b[13], b[14]), k=u("HH", 16), root=u("Q", 64)[0], tree_heap=u("QQ", 80))
    tree, heap = sb["tree_heap"]
    hsize, _, hdata = u("QQQ", heap + 8)
    used = u("H", tree + 6)[0]
    msgs = {}
    for k in range(used):
        snod = u("Q", tree + 24 + (2 * k + 1) * 8)[0]
        for e in range(u("H", snod + 6)[0]):
            off, oh = u("QQ", snod + 8 + 40 * e)
            name = b[hdata + off:b.index(b"\0", hdata + off)].decode()
            p, end, types = oh + 16, oh + 16 + u("I", oh + 8)[0], []
            while p < end:
                t, s = u("HH", p)
                if t not in (0x00, 0x12):  # padding and the modification time
                    types.append(t)
                p += 8 + s
            msgs[name] = types
    return sb, msgs


def test_writer_lays_files_out_as_the_reference(G, tmp_path):
    ref = os.path.join(REF, "z0.001t3.16_v2.Last.h5")
    if not os.path.exists(ref):
        pytest.skip("reference outputs absent")
    path = str(tmp_path / "x.Last.h5")
    G.h5_write_state(path, **random_state(np.random.default_rng(1), 934, 1, 2))
    sa, ma = header_layout(ref)
    sb, mb = header_layout(path)
    assert sa == {**sb, "tree_heap": sa["tree_heap"]} and sa["tree_heap"][0] == sb["tree_heap"][0]
    assert ma == mb  # the same datasets, each with dataspace, datatype, fill value and layout


def h5_doc(path, how="ALL", rng=None, two=False):
    d = json.load(open(TWO if two else SINGLE))
    c = d["SPECIES"]["DEFINE"][0]
    h5 = {"SELECT": how, "LOCATION": [path, "R"], "ALL": [path, "R", "Vel", "State", "Theta", "RHO", "SigmaCore"]}
    if rng is not None:
        h5["RANGE"] = rng
    d["INIT"][c] = {"SELECT": "H5", "H5": h5}
    return d


def load(G, d):
    return G.RunInput(json.dumps(d), is_path=False)


def test_init_h5_all_restarts_the_cell_status(G, tmp_path):
    rng = np.random.default_rng(5)
    n = 64
    st = random_state(rng, n, 1, 2)
    st["pos"] = rng.uniform(0, 40.0, size=(n, 1, 2))  # the fixture's 40 x 40 box
    path = str(tmp_path / "restart.Last.h5")
    G.h5_write_state(path, **st)
    f32 = lambda a: np.asarray(a, np.float64).astype(np.float32).astype(np.float64)  # noqa: E731
    r = load(G, h5_doc(path))
    s = r.cycle_initial_state()
    np.testing.assert_array_equal(s["pos"], f32(st["pos"]).reshape(n, 2))
    np.testing.assert_array_equal(s["vel"], f32(st["vel"]).reshape(n, 2))
    np.testing.assert_array_equal(s["sigma"], f32(st["sigma"]).ravel())
    np.testing.assert_array_equal(s["sigma_t"], s["sigma"])
    np.testing.assert_array_equal(s["theta"], f32(st["theta"]))
    np.testing.assert_array_equal(s["rho"], f32(st["rho"]))
    assert np.all(s["angvel"] > 0)  # the cycle speeds stay those initializeCellStatus draws
    # LOCATION: positions only; the status is the drawn one
    s2 = load(G, h5_doc(path, "LOCATION")).cycle_initial_state()
    np.testing.assert_array_equal(s2["pos"], s["pos"])
    assert np.all(s2["rho"] == 1.0) and np.all(s2["vel"] == 0.0)
    np.testing.assert_array_equal(s2["angvel"], s["angvel"])
    # RANGE [first, end), negative values from the end
    s3 = load(G, h5_doc(path, rng=[10, -4])).cycle_initial_state()
    np.testing.assert_array_equal(s3["pos"], s["pos"][10:n - 4])
    np.testing.assert_array_equal(s3["theta"], s["theta"][10:n - 4])


def test_init_h5_two_element(G, tmp_path):
    rng = np.random.default_rng(6)
    n = 30
    st = random_state(rng, n, 2, 2)
    st["pos"] = rng.uniform(0, 60.0, size=(n, 2, 2))
    path = str(tmp_path / "two.Last.h5")
    G.h5_write_state(path, **st)
    s = load(G, h5_doc(path, two=True)).initial_state()
    np.testing.assert_array_equal(s["pos"], st["pos"].astype(np.float32).astype(np.float64))
    np.testing.assert_array_equal(s["sigma"], st["sigma"].astype(np.float32).astype(np.float64))


def test_init_h5_refusals(G, tmp_path):
    rng = np.random.default_rng(7)
    st = random_state(rng, 20, 1, 2)
    st["pos"] = rng.uniform(0, 40.0, size=(20, 1, 2))
    path = str(tmp_path / "r.Last.h5")
    G.h5_write_state(path, **st)
    for edit, needle in (
            (lambda d: d["INIT"]["C1"]["H5"].update(RANGE=[5, 5]), "Range is empty"),
            (lambda d: d["INIT"]["C1"]["H5"].update(RANGE=[0, 21]), "Range out of bounds"),
            (lambda d: d["INIT"]["C1"]["H5"]["ALL"].__setitem__(2, "Nope"), "no object Nope"),
            (lambda d: d["INIT"]["C1"]["H5"]["ALL"].__setitem__(5, "Vel"), "Inconsistent H5"),
            (lambda d: d["INIT"]["C1"]["H5"].update(ALL=[path, "R"]), "vector should be of size 7")):
        d = copy.deepcopy(h5_doc(path))
        edit(d)
        with pytest.raises(G.CilError) as e:
            load(G, d).cycle_initial_state()
        assert needle in str(e.value), (needle, str(e.value))
    st["state"][3] = 1  # a crawling cell
    G.h5_write_state(path, **st)
    with pytest.raises(G.CilError) as e:
        load(G, h5_doc(path)).cycle_initial_state()
    assert "dividing state" in str(e.value)
    open(path, "wb").write(b"not an hdf5 file at all")
    with pytest.raises(G.CilError) as e:
        load(G, h5_doc(path))
    assert "not an HDF5 file" in str(e.value)


@pytest.mark.parametrize("stem,L", [("cil", 640.0), ("z0.001t3.16_v2", 100.0)])
def test_init_h5_from_the_reference_file(G, stem, L):
    """The reference's own final-state file as INIT H5 ALL, as its restart reads it. In
    z0.001t3.16_v2.Last.h5 one cell sits at x = 100.0 = L: its position just below L rounded up
    when it was stored as FP32, and the reference's restart stops on it ("Input Positions Out of
    Bounds!", the isValidPos check of CIL.cuh:52-66), as this one does."""
    h5 = os.path.join(REF, stem + ".Last.h5")
    if not os.path.exists(h5):
        pytest.skip("reference outputs absent")
    R = G.h5_read(h5, "R")
    n = R.shape[0]
    d = h5_doc(h5)
    d["MD"]["BOX"] = [L, L]
    if np.any(R >= L):
        with pytest.raises(G.CilError) as e:
            load(G, d).cycle_initial_state()
        assert "Out of Bounds" in str(e.value)
        return
    s = load(G, d).cycle_initial_state()
    np.testing.assert_array_equal(s["pos"], R.reshape(n, 2))
    np.testing.assert_array_equal(s["rho"], G.h5_read(h5, "RHO"))
    np.testing.assert_array_equal(s["vel"], G.h5_read(h5, "Vel").reshape(n, 2))


def test_reader_follows_deeper_trees_and_continuations(G, tmp_path):
    """Forms libhdf5 writes for larger files, built here by rewriting a written file: the
    root group's B-tree under a level-1 node, and a dataset whose object header continues in a
    second block (continuation message)."""
    path = str(tmp_path / "x.Last.h5")
    st = random_state(np.random.default_rng(3), 50, 1, 2)
    G.h5_write_state(path, **st)
    b = bytearray(open(path, "rb").read())
    u = lambda f, o: struct.unpack_from("<" + f, b, o)  # noqa: E731
    tree, heap = u("QQ", 80)
    used = u("H", tree + 6)[0]
    last_key = u("Q", tree + 24 + 16 * used)[0]
    # a level-1 node whose one child is the original level-0 node
    top = len(b)
    node = bytearray(b"TREE") + bytes([0, 1]) + struct.pack("<H", 1) + struct.pack("<qq", -1, -1)
    node += struct.pack("<QQQ", 0, tree, last_key)
    b += node + bytes(24 + 33 * 8 + 32 * 8 - len(node))
    struct.pack_into("<Q", b, 80, top)  # the superblock's cached B-tree address
    root = u("Q", 64)[0]
    struct.pack_into("<Q", b, root + 16 + 8, top)  # the root's symbol table message
    # move the messages of dataset "R" after its dataspace into a continuation block
    names = {}
    for k in range(used):
        snod = u("Q", tree + 24 + 16 * k + 8)[0]
        for e in range(u("H", snod + 6)[0]):
            off, oh = u("QQ", snod + 8 + 40 * e)
            names[bytes(b[u("Q", heap + 24)[0] + off:]).split(b"\0")[0].decode()] = oh
    oh = names["R"]
    hsize = u("I", oh + 8)[0]
    p = oh + 16
    first = 8 + u("HH", p)[1]  # the dataspace message, kept
    rest = bytes(b[p + first:p + hsize])
    cont = len(b) + (-len(b)) % 8
    b += bytes(cont - len(b)) + rest
    nmsg = u("H", oh + 2)[0]
    # the freed space: a continuation message, then a NIL message padding to the old size
    cmsg = struct.pack("<HHB3x", 0x10, 16, 0) + struct.pack("<QQ", cont, len(rest))
    pad = hsize - first - len(cmsg)
    nil = struct.pack("<HHB3x", 0, pad - 8, 0) + bytes(pad - 8)
    b[p + first:p + hsize] = cmsg + nil
    struct.pack_into("<H", b, oh + 2, nmsg + 2)
    open(path, "wb").write(bytes(b))
    f32 = lambda a: np.asarray(a, np.float64).astype(np.float32).astype(np.float64)  # noqa: E731
    np.testing.assert_array_equal(G.h5_read(path, "R"), f32(st["pos"]))
    np.testing.assert_array_equal(G.h5_read(path, "/RHO"), f32(st["rho"]))
    np.testing.assert_array_equal(G.h5_read(path, "T0"), st["t0"])
    with pytest.raises(G.CilError) as e:
        G.h5_read(path, "Missing")
    assert "no object Missing" in str(e.value)


def test_reader_refuses_malformed_files(G, tmp_path):
    path = str(tmp_path / "x.Last.h5")
    G.h5_write_state(path, **random_state(np.random.default_rng(4), 10, 1, 2))
    good = open(path, "rb").read()
    for cut, name in ((40, "R"), (200, "R"), (700, "R"), (len(good) - 10, "Vel")):  # Vel's data is written last
        open(path, "wb").write(good[:cut])
        with pytest.raises(G.CilError):
            G.h5_read(path, name)
    open(path, "wb").write(good[:len(good) - 10])
    assert G.h5_read(path, "R").shape == (10, 1, 2)  # the datasets before the cut stay readable
    b = bytearray(good)
    b[8] = 2  # superblock version 2
    open(path, "wb").write(bytes(b))
    with pytest.raises(G.CilError) as e:
        G.h5_read(path, "R")
    assert "superblock version 2" in str(e.value)


def test_frame_file_round_trip(G, tmp_path):
    """The frame file (initHDF5Output / outputHDF5Frame): /params attributes dt, L, Tdump; per
    frame /snapshots/t_<frame> with the datasets and the attribute ts, as the reference's
    analysis (cil.py: f["snapshots/"], .get('R'), attrs['ts'][0], f["/params"].attrs['dt'][0])
    reads them; frames of different sizes, 3D, and more frames than one symbol node holds."""
    path = str(tmp_path / "run.h5")
    w = G.H5Frames(path, box=[12.0, 13.0, 14.0], dt=1e-4, gts=200)
    states = []
    rng = np.random.default_rng(9)
    for k in range(20):
        st = random_state(rng, 5 + 3 * k, 1, 3)
        states.append(st)
        w.write(k, 200 * k, **st)
    w.close()
    np.testing.assert_array_equal(G.h5_attr(path, "params", "dt"), [1e-4])
    np.testing.assert_array_equal(G.h5_attr(path, "/params", "L"), [12.0, 13.0, 14.0])
    np.testing.assert_array_equal(G.h5_attr(path, "params", "Tdump"), [200])
    f32 = lambda a: np.asarray(a, np.float64).astype(np.float32).astype(np.float64)  # noqa: E731
    for k in (0, 7, 19):
        g = "snapshots/t_%d/" % k
        np.testing.assert_array_equal(G.h5_attr(path, "snapshots/t_%d" % k, "ts"), [200 * k])
        np.testing.assert_array_equal(G.h5_read(path, g + "R"), f32(states[k]["pos"]))
        np.testing.assert_array_equal(G.h5_read(path, g + "F"), f32(states[k]["force"]))
        np.testing.assert_array_equal(G.h5_read(path, g + "T0"), states[k]["t0"])
        np.testing.assert_array_equal(G.h5_read(path, g + "CpuTime"), [3.5])
    # an empty run still has its groups
    p2 = str(tmp_path / "empty.h5")
    G.H5Frames(p2, box=[5.0, 5.0], dt=0.1, gts=1).close()
    np.testing.assert_array_equal(G.h5_attr(p2, "params", "L"), [5.0, 5.0])
    with pytest.raises(G.CilError):
        G.h5_read(p2, "snapshots/t_0/R")


def test_frame_file_with_many_frames(G, tmp_path):
    """300 snapshots: more entries than a group B-tree node of K 16 holds (256), so the file's K
    grows to hold them in one node."""
    path = str(tmp_path / "long.h5")
    w = G.H5Frames(path, box=[5.0, 5.0], dt=0.1, gts=1)
    for k in range(300):
        w.write(k, k, pos=np.full((1, 1, 2), 0.01 * k), sigma=np.ones((1, 1)))
    w.close()
    for k in (0, 150, 299):
        np.testing.assert_array_equal(G.h5_attr(path, "snapshots/t_%d" % k, "ts"), [k])
        assert G.h5_read(path, "snapshots/t_%d/R" % k)[0, 0, 0] == np.float32(0.01 * k)
