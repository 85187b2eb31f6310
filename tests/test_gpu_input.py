"""A run started from the reference's JSON run description (include/cil_input.h): the Engine
built from it steps like the oracle with the same parameters and INIT (oracle mode: the
reference's host draws, FP64), and the reference-shaped runner cil_gpu_run (JSON -> GPU step
-> GSD frames) writes the frames and the final-state file of that same run."""
import json
import os
import subprocess

import numpy as np
import pytest

from cil_cuda_gb300.gsd import GSDFile

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FIXTURE = os.path.join(ROOT, "tests", "golden", "input_two_element_2d.json")


def sc_document():
    """The fixture with INTERACTIONS SELECT SC read as the reference's cubic well (no
    GPU.FORCE_LAW): xi = 0.3, Em = 0.5, E0 = 5; dt = 1e-4 for the stiff well."""
    d = json.load(open(FIXTURE))
    del d["GPU"]["FORCE_LAW"]
    d["SPECIES"]["A"]["PAIRFORCES"]["SC"].update(SIGMA_RATIO=[0.3, 0.3 / 0.9], EPSILON_RATIO=[0.1, 0.1])
    d["MD"]["DT"]["MANUAL"] = 1e-4
    return json.dumps(d)


def machine_document():
    """The fixture's dividing cells with the reference's own bond and crawling/dividing states (no
    GPU.SPRING): R0, Rmin and the growth activities added, as the reference requires them."""
    d = json.load(open(FIXTURE))
    del d["GPU"]["SPRING"]
    del d["GPU"]["RNG"]
    d["SPECIES"]["A"]["DIVISION"].update(R0=0.25, Rmin=1.05, Rmin_RATIO=0.0, SWELLING=False)
    d["SPECIES"]["A"].update(GROWTHK0=[0.0, 0.0], GROWTHK1=[1.0, 1.0], GROWTHK2=[0.0, 0.0])
    d["SPECIES"]["A"]["FENE"]["RMAX_DIVISION"] = [1.6]
    return json.dumps(d)


@pytest.mark.parametrize("law", ["softcore", "sc", "machine"])
def test_run_from_json_matches_oracle(gpu_lib, oracle_lib, law):
    G = gpu_lib
    docs = {"softcore": None, "sc": sc_document, "machine": machine_document}
    r = G.RunInput(FIXTURE) if law == "softcore" else G.RunInput(docs[law](), is_path=False)
    assert r.params["force_law"] == (G.FORCE_SC if law == "sc" else G.FORCE_SOFTCORE)
    st = r.initial_state()
    eng = r.engine()
    eng.upload(0, **st)
    steps = r.run["gts"] * r.run["frames"]
    eng.step(steps)
    g = eng.download(0)
    eng.close()
    o = oracle_lib.Oracle(r.params, r.run["capacity"], r.config["seed"])
    o.set_state(**st)
    assert o.step(steps) == 0
    s = o.state()
    assert g["ncells"] == len(s["sigma"]) and (law == "sc" or g["ncells"] != r.run["ncells"])
    np.testing.assert_array_equal(g["tswitch"], s["tswitch"])
    if law == "machine":
        np.testing.assert_array_equal(g["cell_state"], s["cell_state"])
    d = g["pos"] - s["pos"]
    d -= np.round(d / 60.0) * 60.0
    assert np.abs(d).max() <= 1e-9


def test_runner_writes_the_run(gpu_lib, tmp_path):
    G = gpu_lib
    from cil_cuda_gb300 import build
    assert os.path.exists(build.RUNNER)
    doc = json.load(open(FIXTURE))
    doc["OUTPUT"]["DIR"] = str(tmp_path / "out")
    cfg = tmp_path / "run.json"
    cfg.write_text(json.dumps(doc))
    res = subprocess.run([build.RUNNER, str(cfg)], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr
    lines = [ln for ln in res.stderr.splitlines() if ln.startswith("# ts =")]
    assert len(lines) == doc["MD"]["FRAMES"]
    f = GSDFile(str(tmp_path / "out" / "colony.gsd"))
    assert f.nframes == doc["MD"]["FRAMES"] + 1
    gts = doc["MD"]["GTS"]
    assert [int(f.read(k, "configuration/step")[0]) for k in range(f.nframes)] == [k * gts for k in range(f.nframes)]
    assert f.types(0) == ["A_BACK", "A_FRONT"]
    # the same run through the Python binding gives the same final frame
    r = G.RunInput(str(cfg))
    eng = r.engine()
    eng.upload(0, **r.initial_state())
    eng.step(gts * doc["MD"]["FRAMES"])
    g = eng.download(0)
    eng.close()
    E = 2 * g["ncells"]
    assert int(f.read(f.nframes - 1, "particles/N")[0]) == E
    exp = (g["pos"].reshape(E, 2) - 30.0).astype(np.float32)
    np.testing.assert_array_equal(f.read(f.nframes - 1, "particles/position")[:, :2], exp)
    last = GSDFile(str(tmp_path / "out" / "Last" / "colony.Last.gsd"))
    assert last.nframes == 1 and int(last.read(0, "configuration/step")[0]) == 0
    np.testing.assert_array_equal(last.read(0, "particles/position"), f.read(f.nframes - 1, "particles/position"))


SINGLE = os.path.join(ROOT, "tests", "golden", "input_single_element_2d.json")
REFERENCE_FRAME_CHUNKS = ["configuration/step", "configuration/dimensions", "configuration/box", "particles/N",
                          "particles/types", "particles/Z", "particles/diameter", "particles/typeid",
                          "particles/charge", "particles/position", "particles/velocity", "particles/mass"]


@pytest.mark.parametrize("integrator", ["EULER", "DPD"])
def test_runner_single_element_run(gpu_lib, tmp_path, integrator):
    """A single-element run (the shipped configurations' model) through cil_gpu_run: frames of
    the cell-cycle model with the chunks of the reference's own final-state files, equal to the
    same run through the Python binding; with the Euler step and with DPD."""
    G = gpu_lib
    from cil_cuda_gb300 import build
    doc = json.load(open(SINGLE))
    doc["OUTPUT"]["DIR"] = str(tmp_path / "out")
    if integrator == "DPD":
        doc["MD"]["INTEGRATOR"] = {"SELECT": "DPD", "DPD": {"DISSAMCEL": 0.0, "DISDIFCEL": 2.0, "DISBG": 0.5}}
        doc["MD"]["KBT"] = 0.01
    cfg = tmp_path / "single.json"
    cfg.write_text(json.dumps(doc))
    res = subprocess.run([build.RUNNER, str(cfg)], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr
    f = GSDFile(str(tmp_path / "out" / "single.gsd"))
    frames, gts = doc["MD"]["FRAMES"], doc["MD"]["GTS"]
    assert f.nframes == frames + 1
    assert f.chunk_names(0) == REFERENCE_FRAME_CHUNKS and f.types(0) == ["C1"]
    last = GSDFile(str(tmp_path / "out" / "Last" / "single.Last.gsd"))
    assert last.chunk_names(0) == REFERENCE_FRAME_CHUNKS
    r = G.RunInput(str(cfg))
    eng = r.cycle_engine()
    eng.upload(**r.cycle_initial_state())
    for _ in range(frames):
        eng.step(gts)
        eng.check_positions()
    s = eng.download()
    eng.close()
    n = s["ncells"]
    assert n > (200 if integrator == "EULER" else 20) and int(f.read(frames, "particles/N")[0]) == n
    np.testing.assert_array_equal(f.read(frames, "particles/velocity")[:, :2], s["vel"].astype(np.float32))
    exp = (s["pos"] - 20.0).astype(np.float32)
    np.testing.assert_array_equal(f.read(frames, "particles/position")[:, :2], exp)
    np.testing.assert_array_equal(f.read(frames, "particles/charge"), s["rho"].astype(np.float32))
    np.testing.assert_array_equal(f.read(frames, "particles/mass"), s["pressure"].astype(np.float32))
    np.testing.assert_array_equal(last.read(0, "particles/diameter"), s["sigma"].astype(np.float32))


@pytest.mark.parametrize("integrator", ["EULER", "DPD"])
def test_runner_final_state_h5_and_restart(gpu_lib, tmp_path, integrator):
    """OUTPUT.FORMAT with H5: cil_gpu_run writes <NAME>.Last.h5 beside the final GSD frame. Its
    SigmaCore, RHO, PR and Vel are the FP32 values of the GSD file's diameter, charge, mass and
    velocity, as in the reference's own pair of files; F is the force at the final state. A run
    restarted from it with INIT H5 ALL starts from those values."""
    G = gpu_lib
    from cil_cuda_gb300 import build
    doc = json.load(open(SINGLE))
    doc["OUTPUT"]["DIR"] = str(tmp_path / "out")
    doc["OUTPUT"]["FORMAT"] = ["GSD", "H5"]
    if integrator == "DPD":
        doc["MD"]["INTEGRATOR"] = {"SELECT": "DPD", "DPD": {"DISSAMCEL": 0.0, "DISDIFCEL": 2.0, "DISBG": 0.5}}
        doc["MD"]["KBT"] = 0.01
    cfg = tmp_path / "run.json"
    cfg.write_text(json.dumps(doc))
    res = subprocess.run([build.RUNNER, str(cfg)], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr
    name = doc["OUTPUT"]["NAME"]
    h5 = str(tmp_path / "out" / "Last" / (name + ".Last.h5"))
    f = GSDFile(str(tmp_path / "out" / "Last" / (name + ".Last.gsd")))
    n = int(f.read(0, "particles/N")[0])
    assert G.h5_read(h5, "R").shape == (n, 1, 2) and n > 20
    np.testing.assert_array_equal(f.read(0, "particles/diameter"), G.h5_read(h5, "SigmaCore").ravel())
    np.testing.assert_array_equal(f.read(0, "particles/charge"), G.h5_read(h5, "RHO"))
    np.testing.assert_array_equal(f.read(0, "particles/mass"), G.h5_read(h5, "PR"))
    np.testing.assert_array_equal(f.read(0, "particles/velocity")[:, :2], G.h5_read(h5, "Vel").reshape(n, 2))
    # the same run through the binding: F is the force at the final state
    r = G.RunInput(str(cfg))
    eng = r.cycle_engine()
    eng.upload(**r.cycle_initial_state())
    for _ in range(doc["MD"]["FRAMES"]):
        eng.step(doc["MD"]["GTS"])
        eng.check_positions()
    s = eng.download()
    eng.close()
    np.testing.assert_array_equal(G.h5_read(h5, "F").reshape(n, 2), s["force"].astype(np.float32))
    np.testing.assert_array_equal(G.h5_read(h5, "T0"), s["t0"])
    if integrator == "DPD":
        np.testing.assert_array_equal(G.h5_read(h5, "FD").reshape(n, 2), s["force_dis"].astype(np.float32))
    # restart from the file
    c = doc["SPECIES"]["DEFINE"][0]
    doc["INIT"][c] = {"SELECT": "H5", "H5": {"SELECT": "ALL",
                                             "ALL": [h5, "R", "Vel", "State", "Theta", "RHO", "SigmaCore"]}}
    doc["OUTPUT"]["DIR"] = str(tmp_path / "restart")
    doc["MD"]["FRAMES"] = 2
    cfg.write_text(json.dumps(doc))
    st = G.RunInput(str(cfg)).cycle_initial_state()
    np.testing.assert_array_equal(st["pos"], G.h5_read(h5, "R").reshape(n, 2))
    res = subprocess.run([build.RUNNER, str(cfg)], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr
    g = GSDFile(str(tmp_path / "restart" / (name + ".gsd")))
    assert int(g.read(0, "particles/N")[0]) == n
    np.testing.assert_array_equal(g.read(0, "particles/diameter"), f.read(0, "particles/diameter"))


@pytest.mark.parametrize("model", ["spring", "machine"])
def test_runner_two_element_final_state_h5(gpu_lib, tmp_path, model):
    G = gpu_lib
    from cil_cuda_gb300 import build
    doc = json.load(open(FIXTURE)) if model == "spring" else json.loads(machine_document())
    doc["OUTPUT"]["DIR"] = str(tmp_path / "out")
    doc["OUTPUT"]["FORMAT"] = ["GSD", "H5"]
    cfg = tmp_path / "run.json"
    cfg.write_text(json.dumps(doc))
    res = subprocess.run([build.RUNNER, str(cfg)], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr
    h5 = str(tmp_path / "out" / "Last" / "colony.Last.h5")
    r = G.RunInput(str(cfg))
    eng = r.engine()
    eng.upload(0, **r.initial_state())
    eng.step(doc["MD"]["GTS"] * doc["MD"]["FRAMES"])
    g = eng.download(0)
    frc = eng.forces(0)
    eng.close()
    n = g["ncells"]
    np.testing.assert_array_equal(G.h5_read(h5, "R"), g["pos"].astype(np.float32))
    np.testing.assert_array_equal(G.h5_read(h5, "SigmaCore"), g["sigma"].astype(np.float32))
    np.testing.assert_array_equal(G.h5_read(h5, "T0"), g["t0"])
    np.testing.assert_array_equal(G.h5_read(h5, "F"), frc.astype(np.float32))
    np.testing.assert_array_equal(G.h5_read(h5, "State"), g["cell_state"])
    assert G.h5_read(h5, "RHO").shape == (n,)


@pytest.mark.parametrize("fixture", ["two", "single"])
def test_runner_h5_frame_file(gpu_lib, tmp_path, fixture):
    """OUTPUT.FORMAT with H5: the frame file <NAME>.h5 (/params dt, L, Tdump; /snapshots/t_<k>
    with R, F, ... and ts) holds the same frames as the GSD file, and writing it leaves the run
    unchanged (the GSD frames equal those of a GSD-only run)."""
    G = gpu_lib
    from cil_cuda_gb300 import build
    doc = json.load(open(FIXTURE if fixture == "two" else SINGLE))
    name = doc["OUTPUT"]["NAME"]
    outs = {}
    for fmt in (["GSD"], ["GSD", "H5"]):
        d = json.loads(json.dumps(doc))
        d["OUTPUT"]["DIR"] = str(tmp_path / "_".join(fmt))
        d["OUTPUT"]["FORMAT"] = fmt
        cfg = tmp_path / ("run_%s.json" % "_".join(fmt))
        cfg.write_text(json.dumps(d))
        res = subprocess.run([build.RUNNER, str(cfg)], capture_output=True, text=True, timeout=300)
        assert res.returncode == 0, res.stderr
        outs["_".join(fmt)] = d["OUTPUT"]["DIR"]
    g0 = GSDFile(os.path.join(outs["GSD"], name + ".gsd"))
    g1 = GSDFile(os.path.join(outs["GSD_H5"], name + ".gsd"))
    assert g0.nframes == g1.nframes == doc["MD"]["FRAMES"] + 1
    h5 = os.path.join(outs["GSD_H5"], name + ".h5")
    L = np.asarray(doc["MD"]["BOX"], float)
    np.testing.assert_array_equal(G.h5_attr(h5, "params", "L"), L)
    np.testing.assert_array_equal(G.h5_attr(h5, "params", "Tdump"), [doc["MD"]["GTS"]])
    for k in range(g0.nframes):
        np.testing.assert_array_equal(g0.read(k, "particles/position"), g1.read(k, "particles/position"))
        step = int(g1.read(k, "configuration/step")[0])
        np.testing.assert_array_equal(G.h5_attr(h5, "snapshots/t_%d" % k, "ts"), [step])
        R = G.h5_read(h5, "snapshots/t_%d/R" % k)
        n = R.shape[0] * R.shape[1]
        assert int(g1.read(k, "particles/N")[0]) == n
        d = g1.read(k, "particles/position")[:, :2].astype(np.float64) - (R.reshape(n, 2) - L / 2)
        assert np.abs(d).max() <= 4 * np.spacing(np.float32(L.max()))
