"""The single-element cell-cycle model on the GPU (include/cil_cycle.h) against its CPU
restatement (oracle/cil_cycle_oracle.cpp), which draws the same counter-based random numbers
and sums the pair forces in the same order: cell counts, division and apoptosis events and
the per-cell states must agree; the remaining differences are the last bits of libm (log,
exp, pow, sin, cos) between the host and the device, so positions and cycle variables are
compared at 1e-9 relative.

The parameters are the shipped configurations' (Hertz contacts E = 100, nu = 0.5, adhesion
0.2, CYCLE_P0 5, V1 15, TAU_DIVISION 1 +- 0.1) with the time step raised 20x so that cells
divide within a short test, and the friction raised with it (dt / zeta = 1e-3 as in
PRX_MDCK_2D.json): with the shipped friction at this time step the random overlaps of the
start are resolved so violently that the last-bit differences grow 14 % per step."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIG0 = 1.1283791670955126


def colony(rng, n, box, dim=2, spread=0.0):
    pos = rng.uniform(0, 1, size=(n, dim)) * np.asarray(box[:dim])
    return dict(pos=pos, sigma=SIG0 * (1 + spread * rng.uniform(-1, 1, n)), theta=rng.uniform(0, 1, n),
                rho=rng.uniform(0.5, 1.0, n), angvel=np.full(n, 2e-3) * rng.uniform(0.5, 1.5, n))


def run_both(G, O, prm, st, steps, cap=20000, seed=11):
    eng = G.CycleEngine(prm, cap, seed=seed)
    eng.upload(**st)
    eng.step(steps)
    g = eng.download()
    eng.close()
    o = O.CycleOracle(prm, cap, seed)
    o.set_state(**st)
    assert o.step(steps) == 0
    return g, o.state()


def close(a, b, L=None, rel=1e-9):
    d = np.asarray(a, float) - np.asarray(b, float)
    if L is not None:
        d = d - np.round(d / L) * L
    scale = max(1.0, float(np.abs(b).max()) if np.size(b) else 1.0)
    return float(np.abs(d).max()) <= rel * scale if np.size(d) else True


def compare(g, s, box):
    assert g["ncells"] == s["ncells"]
    assert g["ts"] == s["ts"]
    np.testing.assert_array_equal(g["tpressure"], s["tpressure"])
    L = np.asarray(box[:g["pos"].shape[1]])
    assert close(g["pos"], s["pos"], L)
    for k in ("sigma", "sigma_t", "theta", "rho", "angvel", "pressure", "vel", "force", "force_dis", "force_ran"):
        assert close(g[k], s[k]), k


@pytest.mark.parametrize("dim", [2, 3])
def test_cycle_model_matches_oracle(gpu_lib, oracle_lib, dim):
    rng = np.random.default_rng(40 + dim)
    box = [30.0, 30.0, 30.0] if dim == 2 else [12.0, 12.0, 12.0]
    n = 400 if dim == 2 else 700
    prm = dict(dim=dim, box=box, periodic=[1, 1, 1], dt=2e-4, motility=1.0, zeta=0.2, noise_D=0.002, v1=15.0)
    st = colony(rng, n, box, dim)
    g, s = run_both(gpu_lib, oracle_lib, prm, st, 300)
    assert s["ndiv"] > 20 and g["ncells"] == n + s["ndiv"]
    compare(g, s, box)
    assert np.all(np.isfinite(g["pressure"])) and np.abs(g["pressure"]).max() > 0


@pytest.mark.parametrize("law", [1, 2, 3, 4, 5])
def test_apoptosis_laws_match_oracle(gpu_lib, oracle_lib, law):
    """CyclePressure (1), PressureTime (2), the constant rate (3), Cycle (4) and CycleExtrude (5)."""
    rng = np.random.default_rng(50 + law)
    box = [30.0, 30.0, 0.0]
    prm = dict(box=box, dt=2e-4, motility=0.5, zeta=0.2, apoptosis=law, apop_rate=40.0, apop_pressure=1.5,
               apop_duration=1.0, extr_gamma=0.5, cycle_p0=5.0)
    if law == 2:
        prm.update(apop_pressure=0.0, apop_duration=0.01)  # removal after 50 steps at non-negative pressure
    st = colony(rng, 600, box)
    if law == 5:  # quiescent cells (rho <= 0.1) under a pressure above APOP_PRESSURE are extruded
        prm.update(apop_rate=5.0, apop_pressure=0.05, extr_rate=2e-3, extr_gamma=1.0)
        st["rho"] = rng.uniform(0.0, 0.3, 600)
    g, s = run_both(gpu_lib, oracle_lib, prm, st, 120)
    assert s["napo"] > 0
    compare(g, s, box)


DPD = dict(integrator=1, mass=1.0, kbt=0.01, dis_diff=2.0, dis_bg=0.5)


@pytest.mark.parametrize("dim", [2, 3])
def test_dpd_matches_oracle(gpu_lib, oracle_lib, dim):
    """The DPD integrator (CIL.cu:1054-1066) with divisions and the PressureTime apoptosis law
    its step applies: the half kicks, the pair dissipative and random forces (one normal per
    pair and axis, shared by the two cells), the background dissipation and the resets at
    division agree with the restatement."""
    rng = np.random.default_rng(90 + dim)
    box = [30.0, 30.0, 30.0] if dim == 2 else [12.0, 12.0, 12.0]
    n = 400 if dim == 2 else 700
    prm = dict(DPD, dim=dim, box=box, periodic=[1, 1, 1], dt=2e-4, motility=1.0, v1=15.0, apoptosis=2,
               apop_pressure=40.0, apop_duration=0.01)  # the random start's deepest overlaps are removed
    st = colony(rng, n, box, dim)
    st["vel"] = rng.normal(0, 0.2, size=(n, dim))
    g, s = run_both(gpu_lib, oracle_lib, prm, st, 150)
    assert s["ndiv"] > 20 and s["napo"] > 0
    compare(g, s, box)
    assert np.abs(g["vel"]).max() > 0


def test_dpd_restart_and_drain(gpu_lib, oracle_lib):
    """A DPD run in frames (cil_cycle_check_positions with DRAIN between them, Ecoli_channel_2D's
    open y axis) against the restatement; then a download and upload of the state (velocities
    included) restarts the run: the forces are evaluated again at the uploaded state, as the
    reference does at its start."""
    G, O = gpu_lib, oracle_lib
    rng = np.random.default_rng(97)
    box = [5.0, 40.0, 0.0]
    prm = dict(DPD, box=box, periodic=[1, 0, 0], dt=2e-4, motility=20.0, drain=1, divide=0)
    st = colony(rng, 60, box)
    st["pos"][:, 1] = rng.uniform(0.02, 1.0, 60)  # near the open lower edge, moving down
    st["vel"] = np.tile([0.0, -10.0], (60, 1)) + rng.normal(0, 1.0, size=(60, 2))
    eng = G.CycleEngine(prm, 4000, seed=5)
    eng.upload(**st)
    o = O.CycleOracle(prm, 4000, 5)
    o.set_state(**st)
    removed = 0
    for _ in range(4):
        eng.step(50)
        assert o.step(50) == 0
        eng.check_positions()
        removed += o.check_positions()
    g, s = eng.download(), o.state()
    assert 0 < removed < 60
    compare(g, s, box)
    keys = ("pos", "vel", "sigma", "sigma_t", "theta", "rho", "angvel", "tpressure")
    eng.upload(ts=g["ts"], **{k: g[k] for k in keys})
    o.set_state(ts=s["ts"], **{k: s[k] for k in keys})
    eng.step(30)
    assert o.step(30) == 0
    compare(eng.download(), o.state(), box)
    eng.close()


def test_drain_removes_cells_off_the_open_axis(gpu_lib, oracle_lib):
    """Ecoli_channel_2D.json's geometry: periodic x, open y, DRAIN on (checkPositions, CIL.cu:945-966)."""
    G, O = gpu_lib, oracle_lib
    rng = np.random.default_rng(61)
    box = [5.0, 40.0, 0.0]
    prm = dict(box=box, periodic=[1, 0, 0], dt=2e-4, motility=20.0, zeta=0.2, drain=1, zeta_p=0.01, zeta_p_beta=3.0)
    st = colony(rng, 40, box)
    st["pos"][:, 1] = rng.uniform(0.3, 8.0, 40)  # near the open lower edge: the cells moving down leave
    eng = G.CycleEngine(prm, 4000, seed=5)
    eng.upload(**st)
    o = O.CycleOracle(prm, 4000, 5)
    o.set_state(**st)
    removed = 0
    for _ in range(4):
        eng.step(50)
        assert o.step(50) == 0
        eng.check_positions()
        removed += o.check_positions()
        g = eng.download()
        assert g["ncells"] == o.state()["ncells"]
    s = o.state()
    assert removed > 0
    compare(g, s, box)
    g2 = eng.download()
    assert np.all(g2["pos"][:, 1] >= 0.0) and np.all(g2["pos"][:, 1] < 40.0)
    eng.close()
    # without drain a cell off the box is an error
    prm["drain"] = 0
    eng = G.CycleEngine(prm, 4000, seed=5)
    eng.upload(**st)
    eng.step(200)
    with pytest.raises(G.CilError) as e:
        eng.check_positions()
    assert e.value.status == 5
    eng.close()


def test_initial_cell_status(gpu_lib):
    """initializeCellStatus (CIL.cuh:253-330): sigma = SIGMA_CORE, rho = 1, theta uniform on
    [0, 1), cycle speed 1 / max(Nint(N(1, 0.1) / dt), 1)."""
    G = gpu_lib
    rng = np.random.default_rng(7)
    n = 20000
    box = [400.0, 400.0, 0.0]
    prm = dict(box=box, dt=1e-3)
    eng = G.CycleEngine(prm, n, seed=3)
    eng.upload(pos=rng.uniform(0, 400.0, size=(n, 2)))
    s = eng.download()
    eng.close()
    assert np.all(s["sigma"] == SIG0) and np.all(s["sigma_t"] == SIG0) and np.all(s["rho"] == 1.0)
    assert 0.0 <= s["theta"].min() and s["theta"].max() < 1.0 and abs(s["theta"].mean() - 0.5) < 0.01
    span = 1.0 / s["angvel"]
    assert np.allclose(span, np.round(span))
    assert abs(span.mean() * 1e-3 - 1.0) < 0.005 and abs(span.std() * 1e-3 - 0.1) < 0.005


def test_shipped_configuration_grows_from_one_cell(gpu_lib):
    """PRX_MDCK_2D.json's model (HZ, adhesion 0.2, motility 1, V1 15, P0 5) from a single cell,
    with dt raised to 2e-4: the colony doubles about once per cycle time and stays finite."""
    G = gpu_lib
    prm = dict(box=[100.0, 100.0, 0.0], dt=2e-4, motility=1.0, zeta=0.2, v1=15.0)
    eng = G.CycleEngine(prm, 4096, seed=9)
    eng.upload(pos=np.array([[50.0, 50.0]]), theta=np.array([0.0]), rho=np.array([1.0]),
               angvel=np.array([2e-4]), sigma=np.array([SIG0]))
    eng.step(25000)  # 5 cycle times
    s = eng.download()
    eng.close()
    assert 16 <= s["ncells"] <= 64, s["ncells"]
    assert np.all(np.isfinite(s["pos"])) and np.all(np.isfinite(s["sigma"]))


FP32_CASES = [(2, 30.0, 400), (3, 12.0, 700), (2, 3.4, 6)]  # the last: 2 bins per axis, whole-axis searches


@pytest.mark.parametrize("dim,L,n", FP32_CASES)
def test_fp32_contacts_follow_fp64(gpu_lib, dim, L, n):
    """precision = 1: FP32 contact arithmetic on packed FP32 records of the bin order. Over 100
    steps it keeps the FP64 run's cells and events, and its positions and pressures to FP32
    rounding; in 2D and 3D, and in a box of two bins per axis, where the search covers each
    axis whole and the FP32 nearest-image fold applies."""
    G = gpu_lib
    rng = np.random.default_rng(71 + dim)
    box = [L, L, L if dim == 3 else 0.0]
    prm = dict(dim=dim, box=box, periodic=[1, 1, 1], dt=2e-4, motility=1.0, zeta=0.2, noise_D=0.002, v1=15.0)
    st = colony(rng, n, box, dim)
    out = []
    for prec in (0, 1):
        eng = G.CycleEngine(dict(prm, precision=prec), 20000, seed=11)
        eng.upload(**st)
        eng.step(100)
        out.append(eng.download())
        eng.close()
    a, b = out
    assert a["ncells"] == b["ncells"] >= n
    d = a["pos"] - b["pos"]
    d -= np.round(d / L) * L
    assert np.abs(d).max() < 1e-4
    assert np.abs(a["pressure"] - b["pressure"]).max() < 1e-3 * max(1.0, np.abs(a["pressure"]).max())
    assert np.abs(a["pressure"]).max() > 0
    np.testing.assert_allclose(a["sigma"], b["sigma"], rtol=1e-5)


@pytest.mark.parametrize("dim,L,n", FP32_CASES)
def test_dpd_fp32_pair_terms_follow_fp64(gpu_lib, dim, L, n):
    """precision = 1 with DPD: the Hertz, dissipative and random pair terms in FP32 (normals
    from the same Philox words by FP32 Box-Muller), velocities, positions and the cell state in
    FP64. Over 100 steps the cells and events are the FP64 run's, the positions agree to 1e-4 and
    the velocities to 1e-3 of their scale."""
    G = gpu_lib
    rng = np.random.default_rng(73 + dim)
    box = [L, L, L if dim == 3 else 0.0]
    prm = dict(DPD, dim=dim, box=box, periodic=[1, 1, 1], dt=2e-4, motility=1.0, v1=15.0)
    st = colony(rng, n, box, dim)
    st["vel"] = rng.normal(0, 0.2, size=(n, dim))
    out = []
    for prec in (0, 1):
        eng = G.CycleEngine(dict(prm, precision=prec), 20000, seed=11)
        eng.upload(**st)
        eng.step(100)
        out.append(eng.download())
        eng.close()
    a, b = out
    assert a["ncells"] == b["ncells"] >= n
    d = a["pos"] - b["pos"]
    d -= np.round(d / L) * L
    assert np.abs(d).max() < 1e-4
    assert np.abs(a["vel"] - b["vel"]).max() < 1e-3 * max(1.0, np.abs(a["vel"]).max())
    np.testing.assert_allclose(a["sigma"], b["sigma"], rtol=1e-5)


@pytest.mark.parametrize("integrator,precision,apoptosis", [(0, 0, 1), (1, 0, 2), (0, 1, 0), (1, 1, 2)])
def test_graph_replay_equals_launches(gpu_lib, integrator, precision, apoptosis):
    """Captured steps (the default) compute what the same steps launched kernel by kernel
    compute (CIL_CYCLE_NO_GRAPH), bit for bit, through divisions, removals (which rotate the
    state sets), calls of different lengths and a download between calls."""
    G = gpu_lib
    rng = np.random.default_rng(81 + 2 * integrator + precision)
    box = [30.0, 30.0, 0.0]
    prm = dict(box=box, dt=2e-4, motility=1.0, zeta=0.2, v1=15.0, precision=precision, apoptosis=apoptosis,
               apop_rate=40.0, apop_pressure=1.5, apop_duration=1.0, extr_gamma=0.5)
    if integrator:
        prm.update(DPD, apoptosis=apoptosis, apop_pressure=40.0, apop_duration=0.01)
    st = colony(rng, 400, box)
    out = []
    for flags in (0, G.CYCLE_NO_GRAPH):
        eng = G.CycleEngine(dict(prm, flags=flags), 20000, seed=11)
        eng.upload(**st)
        for n in (1, 7, 40, 1, 30):
            eng.step(n)
            eng.download()
        out.append(eng.download())
        eng.close()
    a, b = out
    assert a["ncells"] == b["ncells"] > 0
    for k in ("pos", "vel", "sigma", "theta", "rho", "pressure", "tpressure", "force"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
