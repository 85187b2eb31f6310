"""The reference's JSON run description read by the library (include/cil_input.h): settings
mapped into cil_config / cil_colony_params, INIT RANDOM equal bit for bit to the reference's
own draws (golden file written from the reference's Random:: by
tests/golden/make_input_golden.py, and live where the reference's RNG is built), INIT JSON,
and the refusals, with the key that caused them, for what the GPU step does not model. No GPU."""
import copy
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, GOLDEN)

import reference_init as R  # noqa: E402
from oracle.refdir import reference_path  # noqa: E402

FIXTURE = os.path.join(GOLDEN, "input_two_element_2d.json")
REF_DIR = reference_path()


@pytest.fixture(scope="module")
def G():
    import cil_cuda_gb300 as G
    if not os.path.exists(G.LIB_PATH):
        from cil_cuda_gb300 import build
        build.build()
    G.lib()
    return G


def doc():
    return json.load(open(FIXTURE))


def load(G, d):
    return G.RunInput(json.dumps(d), is_path=False)


def test_settings_are_mapped(G):
    r = G.RunInput(FIXTURE)
    c, p, run = r.config, r.params, r.run
    assert (c["dim"], c["precision"], c["rng_mode"], c["seed"], c["num_colonies"]) == (2, G.PREC_FP64, G.RNG_DSFMT,
                                                                                        4357, 1)
    assert c["force_law"] == p["force_law"] == G.FORCE_SOFTCORE
    assert p["box"][:2] == [60.0, 60.0] and p["periodic"][:2] == [1, 1]
    assert p["motility"] == [0.0, 1.0] and p["zeta"] == [1.0, 1.0]
    assert (p["epsilon"], p["rcut_scale"], p["kappa"], p["rest0"], p["rest1"]) == (5.0, 1.0, 1.0, 0.5, 1.0)
    assert (p["noise_D"], p["dt"], p["divide"], p["div_tau_mu"], p["div_tau_sigma"], p["apop_rate"]) == \
        (0.001, 0.001, 1, 0.05, 0.005, 0.5)
    assert (run["gts"], run["frames"], run["output_gsd"], run["output_h5"], run["ncells"], run["capacity"]) == \
        (25, 4, 1, 0, 300, 4000)
    assert (run["output_dir"], run["output_name"], run["cell_name"], run["elem_names"]) == \
        ("output", "colony", "A", ["BACK", "FRONT"])


def test_random_init_matches_reference_golden(G):
    st = G.RunInput(FIXTURE).initial_state()
    gold = json.load(open(os.path.join(GOLDEN, "input_random_init_golden.json")))
    pos = np.array([float.fromhex(x) for x in gold["pos"]]).reshape(st["pos"].shape)
    np.testing.assert_array_equal(st["pos"], pos)
    np.testing.assert_array_equal(st["tswitch"], np.array(gold["tswitch"], np.int32))
    assert np.all(st["t0"] == 0)
    np.testing.assert_array_equal(st["sigma"], np.tile([1.0, 0.9], (300, 1)))


@pytest.mark.parametrize("variant", ["euler_no_division", "const_force", "open_y"])
def test_random_init_matches_reference_live(G, variant):
    if not os.path.exists(R.LIB):
        pytest.skip("reference RNG not built (reference tree absent)")
    d = doc()
    loc = d["SPECIES"]["A"]
    if variant == "euler_no_division":
        d["MD"]["INTEGRATOR"]["SELECT"] = "EULER"
        loc["DIVISION"]["ENABLED"] = False
        d["RUNTIME"]["RNG"]["SEED"] = 99
    elif variant == "const_force":
        loc["DIVISION"]["CONST_FORCE"] = True
        d["INIT"]["A"]["RANDOM"]["NUMBER"] = 57
    else:  # 2D with an open axis: no wrap along y
        d["MD"]["PBC"] = [True, False]
        d["RUNTIME"]["RNG"]["SEED"] = 7
    r = load(G, d)
    st = r.initial_state()
    args = R.from_fixture(d)
    pos, tsw = R.reference_init(**args)
    np.testing.assert_array_equal(st["pos"], pos)
    if loc["DIVISION"]["ENABLED"]:
        np.testing.assert_array_equal(st["tswitch"], tsw)
    else:
        assert np.all(st["tswitch"] == -1)


def test_json_init(G):
    d = doc()
    rows = [[1.0 + k, 2.0 + 0.5 * k] for k in range(8)]
    d["INIT"]["A"] = {"SELECT": "JSON", "JSON": rows}
    st = load(G, d).initial_state()
    np.testing.assert_array_equal(st["pos"].reshape(-1, 2), np.array(rows))
    assert len(st["sigma"]) == 4


def test_random_init_3d_out_of_bounds_is_refused(G):
    """In 3D the reference draws sin(phi) as uniform() * pi (Input.cpp:747), so most cells get
    sqrt(1 - sin^2) of a negative number: the reference stops with "Input Positions Out of
    Bounds!" when z is periodic; the library refuses the start in every case."""
    d = doc()
    d["MD"].update(DIM=3, BOX=[20, 20, 20], PBC=[True, True, True])
    r = load(G, d)
    with pytest.raises(G.CilError) as e:
        r.initial_state()
    assert "Out of Bounds" in str(e.value)


@pytest.mark.parametrize("edit,needle", [
    (lambda d: d["UNITS"].update(LENGTH=2), "UNITS.LENGTH"),
    (lambda d: d["MD"]["INTEGRATOR"].update(SELECT="DPD"), "MD.INTEGRATOR.DPD : key not found"),
    (lambda d: (d["MD"]["INTEGRATOR"].update(SELECT="DPD", DPD=dict(DISSAMCEL=1, DISDIFCEL=1, DISBG=0)),
                d["MD"].update(KBT=0.01)), "runs DPD for single-element cells"),
    (lambda d: (d["MD"]["INTEGRATOR"].update(SELECT="STOCHASTIC_HEUN"),
                d["SPECIES"]["A"]["NOISE"].update(RADIAL=0.1, ANGULAR=0.0)), "SPECIES.A.NOISE.RADIAL"),
    (lambda d: d["MD"]["INTEGRATOR"].update(SELECT="VERLET"), "not one of"),
    (lambda d: d["MD"]["DT"].update(SELECT="AUTOSCALE"), "MD.DT.SELECT"),
    (lambda d: d["MD"].update(BOX=[60]), "vector should be of size 2. Got 1"),
    (lambda d: d["SPECIES"].update(DEFINE=["A", "B"]), "SPECIES.DEFINE"),
    (lambda d: d["SPECIES"]["A"].update(NELEM=3), "SPECIES.A.NELEM"),
    (lambda d: d["SPECIES"]["A"].update(NELEM=1), "SPECIES.A.NAMES : vector should be of size 1"),
    (lambda d: d["SPECIES"]["A"].pop("MOTILITY"), "SPECIES.A.MOTILITY : key not found"),
    (lambda d: d["GPU"].pop("SPRING"), "SPECIES.A.DIVISION.R0 : key not found"),
    (lambda d: (d["GPU"].pop("FORCE_LAW"), d["INTERACTIONS"]["PAIRFORCES"].update(SELECT="HZ"),
                d["SPECIES"]["A"]["PAIRFORCES"].update(HZ={"SIGMA_CORE": [1.0, 0.9]})),
     "GPU.FORCE_LAW : the reference's two-element HZ force is zero for every pair"),
    (lambda d: d["INIT"]["A"].update(SELECT="H5"), "INIT.A.H5 : key not found"),
    (lambda d: d["INIT"]["A"].update(SELECT="H5", H5={"SELECT": "LOCATION", "LOCATION": ["/nonexistent.h5", "R"]}),
     "/nonexistent.h5: cannot open"),
    (lambda d: d["SPECIES"]["A"]["APOPTOSIS"].update(APOP_RATE=5000.0), "Apoptosis rate per time step >= 1"),
])
def test_refusals_name_the_key(G, edit, needle):
    d = copy.deepcopy(doc())
    edit(d)
    with pytest.raises(G.CilError) as e:
        load(G, d)
    assert needle in str(e.value)


def test_lj_is_the_reference_law(G):
    d = doc()
    d["INTERACTIONS"]["PAIRFORCES"] = {"SELECT": "LJ", "LJ": {"ATTRACTION": {"SELECT": "OFF"}}}
    del d["GPU"]["FORCE_LAW"]
    r = load(G, d)
    assert r.params["force_law"] == G.FORCE_LJ_WCA and r.params["epsilon"] == 1.0
    assert abs(r.params["rcut_scale"] - 2 ** (1 / 6)) < 1e-15
    assert r.params["force_shifted"] == 0


def lj_attraction_doc(shift="FORCE", domain=None, rcut=2.5):
    d = copy.deepcopy(doc())
    del d["GPU"]["FORCE_LAW"]
    on = {"RCUT": rcut, "SHIFT": shift, "DOMAIN": domain or {"SELECT": "ALL"}}
    d["INTERACTIONS"]["PAIRFORCES"] = {"SELECT": "LJ", "LJ": {"ATTRACTION": {"SELECT": "ON", "ON": on}}}
    return d


@pytest.mark.parametrize("shift,domain,rcs", [
    ("FORCE", None, 2.5),
    ("POTENTIAL", None, 2.5),
    ("FORCE", {"SELECT": "SPECIES", "SPECIES": [["A", "A"]]}, 2.5),
    ("FORCE", {"SELECT": "SPECIES", "SPECIES": []}, 2 ** (1 / 6)),
    ("POTENTIAL", {"SELECT": "ELEMENTS", "ELEMENTS": [[["A", "BACK"], ["A", "BACK"]], [["A", "FRONT"], ["A", "BACK"]],
                                                       [["A", "FRONT"], ["A", "FRONT"]]]}, 2.5),
])
def test_lj_attraction_is_read(G, shift, domain, rcs):
    """ATTRACTION ON (readInteractionsLJ, Input.cpp:294-352): rc2 = RCUT^2 over the pairs of its
    DOMAIN, SHIFT FORCE -> the force-shifted law (OPT::FORCE_SHIFTED, which also applies to
    pairs left at the WCA cutoff)."""
    r = load(G, lj_attraction_doc(shift, domain))
    p = r.params
    assert p["force_law"] == G.FORCE_LJ_WCA and p["epsilon"] == 1.0
    assert abs(p["rcut_scale"] - rcs) < 1e-15
    assert p["force_shifted"] == (1 if shift == "FORCE" else 0)


@pytest.mark.parametrize("edit,needle", [
    (lambda d: d["INTERACTIONS"]["PAIRFORCES"]["LJ"]["ATTRACTION"]["ON"].update(RCUT=1.0), "Invalid LJ cutoff"),
    (lambda d: d["INTERACTIONS"]["PAIRFORCES"]["LJ"]["ATTRACTION"]["ON"].update(
        DOMAIN={"SELECT": "ELEMENTS", "ELEMENTS": [[["A", "BACK"], ["A", "FRONT"]]]}), "one cutoff per species"),
    (lambda d: d["INTERACTIONS"]["PAIRFORCES"]["LJ"]["ATTRACTION"]["ON"].update(
        DOMAIN={"SELECT": "ELEMENTS", "ELEMENTS": [[["A", "MID"], ["A", "FRONT"]]]}), "Unknown element name MID"),
    (lambda d: d["INTERACTIONS"]["PAIRFORCES"]["LJ"]["ATTRACTION"]["ON"].update(
        DOMAIN={"SELECT": "SPECIES", "SPECIES": [["A"]]}), "Wrong cell pair specification"),
    (lambda d: d["INTERACTIONS"]["PAIRFORCES"]["LJ"]["ATTRACTION"]["ON"].update(SHIFT="NONE"), "not one of"),
])
def test_lj_attraction_refusals(G, edit, needle):
    d = lj_attraction_doc()
    edit(d)
    with pytest.raises(G.CilError) as e:
        load(G, d)
    assert needle in str(e.value)


def test_fene_bond_is_read_without_division(G):
    """Without GPU.SPRING and with DIVISION off, the species' FENE block and CIL flag select the
    reference's own bond (binaryCellForce, MD.cu:525-598; Input.cpp:22, 115-136)."""
    d = copy.deepcopy(doc())
    del d["GPU"]["SPRING"]
    d["SPECIES"]["A"]["DIVISION"]["ENABLED"] = False
    p = load(G, d).params
    assert p["intra_law"] == G.INTRA_FENE and p["cil"] == 0
    assert (p["fene_kappa"], p["fene_kappa_push"], p["fene_spring_ratio"], p["fene_rmax"]) == (0.2, 0.5, 0.5, 1.2)
    d["SPECIES"]["A"]["CIL"] = True
    assert load(G, d).params["cil"] == 1
    d["SPECIES"]["A"]["FENE"]["SPRING_RATIO"] = [1.0]
    with pytest.raises(G.CilError) as e:
        load(G, d)
    assert "SPECIES.A.FENE.SPRING_RATIO" in str(e.value)



def machine_doc():
    d = copy.deepcopy(doc())
    del d["GPU"]["SPRING"]
    del d["GPU"]["RNG"]
    d["SPECIES"]["A"]["DIVISION"].update(R0=0.25, Rmin=1.05, Rmin_RATIO=0.0, SWELLING=False)
    d["SPECIES"]["A"].update(GROWTHK0=[0.0, 0.1], GROWTHK1=[1.0, 0.9], GROWTHK2=[0.0, 0.01])
    d["SPECIES"]["A"]["FENE"]["RMAX_DIVISION"] = [1.6]
    return d


def test_dividing_cells_with_the_reference_bond_are_read(G):
    """Dividing cells without GPU.SPRING: the reference's crawling/dividing cells with the DIVISION
    block's R0, Rmin, Rmin_RATIO, TAU_MIGRATION, the species' GROWTHK0/1/2 and RMAX_DIVISION
    (Input.cpp:36-38, 153-243), without a Verlet skin, drawn with the reference's stream unless
    GPU.RNG asks otherwise; the initial states follow initializeCellStatus (CIL.cuh:279-290)."""
    r = load(G, machine_doc())
    p, c = r.params, r.config
    assert p["intra_law"] == G.INTRA_FENE and p["divide"] == 1
    assert (p["div_r0"], p["div_rmin"], p["div_rmin_ratio"], p["fene_rmax_division"]) == (0.25, 1.05, 0.0, 1.6)
    assert (p["mig_tau_mu"], p["mig_tau_sigma"]) == (0.08, 0.01)
    assert list(p["growth_k0"]) == [0.0, 0.1] and list(p["growth_k1"]) == [1.0, 0.9]
    assert list(p["growth_k2"]) == [0.0, 0.01] and list(p["sigma_core"]) == [1.0, 0.9]
    assert c["rng_mode"] == G.RNG_DSFMT and c["skin"] == 0.0
    st = r.initial_state()
    assert set(np.unique(st["cell_state"]).tolist()) == {0, 1}
    d = machine_doc()
    d["GPU"]["RNG"] = "PHILOX"  # the device's own draws, asked for
    assert load(G, d).config["rng_mode"] == G.RNG_PHILOX
    assert p["div_swelling"] == 0
    d = machine_doc()
    d["SPECIES"]["A"]["DIVISION"]["SWELLING"] = True
    assert load(G, d).params["div_swelling"] == 1


def test_heun_active_noise_on_the_reference_bond(G):
    """STOCHASTIC_HEUN turns NOISE_ACTIVE on (Input.cpp:533-535): with the reference's bond its
    RADIAL and ANGULAR amplitudes are read (reference draws, no skin); 3D is refused as the
    reference refuses it."""
    d = copy.deepcopy(doc())
    del d["GPU"]["SPRING"]
    d["SPECIES"]["A"]["DIVISION"]["ENABLED"] = False
    d["MD"]["INTEGRATOR"]["SELECT"] = "STOCHASTIC_HEUN"
    d["SPECIES"]["A"]["NOISE"].update(RADIAL=0.01, ANGULAR=0.02)
    r = load(G, d)
    assert (r.params["noise_radial"], r.params["noise_angular"]) == (0.01, 0.02)
    assert r.config["rng_mode"] == G.RNG_DSFMT and r.config["skin"] == 0.0
    d["MD"]["DIM"] = 3
    d["MD"]["BOX"] = [60, 60, 60]
    d["MD"]["PBC"] = [True, True, True]
    with pytest.raises(G.CilError) as e:
        load(G, d)
    assert "Active noise not yet implemented for 3D systems" in str(e.value)


def sc_doc():
    d = copy.deepcopy(doc())
    del d["GPU"]["FORCE_LAW"]
    d["SPECIES"]["A"]["PAIRFORCES"]["SC"].update(SIGMA_RATIO=[0.3, 0.3 / 0.9], EPSILON_RATIO=[0.1, 0.1])
    return d


def test_sc_is_the_reference_law(G):
    """SELECT SC without GPU.FORCE_LAW runs the reference's cubic well: xi = SIGMA_RATIO x
    SIGMA_CORE and Em = EPSILON_RATIO x EPSILON_CORE (Input.cpp:48-62), rc2 = 1."""
    r = load(G, sc_doc())
    p = r.params
    assert p["force_law"] == r.config["force_law"] == G.FORCE_SC
    assert (p["epsilon"], p["rcut_scale"], p["force_shifted"]) == (5.0, 1.0, 0)
    assert p["well_epsilon"] == 0.1 * 5.0 and p["well_sigma"] == 0.3


@pytest.mark.parametrize("key,value,needle", [
    ("SIGMA_RATIO", [0.3, 0.3], "one well width per species"),
    ("SIGMA_RATIO", [1.2, 1.2], "Sigma Ratio > 1"),
    ("EPSILON_CORE", [5, 6], "one core energy per species"),
    ("EPSILON_RATIO", [0.1, 0.2], "one well depth per species"),
])
def test_sc_refusals(G, key, value, needle):
    d = sc_doc()
    d["SPECIES"]["A"]["PAIRFORCES"]["SC"][key] = value
    with pytest.raises(G.CilError) as e:
        load(G, d)
    assert needle in str(e.value) and "SPECIES.A.PAIRFORCES.SC." + key in str(e.value)


def test_parse_errors(G):
    for text, needle in (("{\"A\": 1,}", "expected a string key"), ("[1, 2", "expected ',' or ']'"),
                         ("{\"A\": tru}", "unexpected character"), ("{} x", "trailing characters"),
                         ("{\"A\": \"\\q\"}", "bad escape")):
        with pytest.raises(G.CilError) as e:
            G.RunInput(text, is_path=False)
        assert needle in str(e.value), (text, str(e.value))
    with pytest.raises(G.CilError) as e:
        G.RunInput(os.path.join(GOLDEN, "no_such_file.json"))
    assert e.value.status == 8


@pytest.mark.parametrize("name,needle", [
    ("input/cil.json", "JSON parse error at line"),  # holds an unresolved merge conflict
    ("input/test.2d.json", "SPECIES.C.P_FRICTION : key not found"),  # the reference's readSpecs needs it too
])
def test_reference_configs_refused_with_reason(G, name, needle):
    p = os.path.join(REF_DIR, name)
    if not os.path.exists(p):
        pytest.skip("reference configs absent")
    with pytest.raises(G.CilError) as e:
        G.RunInput(p)
    assert needle in str(e.value), str(e.value)


@pytest.mark.parametrize("name,ncells,drain,v1", [("PRX_MDCK_2D.json", 1, 1, 15.0),
                                                  ("Match_Puliafito_2D.json", 1, 1, 35.0),
                                                  ("Ecoli_channel_2D.json", 2, 1, 3.0)])
def test_shipped_configs_load_as_the_cycle_model(G, name, ncells, drain, v1):
    """The three shipped configurations are single-element runs of the cell-cycle model."""
    p = os.path.join(REF_DIR, name)
    if not os.path.exists(p):
        pytest.skip("reference configs absent")
    r = G.RunInput(p)
    assert r.elements == 1 and r.config is None
    q = r.params
    assert (q["E"], q["nu"], q["adhesion"], q["divide"], q["drain"], q["v1"]) == (100.0, 0.5, 0.2, 1, drain, v1)
    assert r.run["ncells"] == ncells and r.run["output_gsd"] == 1
    st = r.cycle_initial_state()
    assert st["pos"].shape == (ncells, 2) and np.all(st["rho"] == 1.0) and np.all(st["angvel"] > 0)


SINGLE = os.path.join(GOLDEN, "input_single_element_2d.json")


def test_single_element_init_matches_reference_golden(G):
    r = G.RunInput(SINGLE)
    st = r.cycle_initial_state()
    gold = json.load(open(os.path.join(GOLDEN, "input_single_element_golden.json")))
    h = lambda k: np.array([float.fromhex(x) for x in gold[k]])  # noqa: E731
    np.testing.assert_array_equal(st["pos"].ravel(), h("pos"))
    np.testing.assert_array_equal(st["theta"], h("theta"))
    np.testing.assert_array_equal(st["angvel"], h("angvel"))
    assert np.all(st["sigma"] == 1.1283791670955126) and np.all(st["rho"] == 1.0)
    q = r.params
    assert (q["dim"], q["motility"], q["zeta"], q["tau_div_mu"], q["cycle_p0"], q["apoptosis"]) == \
        (2, 1.0, 0.2, 0.2, 5.0, G.APOP_NONE)


def test_single_element_init_matches_reference_live(G):
    if not os.path.exists(R.LIB):
        pytest.skip("reference RNG not built (reference tree absent)")
    d = json.load(open(SINGLE))
    d["RUNTIME"]["RNG"]["SEED"] = 77
    d["INIT"]["C1"]["RANDOM"]["NUMBER"] = 64
    r = load(G, d)
    st = r.cycle_initial_state()
    pos, theta, angvel = R.reference_cycle_init(77, 64, 2, [40.0, 40.0], (0.2, 0.02), 0.0002)
    np.testing.assert_array_equal(st["pos"], pos)
    np.testing.assert_array_equal(st["theta"], theta)
    np.testing.assert_array_equal(st["angvel"], angvel)


def test_heun_is_read(G):
    d = doc()
    d["MD"]["INTEGRATOR"]["SELECT"] = "STOCHASTIC_HEUN"
    d["SPECIES"]["A"]["NOISE"].update(RADIAL=0.0, ANGULAR=0.0)
    r = load(G, d)
    assert r.config["integrator"] == G.INTEGRATOR_HEUN and r.params["noise_D"] == 0.001


def test_single_element_dpd_is_read(G):
    """MD.INTEGRATOR.SELECT = DPD (Input.cpp:538-544): DISSAMCEL / DISDIFCEL / DISBG from
    MD.INTEGRATOR.DPD, KBT from MD, MASS from the species; no passive noise (NOISE_ON belongs to
    the stochastic integrators) and the PressureTime apoptosis law that the DPD step applies."""
    d = json.load(open(SINGLE))
    d["MD"]["INTEGRATOR"] = {"SELECT": "DPD", "DPD": {"DISSAMCEL": 4.5, "DISDIFCEL": 3.0, "DISBG": 0.0045}}
    d["MD"]["KBT"] = 0.002
    c = d["SPECIES"]["DEFINE"][0]
    d["SPECIES"][c]["MASS"] = [2.5]
    d["SPECIES"][c]["NOISE"]["PASSIVE"] = 0.3
    d["SPECIES"][c]["FRICTION"] = [0.0]  # only the Euler step needs a friction
    d["SPECIES"][c]["APOPTOSIS"]["ENABLED"] = True
    q = load(G, d).params
    assert (q["integrator"], q["mass"], q["kbt"], q["dis_same"], q["dis_diff"], q["dis_bg"]) == \
        (G.CYCLE_DPD, 2.5, 0.002, 4.5, 3.0, 0.0045)
    assert q["noise_D"] == 0.0 and q["apoptosis"] == G.APOP_PRESSURE_TIME and q["extr_rate"] == 0.1
    d["SPECIES"][c]["MASS"] = [0.0]
    with pytest.raises(G.CilError) as e:
        load(G, d)
    assert "MASS" in str(e.value)


def test_single_element_precision_is_read(G):
    d = json.load(open(SINGLE))
    assert load(G, d).params["precision"] == 0  # FP64 unless asked
    d["GPU"] = {"PRECISION": "MIXED"}
    assert load(G, d).params["precision"] == 1
    d["GPU"] = {"PRECISION": "FP16"}
    with pytest.raises(G.CilError) as e:
        load(G, d)
    assert "GPU.PRECISION" in str(e.value)
