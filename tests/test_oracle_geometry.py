"""The oracle's box and link-list geometry pinned on the reference's own code (no GPU).

tests/golden/geometry_golden.json holds outputs of the reference's Utils.hpp compiled from its
tree (tests/golden/make_geometry_golden.py): Nint (Utils.hpp:173-175), BoundingBox::distance
and updatePos (Utils.hpp:536-566), LinkListOrtho2D/3D grid sizing, bin ids, LIFO head/link
lists, bin coordinates and half-stencil neighbour ids (Utils.hpp:872-1069), and of its
Lennard-Jones element force LJParams::elemForce with the WCA cutoff (MD.cuh:50-56, 98-113;
Input.cpp:296-301). The oracle's restatement (ora_geom_*, the same functions its step calls)
must reproduce every value bit for bit. Where oracle/ref_build.sh has built the reference here, fresh random inputs are compared
live as well."""
import json
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "geometry_golden.json")


def unhex(a):
    return np.array([float.fromhex(x) for x in a], np.float64)


@pytest.fixture(scope="module")
def golden():
    with open(GOLDEN) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def ora(oracle_lib):
    from oracle import geometry as G
    return G.oracle_geometry()


def bits(a):
    return np.asarray(a, np.float64).view(np.uint64)


def test_nint_matches_reference(golden, ora):
    a = unhex(golden["nint"]["a"])
    np.testing.assert_array_equal(ora.nint(a), np.array(golden["nint"]["out"]))


def test_minimum_image_distance_matches_reference(golden, ora):
    for c in golden["distance"]:
        dim = c["dim"]
        r12, d2 = ora.distance(dim, unhex(c["box"]), c["periodic"], unhex(c["r1"]), unhex(c["r2"]))
        np.testing.assert_array_equal(bits(r12.reshape(-1)), bits(unhex(c["r12"])))
        np.testing.assert_array_equal(bits(d2), bits(unhex(c["d2"])))


def test_position_update_and_wrap_match_reference(golden, ora):
    for c in golden["update_pos"]:
        dim = c["dim"]
        out = ora.update_pos(dim, unhex(c["box"]), c["periodic"], unhex(c["r"]), unhex(c["v"]), float.fromhex(c["dt"]))
        np.testing.assert_array_equal(bits(out.reshape(-1)), bits(unhex(c["out"])))


def test_link_list_matches_reference(golden, ora):
    for c in golden["link_list"]:
        dim = c["dim"]
        L = ora.link_list(dim, float.fromhex(c["rcut"]), unhex(c["box"]), c["periodic"], unhex(c["r"]))
        assert L["ns"].tolist() == c["ns"]
        np.testing.assert_array_equal(L["head"], c["head"])
        np.testing.assert_array_equal(L["list"], c["list"])
        np.testing.assert_array_equal(L["coords"].reshape(-1), c["coords"])
        np.testing.assert_array_equal(L["neighbor_ids"].reshape(-1), c["neighbor_ids"])
    # the collapsed grid is among the cases
    assert any(c["ns"][:2] == [1, 1] for c in golden["link_list"])


def test_lj_force_matches_reference(golden):
    from oracle import geometry as G
    assert len(golden["lj_force"]) == 3
    for c in golden["lj_force"]:
        f0, inside = G.lj_force_oracle(float.fromhex(c["eps"]), 2 ** (1 / 6), unhex(c["r2"]), unhex(c["si"]),
                                       unhex(c["sj"]))
        np.testing.assert_array_equal(inside, c["inside"])
        np.testing.assert_array_equal(bits(f0), bits(unhex(c["f0"])))
        assert 0 < np.sum(inside) < len(inside)


def test_lj_attraction_matches_reference(golden):
    """The LJ law with ATTRACTION ON (LJParams::elemForce, MD.cuh:72-92, rcut2 = RCUT^2 as
    Input.cpp:303-315 sets it), plain and with SHIFT FORCE, at the cutoff and one ulp around it,
    bit for bit."""
    from oracle import geometry as G
    assert len(golden["lj_attr_force"]) == 3
    for c in golden["lj_attr_force"]:
        f0, inside = G.lj_attr_force_oracle(float.fromhex(c["eps"]), float.fromhex(c["rcut"]), c["shifted"],
                                            unhex(c["r2"]), unhex(c["si"]), unhex(c["sj"]))
        np.testing.assert_array_equal(inside, c["inside"])
        np.testing.assert_array_equal(bits(f0), bits(unhex(c["f0"])))
        assert 0 < np.sum(inside) < len(inside)
        f = unhex(c["f0"])
        assert (f > 0).any() and (f < 0).any()  # the attractive tail and the repulsive core


def test_sc_force_matches_reference(golden):
    """The soft-core cubic well (SCParams::elemForce, MD.cuh:134-232): the reference's values at
    its branch points (y = -xi, 0, xi), at both bounds of its window with one ulp either side,
    with and without OPT::FORCE_SHIFTED, bit for bit."""
    from oracle import geometry as G
    assert len(golden["sc_force"]) == 3
    for c in golden["sc_force"]:
        f0, inside = G.sc_force_oracle(float.fromhex(c["eps_core"]), float.fromhex(c["eps_well"]),
                                       float.fromhex(c["xi"]), float.fromhex(c["rcut_scale"]), c["shifted"],
                                       unhex(c["r2"]), unhex(c["si"]), unhex(c["sj"]))
        np.testing.assert_array_equal(inside, c["inside"])
        np.testing.assert_array_equal(bits(f0), bits(unhex(c["f0"])))
        assert 0 < np.sum(inside) < len(inside)
        f = unhex(c["f0"])
        assert (f > 0).any() and (f < 0).any()  # both the attractive well and the repulsive core


def test_live_against_reference_build(ora):
    from oracle import geometry as G
    ref = G.reference_geometry()
    if ref is None:
        pytest.skip("reference Utils.hpp not built here (oracle/ref_build.sh needs the reference tree)")
    rng = np.random.default_rng(7)
    for dim, box, per, rcut in ((2, np.array([61.7, 23.9]), [1, 1], 1.7), (3, np.array([14.1, 9.7, 30.3]), [1, 0, 1], 2.2)):
        r1 = rng.uniform(0, 1, (3000, dim)) * box
        r2 = rng.uniform(0, 1, (3000, dim)) * box
        a = ora.distance(dim, box, per, r1, r2)
        b = ref.distance(dim, box, per, r1, r2)
        assert (bits(a[0]) == bits(b[0])).all() and (bits(a[1]) == bits(b[1])).all()
        v = rng.normal(0, 30.0, r1.shape)
        assert (bits(ora.update_pos(dim, box, per, r1, v, 1e-4)) == bits(ref.update_pos(dim, box, per, r1, v, 1e-4))).all()
        La = ora.link_list(dim, rcut, box, per, r1)
        Lb = ref.link_list(dim, rcut, box, per, r1)
        for k in La:
            np.testing.assert_array_equal(La[k], Lb[k])
    si = rng.uniform(0.7, 1.3, 5000)
    sj = rng.uniform(0.7, 1.3, 5000)
    r2 = (0.5 * (si + sj)) ** 2 * rng.uniform(0.5, 1.3, 5000)
    a = G.lj_force_oracle(1.0, 2 ** (1 / 6), r2, si, sj)
    b = G.lj_force_reference(1.0, r2, si, sj)
    assert b is not None
    assert (bits(a[0]) == bits(b[0])).all() and (a[1] == b[1]).all()
    r2a = (0.5 * (si + sj)) ** 2 * rng.uniform(0.5, 7.0, 5000)
    for shifted, rcut in ((0, 2.5), (1, 2.5), (1, 1.3)):
        a = G.lj_attr_force_oracle(1.3, rcut, shifted, r2a, si, sj)
        b = G.lj_attr_force_reference(1.3, rcut, shifted, r2a, si, sj)
        assert (bits(a[0]) == bits(b[0])).all() and (a[1] == b[1]).all()
    r2 = (0.5 * (si + sj) + rng.uniform(-0.5, 0.5, 5000)) ** 2
    for shifted, rcs in ((0, 1.0), (1, 1.07)):
        a = G.sc_force_oracle(7.0, 0.8, 0.35, rcs, shifted, r2, si, sj)
        b = G.sc_force_reference(7.0, 0.8, 0.35, rcs, shifted, r2, si, sj)
        assert (bits(a[0]) == bits(b[0])).all() and (a[1] == b[1]).all()
