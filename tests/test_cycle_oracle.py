"""The single-element cell-cycle restatement (oracle/cil_cycle_oracle.cpp) on the CPU:
division geometry (singleCellDivision, MD.cu:664-718; calculDivisionsSingle, CIL.cu:560-600),
an isolated cell's cycle (no pressure: rho stays 1, theta advances by the cycle speed) and
drain removal (checkPositions, CIL.cu:945-966)."""
import math

import numpy as np
import pytest

SIG0 = 1.1283791670955126


def test_division_halves_the_area_around_the_mother(oracle_lib):
    prm = dict(box=[20.0, 20.0, 0.0], dt=1e-4, motility=0.0, v1=1.0, cycle_tau_v=1e9, cycle_tau_r=1e9)
    o = oracle_lib.CycleOracle(prm, 16, 1)
    o.set_state(np.array([[10.0, 10.0]]), sigma=np.array([SIG0]), theta=np.array([0.9999]), rho=np.array([1.0]),
                angvel=np.array([0.01]))
    o.step(1)
    s = o.state()
    assert s["ncells"] == 2 and s["ndiv"] == 1
    sig = s["sigma"]
    # the mother's diameter after the step's volume update, split into two of half the area
    assert np.allclose(sig, sig[0]) and abs(2 * (math.pi * sig[0] ** 2 / 4) - math.pi * (sig[0] * math.sqrt(2)) ** 2 / 4) < 1e-12
    d = s["pos"][1] - s["pos"][0]
    assert abs(np.linalg.norm(d) - (sig[0] * math.sqrt(2) - sig[0])) < 1e-12  # |2 dr| = lMom - lDaughter
    assert np.allclose(s["pos"].mean(axis=0), [10.0, 10.0], atol=1e-12)
    assert np.all(s["theta"] == 0.0) and np.all(s["vel"] == 0.0)
    assert s["tpressure"][1] == -1


def test_isolated_cell_cycle(oracle_lib):
    prm = dict(box=[20.0, 20.0, 0.0], dt=1e-4, motility=1.0)
    o = oracle_lib.CycleOracle(prm, 16, 2)
    om = 1e-4
    o.set_state(np.array([[10.0, 10.0]]), sigma=np.array([SIG0]), theta=np.array([0.25]), rho=np.array([1.0]),
                angvel=np.array([om]))
    o.step(100)
    s = o.state()
    assert s["ncells"] == 1 and s["pressure"][0] == 0.0 and s["rho"][0] == 1.0
    assert abs(s["theta"][0] - (0.25 + 100 * om)) < 1e-12
    assert s["sigma"][0] > SIG0  # grows toward V1 times the quiescent volume
    # moving with speed m / (zeta area) along its (random first) direction
    v = np.linalg.norm(s["vel"][0])
    assert abs(v - 1.0 / (0.01 * math.pi * s["sigma"][0] ** 2 / 4)) / v < 0.05


@pytest.mark.parametrize("drain", [1, 0])
def test_check_positions(oracle_lib, drain):
    prm = dict(box=[5.0, 10.0, 0.0], periodic=[1, 0, 0], dt=1e-4, motility=0.0, divide=0, drain=drain)
    o = oracle_lib.CycleOracle(prm, 16, 3)
    o.set_state(np.array([[1.0, 5.0], [2.0, -0.5], [3.0, 10.5]]), sigma=np.full(3, SIG0), theta=np.zeros(3),
                rho=np.ones(3), angvel=np.zeros(3))
    r = o.check_positions()
    if drain:
        assert r == 2 and o.state()["ncells"] == 1
    else:
        assert r == -1 and o.state()["ncells"] == 3
