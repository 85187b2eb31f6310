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


DPD = dict(integrator=1, mass=1.0, kbt=0.01, dis_diff=2.0, dis_bg=0.0, motility=0.0, divide=0)


def test_dpd_pair_forces_conserve_momentum(oracle_lib):
    """With no motility and no background term every DPD force is a pair force, equal and
    opposite on the two cells (the Hertz contact, w (v_i,d - v_j,d) n_d^2, and the random force
    with one normal per pair and axis): the total momentum stays at its start."""
    rng = np.random.default_rng(81)
    n, box = 300, [20.0, 20.0, 0.0]
    prm = dict(DPD, box=box, dt=1e-3)
    o = oracle_lib.CycleOracle(prm, 1000, 4)
    vel = rng.normal(0, 0.3, size=(n, 2))
    o.set_state(rng.uniform(0, 20.0, size=(n, 2)), sigma=np.full(n, SIG0), theta=np.zeros(n), rho=np.ones(n),
                angvel=np.zeros(n), vel=vel)
    p0 = vel.sum(axis=0)
    assert o.step(200) == 0
    s = o.state()
    assert s["ncells"] == n
    assert np.abs(s["vel"].sum(axis=0) - p0).max() < 1e-10
    assert np.abs(s["vel"] - vel).max() > 0.05  # the pair forces did act


def test_dpd_background_damping_of_isolated_cells(oracle_lib):
    """Cells far apart feel only DISBG: Fd = -gamma_bg v after each step, and each half kick
    divides by twice the mass argument 2m (updateVelocities, CIL.cu:894; updateVel,
    Utils.hpp:568-571), so v_k = v_0 (1 - gamma_bg dt / (4m))^(k-1) (the first step kicks with
    the forces of the start, whose Fd is the pair part only)."""
    prm = dict(DPD, box=[40.0, 40.0, 0.0], dt=1e-3, dis_bg=3.0, mass=0.7)
    o = oracle_lib.CycleOracle(prm, 16, 5)
    pos = np.array([[5.0, 5.0], [25.0, 5.0], [5.0, 25.0], [25.0, 25.0]])
    vel = np.array([[1.0, 0.5], [-0.2, 0.3], [0.0, -1.0], [0.4, 0.4]])
    o.set_state(pos, sigma=np.full(4, SIG0), theta=np.zeros(4), rho=np.ones(4), angvel=np.zeros(4), vel=vel)
    k = 50
    assert o.step(k) == 0
    s = o.state()
    f = 1 - 3.0 * 1e-3 / (4 * 0.7)
    np.testing.assert_allclose(s["vel"], vel * f ** (k - 1), rtol=1e-12)
    disp = vel * 1e-3 * sum(f ** max(j - 1, 0) for j in range(1, k + 1))
    np.testing.assert_allclose(s["pos"], pos + disp, rtol=0, atol=1e-12)
