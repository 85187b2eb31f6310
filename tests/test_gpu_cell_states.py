"""The reference's crawling/dividing two-element cells (CIL_INTRA_FENE with divide; calculDivisions,
CIL.cu:369-455, with binaryCellForce's dividing branch, MD.cu:545-567) against the oracle's
restatement, oracle mode (the reference's dSFMT draws, the division outcomes read back from the
device each step):

* forces of a colony with crawling, dividing and undefined cells: 1e-12 (FP64), 2e-5 (mixed);
* 300 steps in which cells start dividing, divide and fail to divide, with apoptosis, Euler and
  the reference's own Heun integrator (also with the bond's active noise): cell counts, birth and
  switch times and states equal, positions 1e-9 (FP64).
"""
import numpy as np
import pytest

from cil_cuda_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


def machine_params(**kw):
    p = S.fene_params(box=60.0, dt=1e-3, noise_D=0.002, divide=1, div_tau_mu=0.15, div_tau_sigma=0.01,
                      fene_rmax_division=1.6, growth_k0=[0.0, 0.0], growth_k1=[1.0, 1.0], growth_k2=[0.0, 0.0],
                      div_r0=0.25, div_rmin=1.05, div_rmin_ratio=0.0, mig_tau_mu=0.08, mig_tau_sigma=0.01,
                      sigma_core=[1.0, 1.0], apop_rate=0.5)
    p.update(kw)
    return p


def colony(p, n=300, seed=3):
    st = S.disk_colony(n, p, seed=seed)
    st["sigma"][:] = 1.0
    st["cell_state"] = np.random.default_rng(seed).integers(0, 3, n).astype(np.int32)
    return st


def minimage(a, b, L):
    d = np.asarray(a) - np.asarray(b)
    return d - np.round(d / L) * L


@pytest.mark.parametrize("precision,active", [(0, False), (1, False), (0, True)])
def test_forces_with_cell_states(gpu_lib, oracle_lib, precision, active):
    G = gpu_lib
    p = machine_params(noise_D=0.0, growth_k0=[0.3, 0.1], growth_k2=[0.05, 0.02])
    if active:  # the bond's active noise, drawn by both sides from the reference's stream
        p.update(noise_D=0.002, noise_radial=0.05, noise_angular=0.03)
    st = colony(p)
    eng = G.Engine([p], [len(st["sigma"])], precision=precision, rng=G.RNG_DSFMT, seed=5)
    eng.upload(0, **st)
    fg = eng.forces(0)
    eng.close()
    o = oracle_lib.Oracle(p, len(st["sigma"]), 5)
    o.set_state(**st)
    fo = o.compute_forces()
    err = np.abs(fg - fo).max() / np.abs(fo).max()
    assert err <= (1e-12 if precision == 0 else 2e-5), err


@pytest.mark.parametrize("integrator,extra", [(0, None), (1, None), (1, "active"), (1, "swelling")])
def test_state_machine_matches_oracle(gpu_lib, oracle_lib, integrator, extra):
    """active: the bond's active noise of StochasticHeun (radial and angular, CIL.cu:803-815);
    swelling: dividing cells' diameters grow towards the larger SIGMA_CORE (CIL.cu:970-991)."""
    G = gpu_lib
    p = machine_params()
    if extra == "active":
        p.update(noise_radial=0.01, noise_angular=0.02)
    elif extra == "swelling":
        p.update(div_swelling=1, sigma_core=[1.0, 1.2])
    st = colony(p)
    cap = 4000
    eng = G.Engine([p], [cap], precision=G.PREC_FP64, rng=G.RNG_DSFMT, seed=7, integrator=integrator)
    eng.upload(0, **st)
    eng.step(300)
    g = eng.download(0)
    eng.close()
    o = oracle_lib.Oracle(p, cap, 7, integrator=integrator)
    o.set_state(**st)
    assert o.step(300) == 0
    s = o.state()
    ev = o.events()
    kinds = {k: int((ev[:, 1] == k).sum()) for k in range(4)}
    assert kinds[0] > 50 and kinds[2] > 50 and kinds[3] > 50 and kinds[1] > 5, kinds  # every transition
    assert g["ncells"] == len(s["sigma"])
    np.testing.assert_array_equal(g["cell_state"], s["cell_state"])
    np.testing.assert_array_equal(g["t0"], s["t0"])
    np.testing.assert_array_equal(g["tswitch"], s["tswitch"])
    np.testing.assert_array_equal(g["sigma"], s["sigma"])
    assert np.abs(minimage(g["pos"], s["pos"], 60.0)).max() <= 1e-9


def test_state_machine_forms_refused(gpu_lib):
    """Bins rebuilt every step (no Verlet skin); the bond's active noise with the reference's draws."""
    G = gpu_lib
    p = machine_params()
    for rng in (G.RNG_DSFMT, G.RNG_PHILOX):
        with pytest.raises(G.CilError):
            G.Engine([p], [1000], rng=rng, precision=G.PREC_MIXED, skin=0.3)
    q = S.fene_params(noise_radial=0.01)
    with pytest.raises(G.CilError):
        G.Engine([q], [1000], rng=G.RNG_PHILOX)


@pytest.mark.parametrize("swelling", [0, 1])
def test_state_machine_philox(gpu_lib, oracle_lib, swelling):
    """The device's own draws (Philox; starts, failures and divisions decided on the device, no
    read-back): graph replay equals launching step by step; the colony grows as the oracle's
    (other random numbers, so the counts agree statistically), every transition happens, and the
    states stay crawling or dividing."""
    G = gpu_lib
    p = machine_params(div_swelling=swelling, sigma_core=[1.0, 1.2] if swelling else [1.0, 1.0])
    st = colony(p)
    outs = []
    for graphs in (True, False):
        eng = G.Engine([p], [4000], precision=G.PREC_FP64, rng=G.RNG_PHILOX, seed=7, graphs=graphs)
        eng.upload(0, **st)
        eng.step(300)
        outs.append(eng.download(0))
        eng.close()
    g, g2 = outs
    assert g["ncells"] == g2["ncells"]
    np.testing.assert_array_equal(g["pos"], g2["pos"])
    np.testing.assert_array_equal(g["cell_state"], g2["cell_state"])
    o = oracle_lib.Oracle(p, 4000, 7)
    o.set_state(**st)
    assert o.step(300) == 0
    n_o = o.ncells
    assert abs(g["ncells"] - n_o) <= 0.2 * n_o, (g["ncells"], n_o)
    assert set(np.unique(g["cell_state"]).tolist()) <= {0, 1, 2}
    assert (g["cell_state"] == 0).sum() > 20 and (g["cell_state"] == 1).sum() > 20
    assert (g["tswitch"] > 300).all()
    if swelling:
        assert np.abs(g["sigma"] - 1.0).max() > 0.0 and g["sigma"].max() <= 1.2
