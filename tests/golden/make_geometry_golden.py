"""Generates tests/golden/geometry_golden.json from the reference's own box, link-list and
Lennard-Jones code.

Runs oracle/ref_build.sh, which compiles the reference's Utils.hpp (Nint, Utils.hpp:173-175;
BoundingBox::distance and updatePos, Utils.hpp:536-566; LinkListOrtho2D/3D get_opt_size,
init/reset, populate_list, get_cellCoord, get_cellID, Utils.hpp:872-1069) from the reference
tree into oracle/_ref/libref_utils.so, with oracle/boost_shim standing in for the two Boost
headers, then records its outputs on seeded inputs and edge cases: half-integer and near-half
ratios for Nint, separations of exactly half a box and just around it, positions at 0 and just
below L, displacements that wrap once either way, bin boundaries, grids that collapse to one
bin, open and periodic axes in 2D and 3D. It also records the reference's SCParams::elemForce
(the soft-core cubic well, plain and shifted) and its LJParams::elemForce
(MD.cuh:50-56, 98-113; compiled by the same recipe into oracle/_ref/libref_force.so) with its
WCA cutoff, at three well depths, on polydisperse pairs and at the cutoff and one ulp around it,
and with the attraction's cutoff (rcut2 = RCUT^2), plain and force-shifted.
Doubles are stored as hex strings (bit-exact).
tests/test_oracle_geometry.py checks the oracle's restatement (ora_geom_*) against this file.

Usage: python tests/golden/make_geometry_golden.py   (needs the reference tree; not run by tests)
"""
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def hexs(a):
    return [float(x).hex() for x in np.asarray(a, np.float64).reshape(-1)]


def nint_inputs(rng):
    k = np.arange(-6, 7, dtype=np.float64)
    edge = np.concatenate([k + 0.5, k - 0.5, np.nextafter(k + 0.5, -np.inf), np.nextafter(k + 0.5, np.inf),
                           [0.0, -0.0, 0.49999999999999994, -0.49999999999999994, 1e-300, -1e-300, 1e9 + 0.5,
                            -(1e9 + 0.5)]])
    return np.concatenate([edge, rng.normal(0.0, 3.0, 400)])


def distance_cases(rng):
    cases = []
    for dim, box, per in ((2, [37.3, 51.7], [1, 1]), (2, [20.0, 13.1], [1, 0]), (3, [12.9, 17.5, 9.1], [1, 1, 0]),
                          (3, [8.0, 8.0, 8.0], [1, 1, 1])):
        box = np.array(box)
        n = 200
        r1 = rng.uniform(0, 1, (n, dim)) * box
        r2 = rng.uniform(0, 1, (n, dim)) * box
        # separations of exactly half a box, and one ulp either side, along every axis
        m = 20
        a = rng.uniform(0, 1, (m, dim)) * box * 0.5
        for j, f in enumerate((0.5, np.nextafter(0.5, 0), np.nextafter(0.5, 1))):
            b = a.copy()
            b[:, j % dim] = a[:, j % dim] + f * box[j % dim]
            r1 = np.vstack([r1, a, b])
            r2 = np.vstack([r2, b, a])
        r1 = np.vstack([r1, r1[:10]])
        r2 = np.vstack([r2, r1[:10]])  # coincident points
        cases.append(dict(dim=dim, box=box, periodic=per, r1=r1, r2=r2))
    return cases


def update_cases(rng):
    cases = []
    for dim, box, per, dt in ((2, [37.3, 51.7], [1, 1], 1e-4), (2, [37.3, 51.7], [1, 1], 0.0),
                              (3, [12.9, 17.5, 9.1], [1, 1, 0], 5e-5), (3, [12.9, 17.5, 9.1], [1, 1, 0], 0.0)):
        box = np.array(box)
        n = 150
        r = rng.uniform(0, 1, (n, dim)) * box
        edge = np.vstack([np.zeros(dim), np.nextafter(box, 0), box * 1e-17, box - box * 1e-15])
        r = np.vstack([r, np.repeat(edge, 25, axis=0)])
        scale = 1.0 if dt == 0.0 else 1.0 / dt
        v = rng.normal(0.0, 1e-3, r.shape) * scale
        # displacements that cross 0 or L exactly or by an ulp
        v[n:n + 25] = -scale * 1e-12
        v[n + 25:n + 50] = scale * 1e-12
        v[n + 50:n + 75] = -scale * 1e-300
        v[n + 75:n + 100] = scale * (box * 2e-15)
        cases.append(dict(dim=dim, box=box, periodic=per, dt=dt, r=r, v=v))
    return cases


def link_cases(rng):
    cases = []
    for dim, box, per, rcut in ((2, [37.3, 51.7], [1, 1], 2.3), (2, [37.3, 51.7], [1, 0], 3.6),
                                (2, [9.0, 40.0], [1, 1], 3.5),  # 2 bins along x: collapses to one bin
                                (3, [8.9, 9.5, 9.1], [1, 1, 0], 1.1), (3, [8.0, 8.0, 8.0], [1, 1, 1], 2.0)):
        box = np.array(box)
        n = 300
        r = rng.uniform(0, 1, (n, dim)) * box
        ns = np.floor(box / (rcut + box.min() * 1e-8)).astype(int)
        ns = np.maximum(ns, 1)
        # positions on bin boundaries, at 0 and just below L
        k = rng.integers(0, ns, (80, dim))
        r = np.vstack([r, k * (box / ns), np.zeros((3, dim)), np.tile(np.nextafter(box, 0), (3, 1))])
        cases.append(dict(dim=dim, box=box, periodic=per, rcut=rcut, r=r))
    return cases


def lj_inputs(rng):
    n = 400
    si = np.clip(rng.normal(1.0, 0.1, n), 0.5, None)
    sj = np.clip(rng.normal(1.0, 0.1, n), 0.5, None)
    sij2 = (0.5 * (si + sj)) ** 2
    r2 = sij2 * rng.uniform(0.55, 1.4, n)
    # exactly at the WCA cutoff and one ulp either side (the cutoff is inclusive)
    rc2 = sij2[:40] * (2.0 ** (1.0 / 3.0))
    r2 = np.concatenate([r2, rc2, np.nextafter(rc2, 0), np.nextafter(rc2, np.inf)])
    si = np.concatenate([si, si[:40], si[:40], si[:40]])
    sj = np.concatenate([sj, sj[:40], sj[:40], sj[:40]])
    return r2, si, sj


LJ_ATTR_CASES = ((1.0, 2.5, 0), (1.0, 2.5, 1), (0.6, 1.5, 1))


def lj_attr_inputs(rng, rcut):
    n = 400
    si = np.clip(rng.normal(1.0, 0.1, n), 0.5, None)
    sj = np.clip(rng.normal(1.0, 0.1, n), 0.5, None)
    sij2 = (0.5 * (si + sj)) ** 2
    r2 = sij2 * rng.uniform(0.55, 1.1 * rcut * rcut, n)
    # exactly at the cutoff sij2 RCUT^2 and one ulp either side (the cutoff is inclusive)
    rc2 = sij2[:40] * (rcut * rcut)
    r2 = np.concatenate([r2, rc2, np.nextafter(rc2, 0), np.nextafter(rc2, np.inf)])
    si = np.concatenate([si, si[:40], si[:40], si[:40]])
    sj = np.concatenate([sj, sj[:40], sj[:40], sj[:40]])
    return r2, si, sj


SC_CASES = ((10.0, 0.5, 0.3, 1.0, 0), (10.0, 0.5, 0.3, 1.1, 1), (3.0, 1.2, 0.15, 1.0, 1))


def sc_inputs(rng, xi, rcs):
    n = 400
    si = np.clip(rng.normal(1.0, 0.1, n), 0.5, None)
    sj = np.clip(rng.normal(1.0, 0.1, n), 0.5, None)
    sij = 0.5 * (si + sj)
    r = sij + rng.uniform(-1.5 * xi, 1.5 * xi, n)
    r2 = r * r
    # the branch points y = -xi, 0, xi and the two bounds of the window, with one ulp either side
    k = 25
    pts = [(sij[:k] - xi) ** 2, sij[:k] ** 2, (sij[:k] + xi) ** 2, (rcs * (sij[:k] - xi)) ** 2,
           (rcs * rcs) * ((sij[:k] + xi) * (sij[:k] + xi))]
    extra = []
    for q in pts:
        extra += [q, np.nextafter(q, 0), np.nextafter(q, np.inf)]
    r2 = np.concatenate([r2] + extra)
    si = np.concatenate([si] + [si[:k]] * len(extra))
    sj = np.concatenate([sj] + [sj[:k]] * len(extra))
    return r2, si, sj


def main():
    subprocess.run(["bash", os.path.join(ROOT, "oracle", "ref_build.sh")], check=True)
    from oracle import geometry as G
    ref = G.reference_geometry()
    assert ref is not None, "oracle/_ref/libref_utils.so was not built (reference tree missing?)"
    rng = np.random.default_rng(20251204)
    out = {"source": "reference Utils.hpp (Nint, BoundingBox, LinkListOrtho2D/3D) compiled by oracle/ref_build.sh",
           "nint": None, "distance": [], "update_pos": [], "link_list": []}
    a = nint_inputs(rng)
    out["nint"] = {"a": hexs(a), "out": [int(x) for x in ref.nint(a)]}
    for c in distance_cases(rng):
        r12, d2 = ref.distance(c["dim"], c["box"], c["periodic"], c["r1"], c["r2"])
        out["distance"].append(dict(dim=c["dim"], box=hexs(c["box"]), periodic=c["periodic"], r1=hexs(c["r1"]),
                                    r2=hexs(c["r2"]), r12=hexs(r12), d2=hexs(d2)))
    for c in update_cases(rng):
        r = ref.update_pos(c["dim"], c["box"], c["periodic"], c["r"], c["v"], c["dt"])
        out["update_pos"].append(dict(dim=c["dim"], box=hexs(c["box"]), periodic=c["periodic"], dt=float(c["dt"]).hex(),
                                      r=hexs(c["r"]), v=hexs(c["v"]), out=hexs(r)))
    for c in link_cases(rng):
        L = ref.link_list(c["dim"], c["rcut"], c["box"], c["periodic"], c["r"])
        out["link_list"].append(dict(dim=c["dim"], box=hexs(c["box"]), periodic=c["periodic"],
                                     rcut=float(c["rcut"]).hex(), r=hexs(c["r"]), ns=[int(x) for x in L["ns"]],
                                     head=L["head"].tolist(), list=L["list"].tolist(),
                                     coords=L["coords"].reshape(-1).tolist(),
                                     neighbor_ids=L["neighbor_ids"].reshape(-1).tolist()))
    out["lj_force"] = []
    r2, si, sj = lj_inputs(rng)
    for eps in (1.0, 0.37, 5.0):
        f0, inside = G.lj_force_reference(eps, r2, si, sj)
        out["lj_force"].append(dict(eps=float(eps).hex(), r2=hexs(r2), si=hexs(si), sj=hexs(sj), f0=hexs(f0),
                                    inside=inside.tolist()))
    out["lj_attr_force"] = []
    for eps, rcut, shifted in LJ_ATTR_CASES:
        r2, si, sj = lj_attr_inputs(rng, rcut)
        f0, inside = G.lj_attr_force_reference(eps, rcut, shifted, r2, si, sj)
        out["lj_attr_force"].append(dict(eps=float(eps).hex(), rcut=float(rcut).hex(), shifted=shifted, r2=hexs(r2),
                                         si=hexs(si), sj=hexs(sj), f0=hexs(f0), inside=inside.tolist()))
    out["sc_force"] = []
    for e0, em, xi, rcs, shifted in SC_CASES:
        r2, si, sj = sc_inputs(rng, xi, rcs)
        f0, inside = G.sc_force_reference(e0, em, xi, rcs, shifted, r2, si, sj)
        out["sc_force"].append(dict(eps_core=float(e0).hex(), eps_well=float(em).hex(), xi=float(xi).hex(),
                                    rcut_scale=float(rcs).hex(), shifted=shifted, r2=hexs(r2), si=hexs(si),
                                    sj=hexs(sj), f0=hexs(f0), inside=inside.tolist()))
    path = os.path.join(HERE, "geometry_golden.json")
    with open(path, "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print(f"wrote {path} ({os.path.getsize(path)} bytes)")


if __name__ == "__main__":
    main()
