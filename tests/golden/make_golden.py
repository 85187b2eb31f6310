"""Generates the RNG golden vectors in this folder from the reference's own code.

Runs oracle/ref_build.sh, which compiles the reference's vendored mt/dSFMT.c and its
header-only Random.hpp (Random.hpp:9-114) from the reference tree into oracle/_ref/, then
records the outputs of those functions for a few seeds. The oracle's restated RNG and the
library's host RNG (used in oracle mode) are checked against these files by
tests/test_oracle.py and tests/test_abi.py.

Usage: python tests/golden/make_golden.py   (needs the reference tree; not run by tests)
"""
import ctypes as C
import json
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
SEEDS = [0, 4357, 12345]
COUNT = 800  # crosses two refills of the 382-double state block


def main():
    subprocess.run(["bash", os.path.join(ROOT, "oracle", "ref_build.sh")], check=True)
    L = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libref_random.so"))
    for name in ("ref_close_open", "ref_open_open", "ref_uniform", "ref_normal"):
        getattr(L, name).restype = C.c_double
    L.ref_uniform0x.restype = C.c_double
    L.ref_uniform0x.argtypes = [C.c_double]
    L.ref_normal_ms.restype = C.c_double
    L.ref_normal_ms.argtypes = [C.c_double, C.c_double]
    L.ref_on_dsphere.argtypes = [C.c_int, C.POINTER(C.c_double)]
    L.ref_init.argtypes = [C.c_int]

    out = {"source": "reference mt/dSFMT.c + Random.hpp compiled by oracle/ref_build.sh",
           "seeds": {}}
    for s in SEEDS:
        rec = {}
        L.ref_init(s)
        rec["close_open"] = [L.ref_close_open() for _ in range(COUNT)]
        L.ref_init(s)
        rec["open_open"] = [L.ref_open_open() for _ in range(COUNT)]
        L.ref_init(s)
        rec["uniform"] = [L.ref_uniform() for _ in range(COUNT)]
        L.ref_init(s)
        rec["normal"] = [L.ref_normal() for _ in range(COUNT)]
        L.ref_init(s)
        buf = (C.c_double * 3)()
        v2 = []
        for _ in range(120):
            L.ref_on_dsphere(2, buf)
            v2.append([buf[0], buf[1]])
        v3 = []
        for _ in range(120):
            L.ref_on_dsphere(3, buf)
            v3.append([buf[0], buf[1], buf[2]])
        rec["on_dsphere2_then3"] = {"d2": v2, "d3": v3}
        # a division-like draw sequence: 2 sphere points, 2 normal(1, 0.1), uniform0x(1)
        L.ref_init(s)
        seq = []
        for _ in range(100):
            L.ref_on_dsphere(2, buf)
            a = [buf[0], buf[1]]
            L.ref_on_dsphere(2, buf)
            b = [buf[0], buf[1]]
            seq.append(a + b + [L.ref_normal_ms(1.0, 0.1), L.ref_normal_ms(1.0, 0.1),
                                L.ref_uniform0x(1.0)])
        rec["division_sequence"] = seq
        out["seeds"][str(s)] = rec
    path = os.path.join(HERE, "dsfmt_random_golden.json")
    with open(path, "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
