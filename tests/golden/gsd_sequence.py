"""A deterministic sequence of GSD chunks that exercises every branch of the GSD 1.0 writer:
all ten element types, frames with varying chunk sets and row counts, more than 128 and more
than 256 index entries (two index moves), a name longer than 63 characters (which gsd.c stores
truncated and never matches again, so every use takes a new name-list entry), and more
than 128 names (names beyond the list get id 65535). Shared by make_gsd_golden.py, which
writes it with the reference's gsd.c, and tests/test_gsd.py, which writes it with the
library."""
import numpy as np

TYPES = {1: np.uint8, 2: np.uint16, 3: np.uint32, 4: np.uint64, 5: np.int8, 6: np.int16, 7: np.int32,
         8: np.int64, 9: np.float32, 10: np.float64}
LONG_NAME = "particles/" + "x" * 70


def frames():
    rng = np.random.default_rng(20261203)
    out = []
    for f in range(72):
        n = 1 + f % 7
        fr = [("configuration/step", 4, np.array([1000 * f], np.uint64)),
              ("configuration/box", 9, np.array([64.0, 48.0, 1.5, 0, 0, 0], np.float32)),
              ("particles/N", 3, np.array([n], np.uint32))]
        if f == 0:
            t = np.zeros((2, 63), np.int8)
            t[0, :6] = np.frombuffer(b"A_BACK", np.int8)
            t[1, :7] = np.frombuffer(b"A_FRONT", np.int8)
            fr.append(("particles/types", 5, t))
        fr.append(("particles/position", 9, rng.normal(size=(n, 3)).astype(np.float32)))
        typ = 1 + f % 10
        fr.append((f"extra/t{typ}", typ, (rng.integers(0, 100, size=(n, 2))).astype(TYPES[typ])))
        if f in (5, 6):
            fr.append((LONG_NAME, 9, np.array([f], np.float32)))
        if f == 40:
            fr += [(f"many/{k:03d}", 7, np.array([k], np.int32)) for k in range(130)]
        out.append(fr)
    return out


def names(seq):
    seen = []
    for fr in seq:
        for name, _, _ in fr:
            if name not in seen:
                seen.append(name)
    return seen
