"""Reader of GSD 1.0 files (the format of the reference's frame output, OutputWriter.cpp:505-644)
in numpy, for the files cil_frame_* and cil_gsd_* write and for the reference's own outputs.

It follows the reading rules of the reference's vendored gsd.c:
  * header checks: magic 0x65DF65DF65DF65DF, format version >= 1.0 (or 0.3) and < 2.0
    (gsd.c:279-286);
  * number of index entries: binary search for the first entry whose location is 0
    (gsd.c:355-379); number of names: the first empty name-list entry (gsd.c:381-394);
  * frames: the last index entry's frame + 1 (gsd.c:396-404);
  * chunk lookup: within the entries of the requested frame, the last one with the name's id
    (gsd_find_chunk, gsd.c:835-880).
"""
from __future__ import annotations

import numpy as np

MAGIC = 0x65DF65DF65DF65DF
HEADER = np.dtype([("magic", "<u8"), ("index_location", "<u8"), ("index_allocated_entries", "<u8"),
                   ("namelist_location", "<u8"), ("namelist_allocated_entries", "<u8"),
                   ("schema_version", "<u4"), ("gsd_version", "<u4"), ("application", "S64"),
                   ("schema", "S64"), ("reserved", "S80")])
ENTRY = np.dtype([("frame", "<u8"), ("N", "<u8"), ("location", "<i8"), ("M", "<u4"), ("id", "<u2"),
                  ("type", "u1"), ("flags", "u1")])
DTYPES = {1: "<u1", 2: "<u2", 3: "<u4", 4: "<u8", 5: "<i1", 6: "<i2", 7: "<i4", 8: "<i8", 9: "<f4", 10: "<f8"}
assert HEADER.itemsize == 256 and ENTRY.itemsize == 32


def make_version(major: int, minor: int) -> int:
    return (major << 16) | minor


class GSDFile:
    def __init__(self, path: str):
        with open(path, "rb") as fh:
            self.raw = fh.read()
        if len(self.raw) < HEADER.itemsize:
            raise ValueError("not a GSD file: shorter than its header")
        self.header = np.frombuffer(self.raw, HEADER, 1)[0]
        h = self.header
        if int(h["magic"]) != MAGIC:
            raise ValueError("not a GSD file: bad magic")
        v = int(h["gsd_version"])
        if (v < make_version(1, 0) and v != make_version(0, 3)) or v >= make_version(2, 0):
            raise ValueError(f"unsupported GSD version {v >> 16}.{v & 0xffff}")
        n_idx = int(h["index_allocated_entries"])
        loc = int(h["index_location"])
        if loc + ENTRY.itemsize * n_idx > len(self.raw):
            raise ValueError("truncated GSD index")
        idx = np.frombuffer(self.raw, ENTRY, n_idx, loc)
        n_names = int(h["namelist_allocated_entries"])
        nloc = int(h["namelist_location"])
        if nloc + 64 * n_names > len(self.raw):
            raise ValueError("truncated GSD name list")
        names = np.frombuffer(self.raw, "S64", n_names, nloc)
        # entries in use: the first with location 0 (binary search, as the writer fills in order)
        if n_idx == 0 or idx[0]["location"] == 0:
            used = 0
        else:
            lo, hi = 0, n_idx
            while hi - lo > 1:
                m = (lo + hi) // 2
                if idx[m]["location"] != 0:
                    lo = m
                else:
                    hi = m
            used = hi
        self.index = idx[:used]
        self.names = []
        for nm in names:
            if not nm:
                break
            self.names.append(nm.decode())
        self.nframes = int(self.index[-1]["frame"]) + 1 if used else 0
        self.application = bytes(h["application"]).decode()
        self.schema = bytes(h["schema"]).decode()
        self.schema_version = int(h["schema_version"])
        self.gsd_version = v

    def find(self, frame: int, name: str):
        """The index entry of chunk `name` in `frame`, or None."""
        if frame >= self.nframes or name not in self.names:
            return None
        nid = self.names.index(name)
        frames = self.index["frame"]
        hi = int(np.searchsorted(frames, frame, side="right"))
        for k in range(hi - 1, -1, -1):
            e = self.index[k]
            if int(e["frame"]) != frame:
                break
            if int(e["id"]) == nid:
                return e
        return None

    def read(self, frame: int, name: str):
        """Chunk data as an array of shape (N,) for M == 1 else (N, M); None if absent."""
        e = self.find(frame, name)
        if e is None:
            return None
        n, m = int(e["N"]), int(e["M"])
        a = np.frombuffer(self.raw, DTYPES[int(e["type"])], n * m, int(e["location"]))
        return a.copy() if m == 1 else a.reshape(n, m).copy()

    def chunk_names(self, frame: int):
        sel = self.index[self.index["frame"] == frame]
        return [self.names[int(i)] if int(i) < len(self.names) else None for i in sel["id"]]

    def types(self, frame: int = 0):
        """particles/types rows as strings (int8 [ntypes][63], zero padded)."""
        t = self.read(frame, "particles/types")
        if t is None:
            return None
        return [bytes(r.astype(np.uint8)).split(b"\0", 1)[0].decode() for r in t]
