"""ctypes binding of the reference's vendored GSD library (gsd.c, gsd.h:110-155), compiled by
oracle/ref_build.sh into oracle/_ref/libref_gsd.so. Test infrastructure: it writes the golden
GSD files the library's writer must reproduce byte for byte and reads the files the library
writes. Not used by the product."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libref_gsd.so")
OPEN_READWRITE, OPEN_READONLY, OPEN_APPEND = 1, 2, 3
DTYPES = {1: np.uint8, 2: np.uint16, 3: np.uint32, 4: np.uint64, 5: np.int8, 6: np.int16, 7: np.int32,
          8: np.int64, 9: np.float32, 10: np.float64}
HANDLE_BYTES = 4096  # larger than struct gsd_handle (gsd.h:93-107)


class IndexEntry(C.Structure):  # gsd.h:65-75
    _fields_ = [("frame", C.c_uint64), ("N", C.c_uint64), ("location", C.c_int64), ("M", C.c_uint32),
                ("id", C.c_uint16), ("type", C.c_uint8), ("flags", C.c_uint8)]


def available() -> bool:
    return os.path.exists(LIB)


def load():
    L = C.CDLL(LIB)
    vp = C.c_void_p
    L.gsd_make_version.restype = C.c_uint32
    L.gsd_make_version.argtypes = [C.c_uint, C.c_uint]
    L.gsd_create.restype = C.c_int
    L.gsd_create.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_uint32]
    L.gsd_open.restype = C.c_int
    L.gsd_open.argtypes = [vp, C.c_char_p, C.c_int]
    L.gsd_close.restype = C.c_int
    L.gsd_close.argtypes = [vp]
    L.gsd_end_frame.restype = C.c_int
    L.gsd_end_frame.argtypes = [vp]
    L.gsd_write_chunk.restype = C.c_int
    L.gsd_write_chunk.argtypes = [vp, C.c_char_p, C.c_int, C.c_uint64, C.c_uint32, C.c_uint8, vp]
    L.gsd_find_chunk.restype = C.POINTER(IndexEntry)
    L.gsd_find_chunk.argtypes = [vp, C.c_uint64, C.c_char_p]
    L.gsd_read_chunk.restype = C.c_int
    L.gsd_read_chunk.argtypes = [vp, vp, C.POINTER(IndexEntry)]
    L.gsd_get_nframes.restype = C.c_uint64
    L.gsd_get_nframes.argtypes = [vp]
    return L


def write_sequence(path: str, frames, application="CIL", schema="hoomd", schema_version=(1, 1)):
    """frames: list of frames, each a list of (name, gsd type, array of N x M). Opens the file as
    initGSDOutput does (OutputWriter.cpp:619-621): gsd_create, then gsd_open(GSD_OPEN_APPEND)."""
    L = load()
    ver = L.gsd_make_version(*schema_version)
    assert L.gsd_create(os.fsencode(path), application.encode(), schema.encode(), ver) == 0
    h = C.create_string_buffer(HANDLE_BYTES)
    assert L.gsd_open(h, os.fsencode(path), OPEN_APPEND) == 0
    for fr in frames:
        for name, typ, arr in fr:
            a = np.ascontiguousarray(arr)
            n = a.shape[0] if a.ndim else 1
            m = a.shape[1] if a.ndim > 1 else 1
            rc = L.gsd_write_chunk(h, name.encode(), typ, n, m, 0, a.ctypes.data_as(C.c_void_p))
            assert rc == 0, (name, rc)
        assert L.gsd_end_frame(h) == 0
    assert L.gsd_close(h) == 0


def read_all(path: str, names):
    """{(frame, name): array} of every listed name present in every frame, read by gsd.c."""
    L = load()
    h = C.create_string_buffer(HANDLE_BYTES)
    assert L.gsd_open(h, os.fsencode(path), OPEN_READONLY) == 0
    out = {}
    try:
        nf = int(L.gsd_get_nframes(h))
        for f in range(nf):
            for name in names:
                e = L.gsd_find_chunk(h, f, name.encode())
                if not e:
                    continue
                e = e.contents
                a = np.empty(int(e.N) * int(e.M), DTYPES[int(e.type)])
                assert L.gsd_read_chunk(h, a.ctypes.data_as(C.c_void_p), C.byref(e)) == 0
                out[(f, name)] = a if e.M == 1 else a.reshape(int(e.N), int(e.M))
    finally:
        L.gsd_close(h)
    return out, nf
