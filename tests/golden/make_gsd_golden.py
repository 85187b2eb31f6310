"""Writes gsd_ref_sequence.gsd in this folder with the reference's own GSD library.

Runs oracle/ref_build.sh, which compiles the reference's vendored gsd.c into
oracle/_ref/libref_gsd.so, and writes the chunk sequence of gsd_sequence.py through it,
opening the file as the reference's output code does (gsd_create, then
gsd_open(GSD_OPEN_APPEND), OutputWriter.cpp:619-621). tests/test_gsd.py writes the same
sequence with the library's cil_gsd_* and compares the files byte for byte.

Usage: python tests/golden/make_gsd_golden.py   (needs the reference tree; not run by tests)
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import gsd_sequence  # noqa: E402
from oracle import ref_gsd  # noqa: E402


def main():
    subprocess.run(["bash", os.path.join(ROOT, "oracle", "ref_build.sh")], check=True)
    out = os.path.join(HERE, "gsd_ref_sequence.gsd")
    ref_gsd.write_sequence(out, gsd_sequence.frames())
    print(out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    main()
