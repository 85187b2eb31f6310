"""Where the reference tree is, for test infrastructure that reads its files.

The location is CIL_REFERENCE_DIR when set, else the one that oracle/ref_build.sh (the recipe
that compiles the reference's standalone parts) recorded in oracle/_ref/reference_dir when it
last built them; None when neither names an existing directory (then the tests that read the
reference's own files skip, as on a machine without the reference tree)."""
import os

HERE = os.path.dirname(os.path.abspath(__file__))
RECORD = os.path.join(HERE, "_ref", "reference_dir")


def reference_dir():
    d = os.environ.get("CIL_REFERENCE_DIR")
    if not d and os.path.exists(RECORD):
        with open(RECORD) as f:
            d = f.read().strip()
    return d if d and os.path.isdir(d) else None


def reference_path(*parts):
    """A path inside the reference tree, or a path that does not exist when there is none."""
    d = reference_dir()
    return os.path.join(d, *parts) if d else os.path.join(HERE, "_ref", "no-reference-tree", *parts)
