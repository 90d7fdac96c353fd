"""Recipe: compile the reference's own C++ sources into ``oracle/_ref/``.

Builds ``csrc/init.cpp``, ``csrc/triangular_mesh.cpp`` and
``csrc/distpart.cpp`` of the EASIER source tree, where they lie, as the
torch extension they are written for (its only dependency, torch, is
installed).  The result is test infrastructure: ``tests/golden/make_golden.py``
uses it (as ``easier.cpp_extension``) to run the reference here.  Nothing
here is imported by the product.  Outputs only into ``oracle/_ref/``
(git-ignored).  Usage: ``python oracle/build_ref.py [REFERENCE_ROOT]``.

The reference tree is found by ``reference_root()``: ``EASIER_REFERENCE_ROOT``
when set, else the read-only mount this recipe was written against, else
nothing (and every caller skips the reference build).  This recipe is the
only file that names that mount.
"""
import os
import sys
from pathlib import Path

OUT = Path(__file__).resolve().parent / "_ref"
_MOUNT = Path("/root/reference")


def reference_root():
    """The EASIER source tree to build from, or None when there is none."""
    env = os.environ.get("EASIER_REFERENCE_ROOT")
    if env:
        return Path(env)
    return _MOUNT if (_MOUNT / "csrc").is_dir() else None


def build(ref_root=None, verbose: bool = False):
    ref_root = ref_root if ref_root is not None else reference_root()
    if ref_root is None:
        raise FileNotFoundError("no reference tree: set EASIER_REFERENCE_ROOT")
    from torch.utils.cpp_extension import load
    ref_root = Path(ref_root)
    srcs = [ref_root / "csrc" / f for f in ("init.cpp", "triangular_mesh.cpp", "distpart.cpp")]
    missing = [str(s) for s in srcs if not s.exists()]
    if missing:
        raise FileNotFoundError(f"reference sources not found: {missing}")
    OUT.mkdir(parents=True, exist_ok=True)
    return load(name="cpp_extension", sources=[str(s) for s in srcs], extra_cflags=["-O2", "-fopenmp"],
                extra_ldflags=["-fopenmp"], build_directory=str(OUT), verbose=verbose)


if __name__ == "__main__":
    mod = build(Path(sys.argv[1]) if len(sys.argv) > 1 else None, verbose=True)
    print(mod.__file__)
