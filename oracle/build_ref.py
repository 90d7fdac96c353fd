"""Recipe: compile the reference's own C++ sources into ``oracle/_ref/``.

Builds ``csrc/init.cpp``, ``csrc/triangular_mesh.cpp`` and
``csrc/distpart.cpp`` of the EASIER source tree, where they lie, as the
torch extension they are written for (its only dependency, torch, is
installed).  The result is test infrastructure: ``tests/golden/make_golden.py``
uses it (as ``easier.cpp_extension``) to run the reference here.  Nothing
here is imported by the product.  Outputs only into ``oracle/_ref/``
(git-ignored).  Usage: ``python oracle/build_ref.py [REFERENCE_ROOT]``.
"""
import os
import sys
from pathlib import Path

OUT = Path(__file__).resolve().parent / "_ref"
DEFAULT_REF = Path(os.environ.get("EASIER_REFERENCE_ROOT", "/root/reference"))


def build(ref_root: Path = DEFAULT_REF, verbose: bool = False):
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
    mod = build(Path(sys.argv[1]) if len(sys.argv) > 1 else DEFAULT_REF, verbose=True)
    print(mod.__file__)
