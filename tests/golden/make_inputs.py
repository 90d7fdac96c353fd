"""Write the seeded synthetic inputs once as fixtures (``inputs_seeded.npz``).

The generators live in ``easier_gb300/mesh.py`` and
``easier_gb300/numeric/batched.py``; this script records their output for
small sizes so a later machine (another CPU architecture, another numpy)
can check it reproduces them:
  * Gaussian-bump initial depth on the N=20 tutorial mesh (cell centroids);
  * random-mode right hand side (16 sine modes, seeds 0 and 1) on n=32;
  * Gaussian random field (spectral synthesis, correlation length 0.1,
    variance 1, seed 0) on n=32 and its per-triangle kappa;
  * the P1 system (row, col, Ae, Av) on n=16 with that kind of kappa;
  * the first three instances of the seeded batch (sizes, the first
    2,048 RHS entries of instance 0).

Usage:  python tests/golden/make_inputs.py
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from easier_gb300 import mesh  # noqa: E402
from easier_gb300.numeric.batched import p1_instances  # noqa: E402


def make() -> dict:
    m = mesh.triangular_mesh(20)
    g = mesh.swe_geometry(m)
    out = {"bump_n20": mesh.gaussian_bump(g.x, g.y)}
    out["rhs_n32_s0"] = mesh.random_mode_rhs(32, 0)
    out["rhs_n32_s1"] = mesh.random_mode_rhs(32, 1)
    grf = mesh.gaussian_random_field(32, 0)
    out["grf_n32_s0"] = grf
    out["kappa_n32_s0"] = mesh.kappa_from_field(grf)
    k16 = mesh.kappa_from_field(mesh.gaussian_random_field(16, 0))
    s = mesh.p1_system(16, k16)
    out.update(p1_n16_row=s.row, p1_n16_col=s.col, p1_n16_Ae=s.Ae, p1_n16_Av=s.Av)
    insts = p1_instances(3, 32, 512, seed=0)
    out["batch_s0_sizes"] = np.array([i.n for i in insts], np.int64)
    out["batch_s0_b0_head"] = np.asarray(insts[0].b)[:2048]
    return out


if __name__ == "__main__":
    np.savez_compressed(HERE / "inputs_seeded.npz", **make())
    print("wrote", HERE / "inputs_seeded.npz")
