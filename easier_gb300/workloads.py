"""The reference tutorial's workloads written against this API.

``ShallowWaterEquation`` is tutorial/shallow_water_equation/swe_main.py
:13-141 and ``Poisson`` is tutorial/poisson/poisson_main.py:16-53, with the
HDF5 inputs replaced by in-memory arrays (h5py is not part of this image).
``P1Poisson`` is the benchmark's P1 finite-element system in the same
``Linsys`` form.  The builders generate the mesh and geometry with the
native host code (``mesh.py``).
"""
from __future__ import annotations

from typing import Optional

import numpy as np
import torch

from . import mesh as _mesh
from . import module as esr
from .numeric import Linsys


def _t(a, dtype=None):
    t = a if isinstance(a, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(a))
    return t.to(dtype) if dtype is not None else t


class ShallowWaterEquation(esr.Module):
    """Shallow-water equations on a triangular mesh (swe_main.py:13-141)."""

    def __init__(self, src, dst, bcells, geometry: dict, h, dt=0.005, uh=None, vh=None, device="cpu") -> None:
        super().__init__()
        self.dt = dt
        nc = geometry["area"].shape[0]
        self.ne = len(src)
        self.nc = nc
        self.nbc = len(bcells)
        self.scatter = esr.Reducer(_t(dst, torch.long), nc)
        self.gather_src = esr.Selector(_t(src, torch.long))
        self.gather_dst = esr.Selector(_t(dst, torch.long))
        self.scatter_b = esr.Reducer(_t(bcells, torch.long), nc)
        self.gather_b = esr.Selector(_t(bcells, torch.long))
        f = torch.float64
        self.x = esr.Tensor(_t(geometry["x"], f), mode="partition")
        self.y = esr.Tensor(_t(geometry["y"], f), mode="partition")
        self.area = esr.Tensor(_t(geometry["area"], f), mode="partition")
        self.sx = esr.Tensor(_t(geometry["sx"], f), mode="partition")
        self.sy = esr.Tensor(_t(geometry["sy"], f), mode="partition")
        self.bsx = esr.Tensor(_t(geometry["bsx"], f), mode="partition")
        self.bsy = esr.Tensor(_t(geometry["bsy"], f), mode="partition")
        self.h = esr.Tensor(_t(h, f), mode="partition")
        self.alpha = esr.Tensor(_t(geometry["alpha"], f), mode="partition")
        self.uh = esr.Tensor(esr.zeros((nc,), dtype=f) if uh is None else _t(uh, f), mode="partition")
        self.vh = esr.Tensor(esr.zeros((nc,), dtype=f) if vh is None else _t(vh, f), mode="partition")
        self.to(device)

    def face_reconstruct(self, phi):
        return (1 - self.alpha) * self.gather_src(phi) + self.alpha * self.gather_dst(phi)

    def delta(self, h, uh, vh):
        h_f = self.face_reconstruct(h)
        uh_f = self.face_reconstruct(uh)
        vh_f = self.face_reconstruct(vh)
        u_f = uh_f / h_f
        v_f = vh_f / h_f
        h_f_square = 0.5 * h_f * h_f
        uh_f_times_sx = uh_f * self.sx
        vh_f_times_sy = vh_f * self.sy
        gather_b_h_square = 0.5 * self.gather_b(h) ** 2
        delta_h = -(self.scatter(uh_f_times_sx + vh_f_times_sy)) / self.area
        delta_uh = -(self.scatter((u_f * uh_f + h_f_square) * self.sx + u_f * vh_f_times_sy)
                     + self.scatter_b(gather_b_h_square * self.bsx)) / self.area
        delta_vh = -(self.scatter(v_f * uh_f_times_sx + (v_f * vh_f + h_f_square) * self.sy)
                     + self.scatter_b(gather_b_h_square * self.bsy)) / self.area
        return delta_h, delta_uh, delta_vh

    def forward(self):
        dh1, duh1, dvh1 = self.delta(self.h, self.uh, self.vh)
        dh2, duh2, dvh2 = self.delta(self.h + 0.5 * self.dt * dh1, self.uh + 0.5 * self.dt * duh1,
                                     self.vh + 0.5 * self.dt * dvh1)
        dh3, duh3, dvh3 = self.delta(self.h + 0.5 * self.dt * dh2, self.uh + 0.5 * self.dt * duh2,
                                     self.vh + 0.5 * self.dt * dvh2)
        dh4, duh4, dvh4 = self.delta(self.h + self.dt * dh3, self.uh + self.dt * duh3, self.vh + self.dt * dvh3)
        self.h[:] += self.dt / 6 * (dh1 + dh2 + dh3 + dh4)
        self.uh[:] += self.dt / 6 * (duh1 + duh2 + duh3 + duh4)
        self.vh[:] += self.dt / 6 * (dvh1 + dvh2 + dvh3 + dvh4)


def make_swe(n: int, dt: float = 5e-4, dtype: torch.dtype = torch.float64, bump: str = "centre",
             device="cpu", h=None) -> ShallowWaterEquation:
    """SWE on the n x n tutorial mesh.  bump='centre': the benchmark's
    h = 1 + 0.1 exp(-((x-.5)^2+(y-.5)^2)/0.01); 'corner': the tutorial's.
    With a CUDA ``device`` the mesh and geometry are generated on it (the
    same values bit for bit); h is evaluated on the host either way."""
    gen = device if torch.device(device).type == "cuda" else None
    m = _mesh.triangular_mesh(n, device=gen)
    g = _mesh.swe_geometry(m)
    geom = dict(sx=g.sx, sy=g.sy, alpha=g.alpha, area=g.area, x=g.x, y=g.y, bsx=g.bsx, bsy=g.bsy)
    if h is None:
        x = g.x.cpu().numpy() if isinstance(g.x, torch.Tensor) else g.x
        y = g.y.cpu().numpy() if isinstance(g.y, torch.Tensor) else g.y
        if bump == "centre":
            h = _mesh.gaussian_bump(x, y, 0.5, 0.5, 0.01)
        else:
            h = _mesh.gaussian_bump(x, y, 0.0, 0.0, 0.01)
    eqn = ShallowWaterEquation(m.src, m.dst, m.bcells, geom, h, dt=dt, device=device)
    if dtype != torch.float64:
        eqn.to(dtype)
    return eqn


class Poisson(esr.Module):
    """Cell-centred FV Poisson (poisson_main.py:16-53)."""

    def __init__(self, src, dst, nc, b, Ac, Af, device="cpu", x=None) -> None:
        super().__init__()
        self.nc = nc
        self.reducer = esr.Reducer(_t(src, torch.long), nc)
        self.selector = esr.Selector(_t(dst, torch.long))
        f = torch.float64
        self.x = esr.Tensor(esr.zeros((nc,), dtype=f), mode="partition") if x is None else x
        self.b = esr.Tensor(_t(b, f), mode="partition")
        self.Ac = esr.Tensor(_t(Ac, f), mode="partition")
        self.Af = esr.Tensor(_t(Af, f), mode="partition")
        self.A = Linsys(self.Ac, self.Af, self.selector, self.reducer)
        self.to(device)


def make_poisson_fv(n: int, device="cpu") -> Poisson:
    m = _mesh.triangular_mesh(n)
    a = _mesh.poisson_fv(m)
    return Poisson(m.src, m.dst, m.nc, a.b, a.Ac, a.Af, device=device)


class P1Poisson(esr.Module):
    """P1 finite elements of -div(kappa grad u) = f, zero Dirichlet, in Linsys
    form: Reducer over rows, Selector over columns."""

    def __init__(self, n: int, kappa: Optional[np.ndarray] = None, b: Optional[np.ndarray] = None,
                 rhs_seed: int = 0, device="cpu") -> None:
        super().__init__()
        sysm = _mesh.p1_system(n, kappa)
        self.n = n
        self.nunk = sysm.nunk
        self.reducer = esr.Reducer(_t(sysm.row), sysm.nunk)
        self.selector = esr.Selector(_t(sysm.col))
        f = torch.float64
        self.Av = esr.Tensor(_t(sysm.Av, f), mode="partition")
        self.Ae = esr.Tensor(_t(sysm.Ae, f), mode="partition")
        rhs = _mesh.random_mode_rhs(n, rhs_seed) if b is None else b
        self.b = esr.Tensor(_t(rhs, f), mode="partition")
        self.x = esr.Tensor(esr.zeros((sysm.nunk,), dtype=f), mode="partition")
        self.A = Linsys(self.Av, self.Ae, self.selector, self.reducer)
        self.to(device)
