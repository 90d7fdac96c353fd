"""Oracle: the shallow-water step (test infrastructure).

torch-CPU restatement of tutorial/shallow_water_equation/swe_main.py:83-141
(face_reconstruct, delta, forward) with the Selector/Reducer semantics of
easier/core/module.py:364-371 and :441-461: the same aten ops in the same
order, so on the same inputs it is bitwise the reference's CPU backend.
"""
import torch


class SweProblem:
    def __init__(self, src, dst, bcells, sx, sy, alpha, bsx, bsy, area, dt, dtype=torch.float64, device="cpu"):
        """device: where the aten ops run (a CUDA device runs the reference's
        op sequence as eager CUDA kernels: its backend='cuda' path without
        the JitEngine interpreter)."""
        t = lambda a: torch.as_tensor(a).to(device=device, dtype=dtype)  # noqa: E731
        self.src = torch.as_tensor(src, dtype=torch.int64).to(device)
        self.dst = torch.as_tensor(dst, dtype=torch.int64).to(device)
        self.bcells = torch.as_tensor(bcells, dtype=torch.int64).to(device)
        self.sx, self.sy, self.alpha = t(sx), t(sy), t(alpha)
        self.bsx, self.bsy, self.area = t(bsx), t(bsy), t(area)
        self.nc = self.area.shape[0]
        self.dt = float(dt)
        self.dtype = dtype

    def _scatter(self, idx, v):
        return torch.zeros(self.nc, dtype=v.dtype, device=v.device).scatter_reduce_(0, idx, v, "sum",
                                                                                 include_self=False)

    def face_reconstruct(self, phi):
        return (1 - self.alpha) * phi[self.src] + self.alpha * phi[self.dst]

    def delta(self, h, uh, vh):
        h_f = self.face_reconstruct(h)
        uh_f = self.face_reconstruct(uh)
        vh_f = self.face_reconstruct(vh)
        u_f = uh_f / h_f
        v_f = vh_f / h_f
        h_f_square = 0.5 * h_f * h_f
        uh_f_times_sx = uh_f * self.sx
        vh_f_times_sy = vh_f * self.sy
        gbh2 = 0.5 * h[self.bcells] ** 2
        d_h = -(self._scatter(self.dst, uh_f_times_sx + vh_f_times_sy)) / self.area
        d_uh = -(self._scatter(self.dst, (u_f * uh_f + h_f_square) * self.sx + u_f * vh_f_times_sy)
                 + self._scatter(self.bcells, gbh2 * self.bsx)) / self.area
        d_vh = -(self._scatter(self.dst, v_f * uh_f_times_sx + (v_f * vh_f + h_f_square) * self.sy)
                 + self._scatter(self.bcells, gbh2 * self.bsy)) / self.area
        return d_h, d_uh, d_vh

    def step(self, h, uh, vh):
        """One forward() (swe_main.py:121-141); returns the new state."""
        dt = self.dt
        d1 = self.delta(h, uh, vh)
        d2 = self.delta(h + 0.5 * dt * d1[0], uh + 0.5 * dt * d1[1], vh + 0.5 * dt * d1[2])
        d3 = self.delta(h + 0.5 * dt * d2[0], uh + 0.5 * dt * d2[1], vh + 0.5 * dt * d2[2])
        d4 = self.delta(h + dt * d3[0], uh + dt * d3[1], vh + dt * d3[2])
        h = h + dt / 6 * (d1[0] + d2[0] + d3[0] + d4[0])
        uh = uh + dt / 6 * (d1[1] + d2[1] + d3[1] + d4[1])
        vh = vh + dt / 6 * (d1[2] + d2[2] + d3[2] + d4[2])
        return h, uh, vh

    def run(self, h, uh, vh, steps):
        h, uh, vh = (torch.as_tensor(a).to(device=self.src.device, dtype=self.dtype).clone() for a in (h, uh, vh))
        for _ in range(steps):
            h, uh, vh = self.step(h, uh, vh)
        return h, uh, vh
