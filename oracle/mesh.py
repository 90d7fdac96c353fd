"""Oracle: mesh generator and geometry / assembly (test infrastructure).

numpy restatement of csrc/triangular_mesh.cpp:10-143 (get_mesh) and torch
restatements of tutorial/shallow_water_equation/assemble_shallow_water.py
:154-253 and tutorial/poisson/assemble_poisson.py:148-230.
"""
import numpy as np
import torch


def triangular_mesh(n: int):
    """get_mesh (triangular_mesh.cpp:10-143); coordinates of shared corners
    as its sequential loop order leaves them."""
    nc, ne, nbc, npt = 4 * n * n, 12 * n * n - 4 * n, 4 * n, (n + 1) ** 2 + n * n
    d = 1.0 / n
    j, i = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    i, j = i.reshape(-1), j.reshape(-1)          # square r = i + j*n in order
    r = i + j * n
    c0 = 4 * r
    p0 = j * (n + 1) + i
    p1 = (j + 1) * (n + 1) + i
    p2 = p1 + 1
    p3 = p0 + 1
    p4 = (n + 1) ** 2 + n * j + i
    points = np.zeros((npt, 2))
    # corner (ii, jj): last writer in loop order (see triangular_mesh.cpp:43-52)
    jj, ii = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij")
    ii, jj = ii.reshape(-1), jj.reshape(-1)
    xs = np.where(ii < n, ii * d, (n - 1) * d + d)
    ys = np.where(jj < n, jj * d, (n - 1) * d + d)
    points[jj * (n + 1) + ii, 0] = xs
    points[jj * (n + 1) + ii, 1] = ys
    points[p4, 0] = i * d + d / 2
    points[p4, 1] = j * d + d / 2
    cells = np.zeros((nc, 3), np.int64)
    cells[c0] = np.stack([p0, p3, p4], 1)
    cells[c0 + 1] = np.stack([p2, p4, p3], 1)
    cells[c0 + 2] = np.stack([p2, p1, p4], 1)
    cells[c0 + 3] = np.stack([p0, p4, p1], 1)
    src = np.zeros(ne, np.int64)
    dst = np.zeros(ne, np.int64)
    for k in range(4):
        a, b = c0 + k, c0 + (k + 1) % 4
        src[8 * r + 2 * k], dst[8 * r + 2 * k] = a, b
        src[8 * r + 2 * k + 1], dst[8 * r + 2 * k + 1] = b, a
    base = 8 * n * n
    bcells = np.zeros(nbc, np.int64)
    bpoints = np.zeros((nbc, 2), np.int64)
    m = j != 0
    e = base + n * (j[m] - 1) + i[m]
    src[e], dst[e] = c0[m], c0[m] - 4 * n + 2
    m = j == 0
    bcells[i[m]] = c0[m]
    bpoints[i[m]] = np.stack([p0[m], p3[m]], 1)
    m = j != n - 1
    e = base + n * (n - 1) + n * j[m] + i[m]
    src[e], dst[e] = c0[m] + 2, c0[m] + 4 * n
    m = j == n - 1
    bcells[n + i[m]] = c0[m] + 2
    bpoints[n + i[m]] = np.stack([p1[m], p2[m]], 1)
    m = i != 0
    e = base + 2 * n * (n - 1) + (n - 1) * j[m] + i[m] - 1
    src[e], dst[e] = c0[m] + 3, c0[m] - 3
    m = i == 0
    bcells[2 * n + j[m]] = c0[m] + 3
    bpoints[2 * n + j[m]] = np.stack([p0[m], p1[m]], 1)
    m = i != n - 1
    e = base + 3 * n * (n - 1) + (n - 1) * j[m] + i[m]
    src[e], dst[e] = c0[m] + 1, c0[m] + 7
    m = i == n - 1
    bcells[3 * n + j[m]] = c0[m] + 1
    bpoints[3 * n + j[m]] = np.stack([p2[m], p3[m]], 1)
    return dict(src=src, dst=dst, cells=cells, bcells=bcells, bpoints=bpoints, points=points)


def _face_norm(p0, p1, p2):
    """get_face_norm (assemble_shallow_water.py:173-183)."""
    a1, a2 = p0[:, 0], p0[:, 1]
    b1, b2 = p1[:, 0], p1[:, 1]
    c1, c2 = p2[:, 0], p2[:, 1]
    s = torch.sign((b1 - c1) * (a2 - c2) - (b2 - c2) * (a1 - c1))
    return s * (b2 - c2), -s * (b1 - c1)


def _alpha(sc, dc, p0, p1):
    """get_alpha (assemble_shallow_water.py:154-171)."""
    x1, y1, x2, y2 = sc[:, 0], sc[:, 1], dc[:, 0], dc[:, 1]
    x3, y3, x4, y4 = p0[:, 0], p0[:, 1], p1[:, 0], p1[:, 1]
    y21, y43, y31 = y2 - y1, y4 - y3, y3 - y1
    x31, x21, x43 = x3 - x1, x2 - x1, x4 - x3
    return (x31 * y43 - y31 * x43) / (x21 * y43 - y21 * x43)


def swe_geometry(m):
    """ShallowWaterInitializer.forward (assemble_shallow_water.py:185-253),
    without the initial condition."""
    P = torch.from_numpy(m["points"])
    cells = torch.from_numpy(m["cells"])
    src, dst = torch.from_numpy(m["src"]), torch.from_numpy(m["dst"])
    sp = [P[cells[src, k]] for k in range(3)]
    dp = [P[cells[dst, k]] for k in range(3)]
    sc = (sp[0] + sp[1] + sp[2]) / 3.
    dc = (dp[0] + dp[1] + dp[2]) / 3.
    sx = torch.zeros(src.shape[0], dtype=torch.float64)
    sy = torch.zeros_like(sx)
    al = torch.zeros_like(sx)
    for a, b, c in ((2, 0, 1), (0, 1, 2), (1, 2, 0)):
        nx, ny = _face_norm(sp[a], sp[b], sp[c])
        nx_, ny_ = _face_norm(dc, sp[b], sp[c])
        cond = (nx * nx_ + ny * ny_) < 0
        sx = torch.where(cond, nx, sx)
        sy = torch.where(cond, ny, sy)
        al = torch.where(cond, _alpha(sc, dc, sp[b], sp[c]), al)
    p0, p1, p2 = (P[cells[:, k]] for k in range(3))
    x0, y0, x1, y1, x2, y2 = p0[:, 0], p0[:, 1], p1[:, 0], p1[:, 1], p2[:, 0], p2[:, 1]
    area = 0.5 * torch.abs(x0 * (y1 - y2) + x1 * (y2 - y0) + x2 * (y0 - y1))
    cent = (p0 + p1 + p2) / 3.
    bp = torch.from_numpy(m["bpoints"])
    bc = cent[torch.from_numpy(m["bcells"])]
    bnx, bny = _face_norm(bc, P[bp[:, 0]], P[bp[:, 1]])
    return dict(sx=sx.numpy(), sy=sy.numpy(), alpha=al.numpy(), area=area.numpy(), x=cent[:, 0].numpy(),
                y=cent[:, 1].numpy(), bsx=(-bnx).numpy(), bsy=(-bny).numpy())


def poisson_fv(m):
    """PoissonInitializer.forward (assemble_poisson.py:160-230)."""
    P = torch.from_numpy(m["points"])
    cells = torch.from_numpy(m["cells"])
    src, dst = torch.from_numpy(m["src"]), torch.from_numpy(m["dst"])
    nc = cells.shape[0]
    sp = [P[cells[src, k]] for k in range(3)]
    dp = [P[cells[dst, k]] for k in range(3)]
    sc = (sp[0] + sp[1] + sp[2]) / 3.
    dc = (dp[0] + dp[1] + dp[2]) / 3.
    dist = dc - sc
    nx = torch.zeros(src.shape[0], dtype=torch.float64)
    ny = torch.zeros_like(nx)
    for a, b, c in ((2, 0, 1), (0, 1, 2), (1, 2, 0)):
        ox, oy = _face_norm(sp[a], sp[b], sp[c])
        ox_, oy_ = _face_norm(dc, sp[b], sp[c])
        cond = (ox * ox_ + oy * oy_) < 0
        nx = torch.where(cond, ox, nx)
        ny = torch.where(cond, oy, ny)
    dist = dist / (dist ** 2).sum(dim=1, keepdim=True)
    Af = dist[:, 0] * nx + dist[:, 1] * ny
    Ac = -torch.zeros(nc, dtype=torch.float64).scatter_reduce_(0, src, Af, "sum", include_self=False)
    p0, p1, p2 = (P[cells[:, k]] for k in range(3))
    x0, y0, x1, y1, x2, y2 = p0[:, 0], p0[:, 1], p1[:, 0], p1[:, 1], p2[:, 0], p2[:, 1]
    area = 0.5 * torch.abs(x0 * (y1 - y2) + x1 * (y2 - y0) + x2 * (y0 - y1))
    cent = (p0 + p1 + p2) / 3.
    rho = torch.exp(-0.5 * 400 * ((cent - torch.tensor([[0.5, 0.5]], dtype=torch.float64)) ** 2).sum(1))
    b = rho * area
    bp = torch.from_numpy(m["bpoints"])
    bcells = torch.from_numpy(m["bcells"])
    bc = cent[bcells]
    b_p0, b_p1 = P[bp[:, 0]], P[bp[:, 1]]
    bfc = (b_p0 + b_p1) / 2.
    bnx, bny = _face_norm(bc, b_p0, b_p1)
    bd = bfc - bc
    bd = bd / (bd ** 2).sum(dim=-1, keepdim=True)
    Ac = Ac.sub_(torch.zeros(nc, dtype=torch.float64).scatter_reduce_(
        0, bcells, bd[:, 0] * bnx + bd[:, 1] * bny, "sum", include_self=False))
    return dict(Af=Af.numpy(), Ac=Ac.numpy(), b=b.numpy(), rho=rho.numpy(), centroid=cent.numpy())


def p1_system(n: int, kappa=None):
    """P1 stiffness of -div(kappa grad u) on the n x n square grid split
    along (i,j)-(i+1,j+1), zero Dirichlet boundary, per-triangle kappa
    (no reference counterpart; plain element-by-element assembly)."""
    m = n - 1
    nunk = m * m
    K = np.ones(2 * n * n) if kappa is None else np.asarray(kappa, dtype=np.float64)
    A = {}

    def node(i, j):
        return (j - 1) * m + (i - 1) if 1 <= i <= m and 1 <= j <= m else -1

    for j in range(n):
        for i in range(n):
            for up, tri, right in ((0, ((i, j), (i + 1, j), (i + 1, j + 1)), 1),
                                   (1, ((i, j), (i + 1, j + 1), (i, j + 1)), 2)):
                k = K[2 * (j * n + i) + up]
                R = tri[right]
                others = [v for q, v in enumerate(tri) if q != right]
                local = {(R, R): k, (others[0], others[0]): k / 2, (others[1], others[1]): k / 2,
                         (R, others[0]): -k / 2, (others[0], R): -k / 2,
                         (R, others[1]): -k / 2, (others[1], R): -k / 2}
                for (a, b), v in local.items():
                    ia, ib = node(*a), node(*b)
                    if ia >= 0 and ib >= 0:
                        A[(ia, ib)] = A.get((ia, ib), 0.0) + v
    Av = np.array([A[(u, u)] for u in range(nunk)])
    return Av, A


def p1_arrays(n: int, kappa=None):
    """``p1_system`` as Linsys arrays: (row, col, Ae, Av) with the
    off-diagonal couplings sorted by row, then column."""
    Av, A = p1_system(n, kappa)
    keys = sorted(k for k in A if k[0] != k[1])
    row = np.array([k[0] for k in keys], dtype=np.int64)
    col = np.array([k[1] for k in keys], dtype=np.int64)
    Ae = np.array([A[k] for k in keys], dtype=np.float64)
    return row, col, Ae, Av
