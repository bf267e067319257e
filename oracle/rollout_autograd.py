"""FP64 CPU adjoint of the closed-box rollout by automatic differentiation
(test infrastructure only: imported by tests/ as the checker of the
hand-written GPU adjoint, never by the product).

The forward pass restates, in torch FP64 on the CPU, the velocity stages of
the reference's semi-Lagrangian frame on fixed labels without EMPTY cells:

* applySemiLagrangianAdvection (src/FluidSim2D.cpp:206-235) with
  MACGrid2D::velInterpU/V (include/MACGrid2D.h:80-94), Array2D::triCubic
  (include/Array2D.h:244-359) and clampPos (src/FluidSim2D.cpp:645-651),
  double-buffered (every face traces back through the velocity before the
  stage);
* applyGravity (:237-250);
* applyProjection (:252-467): the same matrix and right-hand side, solved
  exactly (pseudo-inverse; on a closed box the matrix has the constant
  null space, which the velocity update does not see) instead of by PCG;
* updateVelocity (:469-550) with Array2D::extrapolate
  (include/Array2D.h:552-591) of the faces without a fluid side, layer by
  layer as the breadth-first queue visits them.

Reverse mode then comes from torch.autograd, independently of the GPU
kernels' hand-derived transposes.
"""
from __future__ import annotations

from collections import deque

import numpy as np
import torch

EMPTY, FLUID, SOLID = 0, 1, 2


def _cr(t):
    return (-0.5 * t ** 3 + t ** 2 - 0.5 * t,
            1.5 * t ** 3 - 2.5 * t ** 2 + 1.0,
            -1.5 * t ** 3 + 2.0 * t ** 2 + 0.5 * t,
            0.5 * t ** 3 - 0.5 * t ** 2)


def _tricubic(data, W, H, px, py):
    """Catmull-Rom sample of data (H x W) at grid coordinates (px, py)."""
    x = torch.floor(px).detach().long()
    y = torch.floor(py).detach().long()
    wx = _cr(px - x)
    wy = _cr(py - y)
    out = 0.0
    for j in range(4):
        yy = torch.clamp(y + j - 1, 0, H - 1)
        row = 0.0
        for i in range(4):
            xx = torch.clamp(x + i - 1, 0, W - 1)
            row = row + wx[i] * data[yy, xx]
        out = out + wy[j] * row
    return out


class ClosedBoxRollout:
    """Forward model of the rollout on a scene's labels (no EMPTY cell)."""

    def __init__(self, sc):
        self.NX, self.NY = sc["sizeX"], sc["sizeY"]
        self.cells = np.asarray(sc["cells"], np.uint8).reshape(self.NY, self.NX)
        if (self.cells == EMPTY).any():
            raise ValueError("the rollout needs a scene without EMPTY cells")
        self.dx, self.dt, self.rho = sc["dx"], sc["dt"], sc["rho"]
        self.gx, self.gy = sc["gravityX"], sc["gravityY"]
        self._setup()

    # ---- fixed structure: positions, face classes, matrix, extrapolation layers ----
    def _setup(self):
        NX, NY, dx = self.NX, self.NY, self.dx
        c = self.cells
        ju, iu = np.meshgrid(np.arange(NY), np.arange(NX + 1), indexing="ij")
        jv, iv = np.meshgrid(np.arange(NY + 1), np.arange(NX), indexing="ij")
        self.xu = torch.tensor(iu * dx, dtype=torch.float64)
        self.yu = torch.tensor((ju + 0.5) * dx, dtype=torch.float64)
        self.xv = torch.tensor((iv + 0.5) * dx, dtype=torch.float64)
        self.yv = torch.tensor(jv * dx, dtype=torch.float64)

        def cell(i, j):
            return c[j, i] if 0 <= i < NX and 0 <= j < NY else SOLID

        # face classes of updateVelocity: 0 never visited, 1 fluid-fluid, 2 zeroed, 3 unknown
        cu = np.zeros((NY, NX + 1), np.int8)
        for j in range(NY):
            for i in range(NX):
                a, b = cell(i - 1, j), c[j, i]
                if (i > 0 and a == FLUID) or b == FLUID:
                    cu[j, i] = 2 if (i == 0 or a == SOLID or b == SOLID) else 1
                else:
                    cu[j, i] = 3
        cv = np.zeros((NY + 1, NX), np.int8)
        for j in range(NY):
            for i in range(NX):
                a, b = cell(i, j - 1), c[j, i]
                if (j > 0 and a == FLUID) or b == FLUID:
                    cv[j, i] = 2 if (j == 0 or a == SOLID or b == SOLID) else 1
                else:
                    cv[j, i] = 3
        self.cu, self.cv = cu, cv
        self.layers_u = self._layers(cu == 3)
        self.layers_v = self._layers(cv == 3)

        # projection matrix on the fluid cells and its pseudo-inverse
        fl = np.argwhere(c == FLUID)
        idx = -np.ones((NY, NX), np.int64)
        idx[fl[:, 0], fl[:, 1]] = np.arange(len(fl))
        n = len(fl)
        sA = self.dt / (self.rho * dx * dx)
        A = np.zeros((n, n))
        for k, (j, i) in enumerate(fl):
            for (ii, jj) in ((i - 1, j), (i + 1, j), (i, j - 1), (i, j + 1)):
                if cell(ii, jj) == FLUID:
                    A[k, k] += sA
                    A[k, idx[jj, ii]] = -sA
        # one fluid region with solid walls: A is singular with the constant
        # null space; A + (sA/n) 1 1^T is regular and, for a right-hand side
        # with zero sum (the divergence of a closed box), its solution is the
        # one of A orthogonal to the constants
        self.fluid_idx = torch.tensor(fl)
        self.A = A
        self.Ainv = torch.tensor(np.linalg.inv(A + sA / n * np.ones((n, n))), dtype=torch.float64)
        # not-solid masks of the divergence (solid faces carry velocity 0)
        self.nsL = torch.tensor(np.array([[cell(i - 1, j) != SOLID for i in range(NX)] for j in range(NY)]))
        self.nsR = torch.tensor(np.array([[cell(i + 1, j) != SOLID for i in range(NX)] for j in range(NY)]))
        self.nsD = torch.tensor(np.array([[cell(i, j - 1) != SOLID for i in range(NX)] for j in range(NY)]))
        self.nsU = torch.tensor(np.array([[cell(i, j + 1) != SOLID for i in range(NX)] for j in range(NY)]))

    @staticmethod
    def _layers(unknown):
        """Breadth-first layers of Array2D::extrapolate: per layer L >= 1,
        (flat indices, up to 4 lower-layer neighbour indices, weights)."""
        H, W = unknown.shape
        INF = np.iinfo(np.uint32).max
        lay = np.where(unknown, INF, 0).astype(np.int64)
        q = deque()
        for j in range(H):
            for i in range(W):
                if lay[j, i] != 0 and any(
                        0 <= ii < W and 0 <= jj < H and lay[jj, ii] == 0
                        for ii, jj in ((i - 1, j), (i + 1, j), (i, j - 1), (i, j + 1))):
                    lay[j, i] = 1
                    q.append((i, j))
        order = []
        while q:
            i, j = q.popleft()
            order.append((i, j))
            for ii, jj in ((i - 1, j), (i + 1, j), (i, j - 1), (i, j + 1)):
                if 0 <= ii < W and 0 <= jj < H and lay[jj, ii] == INF:
                    lay[jj, ii] = lay[j, i] + 1
                    q.append((ii, jj))
        out = []
        maxL = max((lay[j, i] for i, j in order), default=0)
        for L in range(1, maxL + 1):
            faces = [(i, j) for i, j in order if lay[j, i] == L]
            fi, nb, w = [], [], []
            for i, j in faces:
                fi.append(j * W + i)
                ns, ws = [], []
                for ii, jj in ((i - 1, j), (i + 1, j), (i, j - 1), (i, j + 1)):
                    if 0 <= ii < W and 0 <= jj < H and lay[jj, ii] < L:
                        ns.append(jj * W + ii)
                        ws.append(1.0)
                while len(ns) < 4:
                    ns.append(0)
                    ws.append(0.0)
                nb.append(ns)
                w.append(ws)
            out.append((torch.tensor(fi), torch.tensor(nb), torch.tensor(w, dtype=torch.float64)))
        return out

    # ---- stages ----
    def _interp_u(self, u, x, y):
        NX, NY, dx = self.NX, self.NY, self.dx
        px = torch.clamp(x / dx, 1e-6, NX - 1 - 1e-6)
        py = torch.clamp(y / dx - 0.5, 1e-6, NY - 1 - 1e-6)
        return _tricubic(u, NX + 1, NY, px, py)

    def _interp_v(self, v, x, y):
        NX, NY, dx = self.NX, self.NY, self.dx
        px = torch.clamp(x / dx - 0.5, 1e-6, NX - 1 - 1e-6)
        py = torch.clamp(y / dx, 1e-6, NY - 1 - 1e-6)
        return _tricubic(v, NX, NY + 1, px, py)

    def _departure(self, u, v, x, y):
        dt, dx, NX, NY = self.dt, self.dx, self.NX, self.NY
        k1x, k1y = self._interp_u(u, x, y), self._interp_v(v, x, y)
        ax, ay = x - 0.5 * dt * k1x, y - 0.5 * dt * k1y
        k2x, k2y = self._interp_u(u, ax, ay), self._interp_v(v, ax, ay)
        bx, by = x - 0.75 * dt * k2x, y - 0.75 * dt * k2y
        k3x, k3y = self._interp_u(u, bx, by), self._interp_v(v, bx, by)
        ox = x - ((2. / 9.) * dt * k1x + (3. / 9.) * dt * k2x + (4. / 9.) * dt * k3x)
        oy = y - ((2. / 9.) * dt * k1y + (3. / 9.) * dt * k2y + (4. / 9.) * dt * k3y)
        off = 1e-3
        ox = torch.clamp(ox, (1.0 + off) * dx, (NX - 1.0 - off) * dx)
        oy = torch.clamp(oy, (1.0 + off) * dx, (NY - 1.0 - off) * dx)
        return ox, oy

    def advect(self, u, v):
        xu, yu = self._departure(u, v, self.xu, self.yu)
        xv, yv = self._departure(u, v, self.xv, self.yv)
        return self._interp_u(u, xu, yu), self._interp_v(v, xv, yv)

    def project(self, u, v):
        NX, NY, dx = self.NX, self.NY, self.dx
        u0, u1 = u[:, :NX], u[:, 1:]
        v0, v1 = v[:NY, :], v[1:, :]
        b = -(1.0 / dx) * (u1 * self.nsR - u0 * self.nsL + v1 * self.nsU - v0 * self.nsD)
        fj, fi = self.fluid_idx[:, 0], self.fluid_idx[:, 1]
        pf = self.Ainv @ b[fj, fi]
        p = torch.zeros((NY, NX), dtype=torch.float64).index_put((fj, fi), pf)
        return p

    def update(self, u, v, p):
        NX, NY = self.NX, self.NY
        s = self.dt / (self.rho * self.dx)
        gu = torch.zeros_like(u)
        gu[:, 1:NX] = p[:, 1:] - p[:, :-1]
        gv = torch.zeros_like(v)
        gv[1:NY, :] = p[1:, :] - p[:-1, :]
        cu, cv = torch.tensor(self.cu), torch.tensor(self.cv)
        nu = torch.where(cu == 1, u - s * gu, torch.where(cu == 2, torch.zeros_like(u), u))
        nv = torch.where(cv == 1, v - s * gv, torch.where(cv == 2, torch.zeros_like(v), v))
        return self._extrap(nu, self.layers_u), self._extrap(nv, self.layers_v)

    @staticmethod
    def _extrap(a, layers):
        shape = a.shape
        flat = a.reshape(-1)
        for fi, nb, w in layers:
            val = (flat[nb] * w).sum(1) / w.sum(1)
            flat = flat.index_put((fi,), val)
        return flat.reshape(shape)

    def step(self, u, v):
        u, v = self.advect(u, v)
        u = u + self.dt * self.gx
        v = v + self.dt * self.gy
        p = self.project(u, v)
        return self.update(u, v, p)

    # ---- rollout, loss and gradient ----
    def loss_and_grad(self, u0, v0, ut, vt, steps):
        NX, NY = self.NX, self.NY
        u = torch.tensor(np.asarray(u0, np.float64).reshape(NY, NX + 1), requires_grad=True)
        v = torch.tensor(np.asarray(v0, np.float64).reshape(NY + 1, NX), requires_grad=True)
        uu, vv = u, v
        for _ in range(steps):
            uu, vv = self.step(uu, vv)
        tu = torch.tensor(np.asarray(ut, np.float64).reshape(NY, NX + 1))
        tv = torch.tensor(np.asarray(vt, np.float64).reshape(NY + 1, NX))
        L = torch.sqrt(((uu - tu) ** 2).sum() + ((vv - tv) ** 2).sum())
        L.backward()
        return L.item(), u.grad.numpy().reshape(-1).copy(), v.grad.numpy().reshape(-1).copy(), \
            uu.detach().numpy().reshape(-1).copy(), vv.detach().numpy().reshape(-1).copy()

    def rollout(self, u0, v0, steps):
        NX, NY = self.NX, self.NY
        with torch.no_grad():
            u = torch.tensor(np.asarray(u0, np.float64).reshape(NY, NX + 1))
            v = torch.tensor(np.asarray(v0, np.float64).reshape(NY + 1, NX))
            for _ in range(steps):
                u, v = self.step(u, v)
        return u.numpy().reshape(-1).copy(), v.numpy().reshape(-1).copy()
