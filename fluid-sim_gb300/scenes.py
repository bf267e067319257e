"""Synthetic scene generator for the FluidSim2D step.

The reference ships a single hard-coded demo scene (demo/App.cpp:133-160);
the workloads used here are seeded synthetic scenes in the same unit-domain
form: dx = 1/sizeX, a one-cell SOLID border, and cell (i, j) FLUID when its
centre ((i+0.5)dx, (j+0.5)dx) lies inside the fluid region.  Labels are
written row-major, index j*sizeX + i, which is the layout
FluidSim2D::create copies (src/FluidSim2D.cpp:47).  (The demo writes its
array transposed, i*sizeY + j; that only matters for asymmetric scenes.)
"""
from __future__ import annotations

import numpy as np

EMPTY, FLUID, SOLID = 0, 1, 2
SEMILAGRANGIAN, PICFLIP = 0, 1


def labels(nx, ny, fluid_fn):
    """Cell labels for a unit-width domain with a one-cell solid border."""
    dx = 1.0 / nx
    i = np.arange(nx)
    j = np.arange(ny)
    cx = (i[None, :] + 0.5) * dx
    cy = (j[:, None] + 0.5) * dx
    cells = np.where(fluid_fn(cx, cy), FLUID, EMPTY).astype(np.uint8)
    cells[0, :] = SOLID
    cells[-1, :] = SOLID
    cells[:, 0] = SOLID
    cells[:, -1] = SOLID
    return cells.reshape(-1)


def dam_break(nx, ny=None, *, mode=SEMILAGRANGIAN, dt=1.0 / 120, extent=(0.4, 0.6), disk=None,
              ppc_sqrt=2, pic_flip_alpha=0.05, rho=997.0, gravity=(0.0, -9.8)):
    """Dam break: fluid where x < extent[0] and y < extent[1], optionally
    united with a disk (cx, cy, r)."""
    ny = nx if ny is None else ny

    def fluid(cx, cy):
        m = (cx < extent[0]) & (cy < extent[1])
        if disk is not None:
            dcx, dcy, r = disk
            m = m | ((cx - dcx) ** 2 + (cy - dcy) ** 2 < r * r)
        return m

    return {
        "sizeX": nx, "sizeY": ny, "ppcSqrt": ppc_sqrt, "dt": dt, "dx": 1.0 / nx, "rho": rho,
        "gravityX": gravity[0], "gravityY": gravity[1], "mode": mode,
        "picFlipAlpha": pic_flip_alpha, "cells": labels(nx, ny, fluid),
    }


def sl_dam_break(nx=64, dt=1.0 / 120):
    """Plain semi-Lagrangian dam break (x < 0.4, y < 0.6), 64x64, dt 1/120."""
    return dam_break(nx, mode=SEMILAGRANGIAN, dt=dt)


def pic_dam_break_disk(nx=256, dt=None):
    """PIC/FLIP dam break united with a disk of radius 0.1 at (0.7, 0.7);
    FLIP ratio 0.95 (the reference's picFlipAlpha is the PIC weight, so
    0.05), 4 particles per cell.  dt = 1/240 at 256^2 and scales with dx
    (1/960 at 1024^2) so the CFL number stays the same."""
    if dt is None:
        dt = (1.0 / 240) * (256.0 / nx)
    return dam_break(nx, mode=PICFLIP, dt=dt, disk=(0.7, 0.7, 0.1), pic_flip_alpha=0.05)


def pressure_disks(nx, ny=None, seed=0):
    """Standalone pressure-solve case: a fluid background with random disks
    of air (about 25 % of the cells) and then solid (about 5 %), a solid
    border, a level set of -/+ (0.25..0.75) dx in fluid / non-fluid cells,
    and face velocities drawn from N(0, 1) in FP32.  Returns
    (scene, cell, phi, u, v) with flat arrays in the reference's layouts."""
    ny = nx if ny is None else ny
    rng = np.random.default_rng(seed)
    x = (np.arange(nx) + 0.5)[None, :]
    y = (np.arange(ny) + 0.5)[:, None]
    cells = np.full((ny, nx), FLUID, np.uint8)

    def cover(label, frac):
        target = frac * nx * ny
        while (cells == label).sum() < target:
            cx, cy = rng.uniform(0, nx), rng.uniform(0, ny)
            r = rng.uniform(0.02, 0.08) * min(nx, ny)
            cells[(x - cx) ** 2 + (y - cy) ** 2 < r * r] = label

    cover(EMPTY, 0.25)
    cover(SOLID, 0.05)
    cells[0, :] = cells[-1, :] = SOLID
    cells[:, 0] = cells[:, -1] = SOLID
    sc = dict(dam_break(nx, ny, mode=SEMILAGRANGIAN, extent=(0.0, 0.0)))
    sc["cells"] = cells.reshape(-1)
    dx = sc["dx"]
    mag = (0.25 + 0.5 * rng.random((ny, nx))) * dx
    phi = np.where(cells == FLUID, -mag, mag).reshape(-1)
    u = rng.standard_normal((nx + 1) * ny).astype(np.float32).astype(np.float64)
    v = rng.standard_normal(nx * (ny + 1)).astype(np.float32).astype(np.float64)
    return sc, cells.reshape(-1), phi, u, v


def closed_box(nx, ny=None, *, dt=1.0 / 60, rho=997.0, gravity=(0.0, 0.0)):
    """A closed box of fluid: every interior cell FLUID inside the one-cell
    SOLID border, semi-Lagrangian mode, one particle per cell (the velocity
    rollout does not use them)."""
    ny = nx if ny is None else ny
    sc = dam_break(nx, ny, mode=SEMILAGRANGIAN, dt=dt, extent=(2.0, 2.0), ppc_sqrt=1, rho=rho, gravity=gravity)
    return sc


def fourier_faces(nx, ny, seed, modes=16, amplitude=1.0):
    """A smooth random face-velocity field (u, v): each component is a sum of
    `modes` plane waves a sin(2 pi (kx x + ky y) + phase) with integer wave
    numbers 1..4, N(0, 1) amplitudes and uniform phases, scaled so that its
    largest magnitude over the faces is `amplitude`.  Evaluated at the face
    centres of a unit-width grid (dx = 1/nx): u at (i dx, (j + .5) dx), v at
    ((i + .5) dx, j dx)."""
    rng = np.random.default_rng(seed)
    dx = 1.0 / nx

    def field(x, y):
        k = rng.integers(1, 5, size=(modes, 2))
        a = rng.standard_normal(modes)
        ph = rng.uniform(0, 2 * np.pi, modes)
        f = np.zeros(np.broadcast(x, y).shape)
        for m in range(modes):
            f += a[m] * np.sin(2 * np.pi * (k[m, 0] * x + k[m, 1] * y) + ph[m])
        return f

    iu, ju = np.meshgrid(np.arange(nx + 1), np.arange(ny))
    u = field(iu * dx, (ju + 0.5) * dx)
    iv, jv = np.meshgrid(np.arange(nx), np.arange(ny + 1))
    v = field((iv + 0.5) * dx, jv * dx)
    s = amplitude / max(np.abs(u).max(), np.abs(v).max())
    return (u * s).reshape(-1), (v * s).reshape(-1)


def batch_dam_breaks(count, seed=0, lo=64, hi=512):
    """Independent PIC/FLIP dam breaks of uneven sizes: square grids with a
    side drawn log-uniformly from [lo, hi], fluid block extents (x and y)
    uniform in [0.2, 0.6], 4 particles per cell, FLIP ratio 0.95, dt =
    1/240 scaled by 256/side (the CFL number of the 256^2 scene)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
        ex, ey = rng.uniform(0.2, 0.6, 2)
        out.append(dam_break(n, mode=PICFLIP, dt=(1.0 / 240) * (256.0 / n), extent=(ex, ey), pic_flip_alpha=0.05))
    return out


def batch_closed_boxes(count, seed=0, lo=64, hi=512, dt=1.0 / 60):
    """Closed boxes of fluid with sides drawn log-uniformly from [lo, hi]
    (the differentiable rollout's scenes, in a batch)."""
    rng = np.random.default_rng(seed)
    return [closed_box(int(round(np.exp(rng.uniform(np.log(lo), np.log(hi))))), dt=dt) for _ in range(count)]
