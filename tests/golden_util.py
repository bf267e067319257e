"""Helpers to read the golden vectors made by tests/golden/make_golden.py."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NAMES = ("sl_dam_32", "pic_disk_32", "pic_dam_40x24", "sl_dam_40x24")
FIELDS = ("cell", "phi", "p", "u", "v", "newU", "newV", "particles", "particleVels")
SL_ORDER = ["createWaterLevelSet", "applySemiLagrangianAdvection", "applyGravity", "createSolidLevelSet",
            "applyProjection", "updateVelocity", "applyAdvection"]
PIC_ORDER = ["createWaterLevelSet", "transferVelocityToGrid", "applyGravity", "createSolidLevelSet",
             "applyProjection", "updateVelocity", "updateParticleVelocities", "applyAdvection"]


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: z[k] for k in z.files}


def scene(g):
    sc = {k[len("scene_"):]: g[k] for k in g if k.startswith("scene_")}
    for k in ("sizeX", "sizeY", "ppcSqrt", "mode"):
        sc[k] = int(sc[k])
    for k in ("dt", "dx", "rho", "gravityX", "gravityY", "picFlipAlpha"):
        sc[k] = float(sc[k])
    return sc


def snapshot(g, prefix):
    return {f: g[prefix + f] for f in FIELDS}


def stage_order(sc):
    return SL_ORDER if sc["mode"] == 0 else PIC_ORDER


def pre_stage(g, k):
    return snapshot(g, "init_" if k == 0 else f"s{k - 1}_post_")


def stats_series(seed, frames, stages):
    """Seeded inputs of the statistics writers: per-frame stage times (ms,
    float32, frames x stages, a few exact zeros) and the three conservation
    series, spread over many magnitudes and with values at the rounding
    boundary of the "%f" format."""
    rng = np.random.default_rng(seed)
    ms = rng.lognormal(mean=0.0, sigma=2.0, size=(frames, stages)).astype(np.float32)
    ms[rng.random(ms.shape) < 0.05] = 0.0
    vol = rng.uniform(0.05, 2.5, frames)
    en = rng.normal(0.0, 1.0, frames) * 10.0 ** rng.integers(-3, 7, frames)
    pen = -np.abs(rng.normal(0.0, 1.0, frames)) * 10.0 ** rng.integers(-3, 7, frames)
    vol[0], en[1], pen[2] = 0.0000005, -0.0000005, 1234567.0000005
    return ms, vol, en, pen
