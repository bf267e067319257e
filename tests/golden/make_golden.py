"""Generate the golden vectors in tests/golden/ from the REFERENCE itself.

Runs the unmodified reference simulator (compiled from its own sources by
oracle/build_oracle.py into oracle/_ref/libfs2d_ref.so: scalar path,
serial, -ffp-contract=off) on small seeded scenes and stores, per scene:

* ``init_*``          the state right after FluidSim2D::create (srand(7));
* ``s{k}_post_*``     the state after each stage k of the first frame, in
                      runFrame's stage order (the state before stage k is
                      ``s{k-1}_post_*``, or ``init_*`` for k = 0);
* ``f{n}_*``          the state after frame n (n in FRAMES_SAVED);
* ``stats_f{n}``      waterVolume, totalEnergy, particleTotalEnergy,
                      avgPressure, avgPressureInFluid, maxVelocity.

* ``stats_csv.npz``  the reference's saveStats output for seeded series
                      (see generate_stats_csv).

Usage (needs the reference checkout, named by FS2D_REFERENCE_DIR, so it runs
only where that exists; "stats" regenerates stats_csv.npz alone):
    FS2D_REFERENCE_DIR=<checkout> python tests/golden/make_golden.py [stats]
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "fluid-sim_gb300"))

import build_oracle  # noqa: E402
import oracle_py as O  # noqa: E402
import scenes  # noqa: E402

SEED = 7
FRAMES = 10
FRAMES_SAVED = (1, 10)
SL_ORDER = ["createWaterLevelSet", "applySemiLagrangianAdvection", "applyGravity", "createSolidLevelSet",
            "applyProjection", "updateVelocity", "applyAdvection"]
PIC_ORDER = ["createWaterLevelSet", "transferVelocityToGrid", "applyGravity", "createSolidLevelSet",
             "applyProjection", "updateVelocity", "updateParticleVelocities", "applyAdvection"]


def golden_scenes():
    return {
        "sl_dam_32": scenes.sl_dam_break(32),
        "pic_disk_32": scenes.pic_dam_break_disk(32),
        "pic_dam_40x24": scenes.dam_break(40, 24, mode=scenes.PICFLIP, dt=1.0 / 200,
                                          extent=(0.5, 0.5), pic_flip_alpha=0.05),
        "sl_dam_40x24": scenes.dam_break(40, 24, mode=scenes.SEMILAGRANGIAN, dt=1.0 / 200,
                                         extent=(0.35, 0.55)),
    }


def stage_order(scene):
    return SL_ORDER if scene["mode"] == scenes.SEMILAGRANGIAN else PIC_ORDER


def scene_record(scene):
    return {k: np.asarray(v) for k, v in scene.items()}


def generate(name, scene):
    out = {}
    for k, v in scene_record(scene).items():
        out["scene_" + k] = v
    sim = O.RefSim(scene, seed=SEED)
    for k, v in sim.get_state().items():
        out["init_" + k] = v
    for idx, st in enumerate(stage_order(scene)):
        sim.stage(st)
        for k, v in sim.get_state().items():
            out[f"s{idx}_post_{k}"] = v
    stats = [sim.stats()]
    frame = 1
    if 1 in FRAMES_SAVED:
        for k, v in sim.get_state().items():
            out[f"f1_{k}"] = v
        out["stats_f1"] = np.array(list(stats[-1].values()))
    while frame < FRAMES:
        sim.frame()
        frame += 1
        if frame in FRAMES_SAVED:
            for k, v in sim.get_state().items():
                out[f"f{frame}_{k}"] = v
            out[f"stats_f{frame}"] = np.array(list(sim.stats().values()))
    sim.close()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)


STATS_FRAMES = 45
STATS_SEED = 4242


def generate_stats_csv():
    """stats_csv.npz: the reference's own saveStats output (perf.csv and
    conservation.csv, src/FluidSim2D.cpp:738-750 and
    src/PerformanceCounter.cpp:39-74) for seeded series fed through its
    PerformanceCounter, for both modes (7 and 8 stages), with the inputs."""
    import tempfile
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import golden_util

    out = {}
    for tag, scene in (("sl", scenes.sl_dam_break(16)), ("pic", scenes.pic_dam_break_disk(16))):
        stages = 7 if tag == "sl" else 8
        ms, vol, en, pen = golden_util.stats_series(STATS_SEED + stages, STATS_FRAMES, stages)
        sim = O.RefSim(scene, seed=1)
        with tempfile.TemporaryDirectory() as d:
            perf, cons = sim.save_stats_of(ms, vol, en, pen, d)
        sim.close()
        out.update({f"{tag}_stage_ms": ms, f"{tag}_vol": vol, f"{tag}_en": en, f"{tag}_pen": pen,
                    f"{tag}_perf": np.frombuffer(perf, np.uint8), f"{tag}_cons": np.frombuffer(cons, np.uint8)})
    np.savez_compressed(os.path.join(HERE, "stats_csv.npz"), **out)


def main():
    build_oracle.build_reference()
    if O.get_reference_lib() is None:
        raise SystemExit("reference checkout not available (set FS2D_REFERENCE_DIR); golden vectors cannot be "
                         "regenerated")
    if sys.argv[1:] == ["stats"]:
        generate_stats_csv()
        print("wrote stats_csv")
        return
    for name, scene in golden_scenes().items():
        generate(name, scene)
        print("wrote", name)
    generate_stats_csv()
    print("wrote stats_csv")


if __name__ == "__main__":
    main()
