"""Generates the golden fixtures of the terrace from the UNMODIFIED reference CPU step (oracle/_ref/libswarm_ref.so,
compiled from the reference tree by oracle/Makefile). Run in a container that has the reference tree:

    make -C oracle ref && python tests/golden/make_golden.py

Writes
  stadium_sdf.zlib   the reference's stadium.sdf (130^3 float32, the terrace's baked SDF), zlib-compressed: the input
                     data of the terrace venue, needed where the reference tree is absent
  terrace_ref.npz    spawnBleacherCrowd(4096, seed 1337) (src/crowd_sim.cpp:601-645, this platform's libstdc++
                     distributions), and CpuCrowdSim (SortMode::Counting) after 1 step (state, sorted pairs, cell table,
                     contact bits), after 250 steps (state and its FNV-1a hash, tools/golden_state.hpp:121-126) and after
                     251 steps (one step from the congested state: state, pairs, cells, contacts).
  terrace_metrics_ref.npz  the terrace's metric cell table (computeMetricVenue: threshold masses, walkable area) and
                     MetricsReference (src/metrics.cpp:429-476) after recording the first 250 steps from the spawn:
                     counters, per-cell accumulators, evacuation step per agent.
  terrace_evac_ref.npz  the same spawn run by the reference to full evacuation: the active agents after every step,
                     and the evacuation time (the first step after which none is active).
"""
import os
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))
from oracle import oracle as O  # noqa: E402

def main():
    O.build(ref=True)
    ref_dir = O.ref_dir()
    assert ref_dir, "the reference tree is needed: REF_DIR=<tree> make -C oracle ref"
    sdf_path = os.path.join(ref_dir, "stadium.sdf")
    raw = open(sdf_path, "rb").read()
    with open(os.path.join(HERE, "stadium_sdf.zlib"), "wb") as f:
        f.write(zlib.compress(raw, 9))
    assert O.ref_load_sdf(sdf_path)
    spawn = O.ref_spawn_terrace(4096, 1337)
    sim = O.RefSim("terrace")
    sim.set_state(spawn)
    sim.step(1)
    out = {"spawn": spawn, "state1": sim.state(), "contacts1": sim.contacts(), "cells1": sim.cells()}
    out["grid1_key"], out["grid1_id"] = sim.grid()
    sim.step(249)
    out["state250"] = sim.state()
    sim.step(1)
    out["state251"] = sim.state()
    out["contacts251"] = sim.contacts()
    out["cells251"] = sim.cells()
    out["grid251_key"], out["grid251_id"] = sim.grid()
    out["hash250"] = np.array([O.state_hash(out["state250"])], dtype=np.uint64)
    np.savez_compressed(os.path.join(HERE, "terrace_ref.npz"), **out)

    thr, area = O.ref_terrace_metric_cells()
    met = O.RefMetrics(4096, thr)
    sim = O.RefSim("terrace")
    sim.set_state(spawn)
    prev = spawn
    for _ in range(250):
        sim.step(1)
        cur = sim.state()
        met.record(prev, cur)
        prev = cur
    ctr, cells, evac = met.read()
    np.savez_compressed(os.path.join(HERE, "terrace_metrics_ref.npz"), threshold_mass=thr, walkable_m2=area,
                        counters=ctr, cells=cells, evac_step=evac)
    print("metrics: %d evacuated, exits %s" % (ctr[2], list(ctr[4:9])))

    sim = O.RefSim("terrace")
    sim.set_state(spawn)
    active = []
    while not active or active[-1] > 0:
        sim.step(1)
        active.append(int((sim.state()[:, 3] != 0).sum()))
        if len(active) > 20000:
            raise RuntimeError("the terrace did not evacuate in 20 000 steps")
    np.savez_compressed(os.path.join(HERE, "terrace_evac_ref.npz"), active=np.array(active, np.int32),
                        evacuation_steps=np.array([len(active)], np.int32))
    print("terrace evacuated after %d steps" % len(active))
    print("hash after 250 steps: %016x" % int(out["hash250"][0]))


if __name__ == "__main__":
    main()
