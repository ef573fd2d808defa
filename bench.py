"""Benchmark of the crowd step: agent-steps/s on the 65 536-agent hall, against the HBM roofline.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--no-cpu-baseline]

Workload: the hall 140 m x 140 m with four 4 m exits, 65 536 agents on a 256 x 256 lattice at 0.5 m (jitter 0.05 m,
radius U[0.20, 0.25] m, desired speed N(1.34, 0.26) clipped to [0.6, 2.0] m/s, seed 0), dt 0.05 s, K = 8 Jacobi
sweeps, 0.5 m hash cells; synthetic data generated here. One step = hash, key sort, cell ranges + gather, predict,
7 sweeps, final pass over every agent.

value  agent-steps/s with the state resident in HBM: per timed step, CUDA events on the simulation's stream around
       the step; the L2 (129 MB, larger than the step's 54 MB working set) is flushed by a 256 MiB write before each
       timed step, outside the events. Agent-steps count the agents active at the start of each step.
e2e    the same metric through swarm_step_host: host state in pinned memory -> device, one step, device -> host,
       every step inside the timed region.
roofline  the dominant kernel's algorithmic bytes per launch (bytes per agent x active agents) over its mean launch
       time (the fused step is one launch: the timed steps' own CUDA events, stage timing off; with --phase-kernels
       the library's per-stage events on a replay of the same steps), against the measured HBM copy bandwidth
       (MEASURED_PEAKS.json). details.stage_ms_mean: the in-kernel stage times of that replay (stage timing on).
cpu_baseline  the oracle port of the reference's CPU step (OpenMP, all host threads) on a fixed sample of the same
       workload (400 consecutive steps after 2 warm-up steps from the spawn), with the host's core count and CPU model.
batched  the 256-instance batch as one packed state against the same instances launched one at a time.
bowl   the 63 488-agent seated bowl: the plain step (as value) and its evacuation run to completion.
reference_venue_L  the reference's own seated venue L (63 424 agents) with the reference's constants (K = 32), beside
       the reference's published GPU step on that venue (from the spawn and congested).
reference_venue_S  venue S under the reference's default model (its queue-aware exit choice on its own table, the
       incline speed and stair spacing), from the spawn and congested, beside the reference's published GPU step.
reference_terrace  the reference's baked terrace (4 096 agents, K = 32) from the spawn and congested, beside the
       reference's published GPU step on it.
adjoint  loss and gradient of 400 steps of the 16 384-agent hall (checkpoints every 20 steps, and the full tape)
       against the plain forward of the same steps.
--impl reference  the reference's CPU step (the oracle port: the reference's own build needs its source tree, which
       only exists where the oracle was pinned) on the host cores, same workload, config, metric and unit, timed over
       the same 400-step sample as cpu_baseline; the workload is built by the oracle library, so that process never
       maps the CUDA library.
"""
import argparse
import json

import numpy as np
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "swarm-crowd-simulation_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "agent-steps/s vs HBM roofline: plain, 256-batched, adjoint (≤1e-3 FD rel err)"
UNIT = "agent-steps/s"
WORKLOAD = ("hall 140x140 m, 4 exits of 4 m, 65536 agents (256x256 lattice, 0.5 m), per-agent radius and v0, "
            "dt 0.05 s, K=8 Jacobi sweeps, 0.5 m hash cells, FP32")
# algorithmic bytes per active agent per launch (SoA FP32): predict reads pos, vel, params (48) and writes the
# predicted position, velocity and wall plane (48); a sweep reads position and plane (32) and writes a position (16);
# the final pass reads 64 and writes the 32-byte agent record; the sort stage: hash 24 + sort 16 + ranges 4 + gather 100
BYTES = {"predict": 96.0, "sweep": 48.0, "final": 96.0, "sort": 144.0}
B_STEP = 336.0 + 48.0 * (8 - 1)   # 672 B per agent-step at K = 8
CONGESTED_STEPS = 250             # the reference benchmark's congested state (tools/benchmark/bench_common.hpp)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampled every 200 ms during the timed region."""

    def __init__(self, index=0):
        self.rows = []
        self.proc = None
        self.index = index

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 4 + i and r[4 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def workload():
    from swarm_gb300 import venues
    return venues.hall_c1()


def bench_batched(P, steps=10, warmup=3):
    """The 256-instance batch (N log-uniform in [1 024, 65 536], 1-2 exits of U[1.5, 6] m, halls sized to 4 agents/m^2,
    independent seeds) as one packed state, against the same instances launched one at a time. Both sides run the
    same steps from the same states (the results are bit-identical), so agent-steps are the same: the speed-up is
    the time ratio. The batch's working set (3.8 M agents, 2.1 GB of venue fields) is far larger than L2."""
    import torch
    import swarm_gb300
    from swarm_gb300 import venues
    vens, boids, r, v0, counts = venues.build_batch(256, 0)
    n = int(counts.sum())
    stream = torch.cuda.Stream()
    batch = swarm_gb300.BatchSim(P, vens, counts)
    batch.set_stream(stream.cuda_stream)
    batch.set_state(boids)
    batch.set_agent_params(r, v0)
    tuning = batch.autotune(steps=2)
    batch.set_graph(True)   # single steps replay the fused launch from a CUDA graph
    dev = torch.empty((n, 8), dtype=torch.float32, device="cuda")
    with torch.cuda.stream(stream):
        for _ in range(warmup):
            batch.step(1)
    torch.cuda.synchronize()
    start = batch.state()
    active, t_batch = 0, 0.0
    for _ in range(steps):
        batch.download_device(dev.data_ptr())
        active += int((dev[:, 3] != 0).sum().item())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            batch.step(1)
            e1.record(stream)
        stream.synchronize()
        t_batch += e0.elapsed_time(e1)
    # the same steps chained: one persistent launch runs them all, a grid barrier between steps (the working set is far
    # larger than L2 either way)
    batch.set_state(start)
    torch.cuda.synchronize()
    c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        c0.record(stream)
        batch.step(steps)
        c1.record(stream)
    stream.synchronize()
    t_chain = c0.elapsed_time(c1)
    batch.synchronize()
    batch.close()
    # one at a time: each instance its own handle, all on one stream, stepped in turn
    solos = []
    for i, v in enumerate(vens):
        a, b = int(np.sum(counts[:i])), int(np.sum(counts[:i + 1]))
        sim = swarm_gb300.CrowdSim(P, v, b - a)
        sim.set_stream(stream.cuda_stream)
        sim.set_state(start[a:b])
        sim.set_agent_params(r[a:b], v0[a:b])
        solos.append(sim)
    for _ in range(2):
        for sim in solos:
            sim.step(1)
    torch.cuda.synchronize()
    for i, sim in enumerate(solos):   # back to the same start
        a, b = int(np.sum(counts[:i])), int(np.sum(counts[:i + 1]))
        sim.set_state(start[a:b])
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        for sim in solos:
            sim.step(1)
    e1.record(stream)
    e1.synchronize()
    t_solo = e0.elapsed_time(e1)
    for sim in solos:
        sim.close()
    return {"workload": "256 halls, N log-uniform [1024, 65536] (total %d agents), 1-2 exits U[1.5, 6] m, seed 0" % n,
            "value": active / (t_batch * 1e-3), "unit": UNIT, "ms_per_step": t_batch / steps,
            "chained": {"value": active / (t_chain * 1e-3), "ms_per_step": t_chain / steps, "launches": 1,
                        "fraction_of_hbm_roofline": active / (t_chain * 1e-3) * B_STEP / (peaks()[0] * 1e9)},
            "one_at_a_time": {"value": active / (t_solo * 1e-3), "ms_per_step": t_solo / steps,
                              "launches_per_step": len(vens)},
            "speedup_vs_one_at_a_time": t_solo / t_batch, "tuning": tuning,
            "fraction_of_hbm_roofline": active / (t_batch * 1e-3) * B_STEP / (peaks()[0] * 1e9)}


def bench_bowl(P, steps=50, warmup=5, cap=20000, chunk=100, evacuation=True):
    """The seated bowl (32 sectors x 32 rows x 62 seats = 63 488 agents; stairs, vomitories, perimeter exits): the
    plain step timed as the main workload (CUDA events per step on the handle's stream, the L2 flushed by a 256 MiB
    write before each), then the evacuation run from the seats (checked every `chunk` steps): the steps until 99.9 %
    of the crowd is out, and how many are left after `cap` steps (a few agents end in symmetric standoffs at gangway
    feet that the deterministic model never breaks)."""
    import torch
    import swarm_gb300
    from swarm_gb300 import venues
    venue, (boids, r, v0) = venues.bowl_c2()
    n = boids.shape[0]
    stream = torch.cuda.Stream()
    sim = swarm_gb300.CrowdSim(P, venue, n)
    sim.set_stream(stream.cuda_stream)
    sim.set_state(boids)
    sim.set_agent_params(r, v0)
    sim.set_graph(True)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    with torch.cuda.stream(stream):
        sim.step(warmup)
    torch.cuda.synchronize()
    active, total_ms = 0, 0.0
    for k in range(steps):
        active += int((sim.state()[:, 3] != 0).sum())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            flush.fill_(k & 0xFF)
            e0.record(stream)
            sim.step(1)
            e1.record(stream)
        stream.synchronize()
        total_ms += e0.elapsed_time(e1)
    value = active / (total_ms * 1e-3)
    if not evacuation:   # the timed steps alone (a profiling run)
        sim.close()
        return {"value": value, "unit": UNIT, "ms_per_step": total_ms / steps, "steps": steps, "warmup": warmup,
                "fraction_of_hbm_roofline": value * B_STEP / (peaks()[0] * 1e9)}
    # the evacuation from the seats, through the headless runner (active counts kept on the device every step)
    sim.set_state(boids)
    t0 = time.perf_counter()
    ev, active = sim.run_evacuation(cap)
    wall_s = time.perf_counter() - t0
    out999 = np.nonzero(active <= n // 1000)[0]
    t999 = int(out999[0]) + 1 if out999.size else None
    # the queue-aware exit choice: the 40 exits' own fields (GPU solver), then the step with the choice pass (same
    # per-step timing) and the evacuation
    prev = swarm_gb300.set_nav_solver("gpu")
    t0 = time.perf_counter()
    fields, widths, types = venues.exit_fields(venue)
    fields_s = time.perf_counter() - t0
    swarm_gb300.set_nav_solver(prev)
    sim.set_exit_choice(fields, widths, types)
    del fields
    sim.set_state(boids)
    with torch.cuda.stream(stream):
        sim.step(warmup)
    torch.cuda.synchronize()
    qa_active, qa_ms = 0, 0.0
    for k in range(steps):
        qa_active += int((sim.state()[:, 3] != 0).sum())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            flush.fill_(k & 0xFF)
            e0.record(stream)
            sim.step(1)
            e1.record(stream)
        stream.synchronize()
        qa_ms += e0.elapsed_time(e1)
    sim.set_state(boids)
    t0 = time.perf_counter()
    qev, qactive = sim.run_evacuation(cap)
    qwall_s = time.perf_counter() - t0
    q999 = np.nonzero(qactive <= n // 1000)[0]
    qt999 = int(q999[0]) + 1 if q999.size else None
    _, counters = sim.exit_choice()
    sim.close()
    queue_aware = {"exits": int(widths.shape[0]), "fields_s": fields_s,
                   "value": qa_active / (qa_ms * 1e-3), "unit": UNIT, "ms_per_step": qa_ms / steps,
                   "evacuation": {"t50_s": qev["t50_s"], "t90_s": qev["t90_s"], "t100_s": qev["t100_s"],
                                  "steps_to_99.9pct": qt999,
                                  "seconds_to_99.9pct": None if qt999 is None else qt999 * float(P.dt),
                                  "left_after": {"steps": qev["steps"], "agents": qev["remaining"]}, "wall_s": qwall_s,
                                  "counters": {"evaluations": int(counters[0]), "eligible": int(counters[1]),
                                               "switches": int(counters[2]), "forced": int(counters[3])}}}
    return {"workload": "seated bowl, 32 sectors x 32 rows x 62 seats (63488 agents), seat 0.5 m, row pitch 0.8 m, "
                        "rise 0.4 m, 1.2 m gangway stairs (speed factor 0.6), 2.4 m vomitories at row 16, 8 perimeter "
                        "exits of 4 m; wall SDF 0.05 m, nav 0.1 m",
            "value": value, "unit": UNIT, "ms_per_step": total_ms / steps, "steps": steps, "warmup": warmup,
            "fraction_of_hbm_roofline": value * B_STEP / (peaks()[0] * 1e9),
            "evacuation": {"t50_s": ev["t50_s"], "t90_s": ev["t90_s"], "t100_s": ev["t100_s"],
                           "steps_to_99.9pct": t999, "seconds_to_99.9pct": None if t999 is None else t999 * float(P.dt),
                           "left_after": {"steps": ev["steps"], "agents": ev["remaining"]}, "wall_s": wall_s,
                           "path": "swarm_run_evacuation (C ABI)"},
            "queue_aware_exit_choice": queue_aware,
            "nav_field": bench_nav_field(venue)}


def _timed_steps(sim, stream, flush, steps):
    """CUDA events per step on the handle's stream, the L2 flushed by a 256 MiB write before each step (outside the
    events); returns (agent-steps: the agents active at the start of each step, total ms)."""
    import torch
    active, total = 0, 0.0
    for k in range(steps):
        active += int((sim.state()[:, 3] != 0).sum())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            flush.fill_(k & 0xFF)
            e0.record(stream)
            sim.step(1)
            e1.record(stream)
        stream.synchronize()
        total += e0.elapsed_time(e1)
    return active, total


def _congest(sim, stream, chunk=10, cap=20000):
    """Steps until at most half the agents that were active at the start remain (the reference's "congested" state,
    checked every `chunk` steps); returns (steps taken, agents active)."""
    import torch
    start = int((sim.state()[:, 3] != 0).sum())
    done = 0
    while done < cap:
        with torch.cuda.stream(stream):
            sim.step(chunk)
        done += chunk
        left = int((sim.state()[:, 3] != 0).sum())
        if 2 * left <= start:
            return done, left
    return done, left


def _seated_golden(name):
    import zlib
    from swarm_gb300 import venues
    g = dict(np.load(os.path.join(ROOT, "tests", "golden", "seated_%s.npz" % name)))
    delta = np.frombuffer(zlib.decompress(g["nav_anchor_delta_z"].tobytes()), np.int32)
    info = np.frombuffer(zlib.decompress(g["nav_info_z"].tobytes()), np.uint32)
    cells = venues.nav_cells_from_anchors(np.cumsum(delta.astype(np.int64)), info, g["nav_grid"])
    return g, cells, info


def bench_venue_l(steps=30, warmup=5):
    """The reference's own largest venue in reference-parity mode: seated venue L (63 424 seats in N = 65 536; the
    reference's layout, navigation field and full seat spawn from tests/golden/seated_L.npz, written by the unmodified
    reference), the reference's constants (model units, K = 32: 31 sweeps and the final pass), nearest exit at the level
    speed, and again with the incline speed and stair spacing; both from the spawn and, for the first, again once half
    the crowd has left (the reference's "congested" state). CUDA events per step on the handle's stream, the L2
    flushed by a 256 MiB write before each step. The reference publishes its own GPU step on this venue and spawn
    (OpenGL on an AMD RX 7800 XT, its default model): 1.861 ms a step from the spawn, 3.928 ms congested, of which
    0.2039 / 0.4564 ms is its queue-aware exit choice (results/benchmarks/thesis/perf_tables.md:17-18, :45-46) -- a
    pass not run on L here (its 904 MB candidate table is not part of the fixtures; venue S runs it)."""
    import zlib
    import torch
    import swarm_gb300
    from swarm_gb300 import venues
    g, cells, _ = _seated_golden("L")
    spawn = np.frombuffer(zlib.decompress(g["spawn_z"].tobytes()), np.float32).reshape(-1, 8).copy()
    gr = g["grid"]
    P = swarm_gb300.params_reference()
    K = P.proj_iterations
    b_step = 336.0 + 48.0 * (K - 1)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    out = {"workload": "reference venue L (63424 seated of 65536), reference constants (model units, K=32), full seat "
                       "spawn (seed 1337)", "agents": int(spawn.shape[0]), "bytes_per_agent_step": b_step,
           "published_reference_gpu": {"ms_per_step": 1.861, "exit_choice_ms": 0.2039, "congested_ms_per_step": 3.928,
                                       "congested_exit_choice_ms": 0.4564,
                                       "hardware": "AMD RX 7800 XT, OpenGL 4.3 (published, not measured here)"}}
    for label, incline in (("nearest_exit_level_speed", False), ("incline_speed_stair_spacing", True)):
        inc = g["incline"]
        venue = venues.Venue.seated(g["layout"], int(gr[0]), gr[1], gr[2], gr[3], gr[4], nav_cells=cells,
                                    nav_grid=g["nav_grid"], incline_speed=incline,
                                    stair_times=(inc[4], inc[5]) if incline else None, name="L")
        stream = torch.cuda.Stream()
        sim = swarm_gb300.CrowdSim(P, venue, spawn.shape[0])
        sim.set_stream(stream.cuda_stream)
        sim.set_state(spawn)
        with torch.cuda.stream(stream):
            sim.step(warmup)
        torch.cuda.synchronize()
        active, total = _timed_steps(sim, stream, flush, steps)
        value = active / (total * 1e-3)
        out[label] = {"value": value, "unit": UNIT, "ms_per_step": total / steps, "steps": steps, "warmup": warmup,
                      "fraction_of_hbm_roofline": value * b_step / (peaks()[0] * 1e9)}
        if not incline:
            taken, left = _congest(sim, stream)
            active, total = _timed_steps(sim, stream, flush, steps)
            value = active / (total * 1e-3)
            out[label]["congested"] = {"value": value, "unit": UNIT, "ms_per_step": total / steps, "steps": steps,
                                       "after_steps": warmup + steps + taken, "active_agents": left}
        sim.synchronize()
        sim.close()
    return out


def bench_venue_s(steps=30, warmup=5):
    """The reference's venue S under its default model -- the queue-aware exit choice on the reference's own candidate
    table (tests/golden/seated_S_choice.npz), the incline speed and the stair spacing (EMPIRICAL) --, the model whose
    250-step state the tests pin to the reference's hash: the full seat spawn (3 728 agents in N = 4 096), the
    reference's constants, from the spawn and once half the crowd has left. Each timed step is the choice pass's
    kernels and the step, CUDA events, the L2 flushed before each. The reference publishes its GPU step on this venue
    and model (AMD RX 7800 XT): 0.6775 ms from the spawn, 1.278 ms congested, of which 0.0925 / 0.1777 ms is the exit
    choice (results/benchmarks/thesis/perf_tables.md:13-14, :41-42)."""
    import torch
    import swarm_gb300
    from swarm_gb300 import venues
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from seated_choice import choice_index, decode_choice_entries
    g, cells, info = _seated_golden("S")
    c = dict(np.load(os.path.join(ROOT, "tests", "golden", "seated_S_choice.npz")))
    meta = c["choice_meta"]
    gr, inc = g["grid"], g["incline"]
    venue = venues.Venue.seated(g["layout"], int(gr[0]), gr[1], gr[2], gr[3], gr[4], nav_cells=cells,
                                nav_grid=g["nav_grid"], incline_speed=True, stair_times=(inc[4], inc[5]), name="S")
    spawn = g["nearest_spawn"]
    stream = torch.cuda.Stream()
    sim = swarm_gb300.CrowdSim(swarm_gb300.params_reference(), venue, spawn.shape[0])
    sim.set_stream(stream.cuda_stream)
    sim.set_seated_choice(choice_index(info), decode_choice_entries(c), meta[3:3 + int(meta[0])], float(meta[1]),
                          float(meta[2]), int(c["choice_grid"][2]))
    sim.set_state(spawn)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    with torch.cuda.stream(stream):
        sim.step(warmup)
    torch.cuda.synchronize()
    out = {"workload": "reference venue S (3728 seated of 4096), reference default model (queue-aware exit choice, "
                       "incline speed, stair spacing EMPIRICAL), reference constants (K=32), full seat spawn (seed 1337)",
           "published_reference_gpu": {"ms_per_step": 0.6775, "exit_choice_ms": 0.0925, "congested_ms_per_step": 1.278,
                                       "congested_exit_choice_ms": 0.1777,
                                       "hardware": "AMD RX 7800 XT, OpenGL 4.3 (published, not measured here)"}}
    active, total = _timed_steps(sim, stream, flush, steps)
    out["spawn"] = {"value": active / (total * 1e-3), "unit": UNIT, "ms_per_step": total / steps, "steps": steps,
                    "warmup": warmup}
    taken, left = _congest(sim, stream)
    active, total = _timed_steps(sim, stream, flush, steps)
    out["congested"] = {"value": active / (total * 1e-3), "unit": UNIT, "ms_per_step": total / steps, "steps": steps,
                        "after_steps": warmup + steps + taken, "active_agents": left}
    sim.synchronize()
    sim.close()
    return out


def bench_terrace(steps=30, warmup=5):
    """The reference's own terrace in reference-parity mode: its baked venue (stadium.sdf, the pitch fence, the egress
    router; tests/golden/stadium_sdf.zlib), 4 096 agents from the reference's bleacher spawn as its CPU build draws it on
    this platform (tests/golden/terrace_ref.npz; the reference's published run drew its spawn with another standard
    library), the reference's constants (model units, K = 32), from the spawn and once half the crowd has left. CUDA
    events per step on the handle's stream, the L2 flushed before each step. The reference publishes its GPU step on
    this venue at N = 4 096 from the spawn (OpenGL on an AMD RX 7800 XT): 0.7239 ms
    (results/benchmarks/thesis/perf_tables.md:28)."""
    import zlib
    import torch
    import swarm_gb300
    from swarm_gb300.venues import Venue
    golden = os.path.join(ROOT, "tests", "golden")
    sdf = np.frombuffer(zlib.decompress(open(os.path.join(golden, "stadium_sdf.zlib"), "rb").read()), np.float32).copy()
    spawn = np.load(os.path.join(golden, "terrace_ref.npz"))["spawn"]
    stream = torch.cuda.Stream()
    sim = swarm_gb300.CrowdSim(swarm_gb300.params_reference(), Venue.stadium(sdf), spawn.shape[0])
    sim.set_stream(stream.cuda_stream)
    sim.set_state(spawn)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    with torch.cuda.stream(stream):
        sim.step(warmup)
    torch.cuda.synchronize()
    out = {"workload": "reference terrace (stadium.sdf), 4096 agents from the reference's bleacher spawn, reference "
                       "constants (model units, K=32)",
           "published_reference_gpu": {"ms_per_step": 0.7239,
                                       "hardware": "AMD RX 7800 XT, OpenGL 4.3 (published, not measured here)"}}
    active, total = _timed_steps(sim, stream, flush, steps)
    out["spawn"] = {"value": active / (total * 1e-3), "unit": UNIT, "ms_per_step": total / steps, "steps": steps,
                    "warmup": warmup}
    taken, left = _congest(sim, stream)
    active, total = _timed_steps(sim, stream, flush, steps)
    out["congested"] = {"value": active / (total * 1e-3), "unit": UNIT, "ms_per_step": total / steps, "steps": steps,
                        "after_steps": warmup + steps + taken, "active_agents": left}
    sim.synchronize()
    sim.close()
    return out


def bowl_venue():
    """The seated bowl's venue alone (its nav grid is the solver's workload)."""
    from swarm_gb300 import venues
    return venues.bowl_c2()[0]


def bench_nav_field(venue, clearance=0.2):
    """The navigation-field solver on the bowl's nav grid (3931 x 3931 nodes at 0.1 m; walls where the wall SDF is
    within the clearance, sources at the exit mask, the stair speed factors): host fast marching against the GPU
    solver (wall-clock per call, uploads and downloads included; the GPU's second call), and whether the floats agree."""
    import swarm_gb300
    v = venue.struct
    step = int(round(v.nav_h / v.wall_h))
    wall = venue.arrays["wall"].reshape(v.wall_ny, v.wall_nx)[::step, ::step][:v.nav_ny, :v.nav_nx]
    speed = venue.arrays["speed"].reshape(v.wall_ny, v.wall_nx)[::step, ::step][:v.nav_ny, :v.nav_nx]
    mask = venue.arrays["exit_mask"].reshape(v.nav_ny, v.nav_nx)
    kind = np.where(wall <= clearance, 3, np.where(mask != 0, 1, 0)).astype(np.uint8)
    t0 = time.perf_counter()
    cpu, _ = swarm_gb300.nav_field(kind, v.nav_h, speed=speed, solver="cpu")
    cpu_ms = (time.perf_counter() - t0) * 1e3
    swarm_gb300.nav_field(kind, v.nav_h, speed=speed, solver="gpu")
    t0 = time.perf_counter()
    gpu, st = swarm_gb300.nav_field(kind, v.nav_h, speed=speed, solver="gpu")
    gpu_ms = (time.perf_counter() - t0) * 1e3
    return {"grid": f"{v.nav_nx}x{v.nav_ny}", "cpu_fast_marching_ms": cpu_ms, "gpu_ms": gpu_ms,
            "speedup": cpu_ms / gpu_ms, "gpu_solve_ms": st["ms_solve"], "passes": st["passes"], "tile_runs": st["tile_runs"], "tiles": st["tiles"],
            "equal_to_fast_marching": bool(np.array_equal(cpu.view(np.uint32), gpu.view(np.uint32)))}


def adjoint_bytes(K, steps, ckpt, kept=1):
    """Algorithmic bytes per agent-step of the adjoint with checkpoints every `ckpt` steps, the last `kept` segments
    taped in the checkpoint pass: the forward work (2T - kept x C steps of B_step) plus the tape (written once, read once: per agent (2K + 6) float4 of positions, velocities,
    planes, the predict record and the sweeps' corrections, and 17 B of params, ids and contact bits) plus the
    reverse's own traffic (the state adjoint read and written, 64 B; each sweep's correction-sum adjoint written and
    read, 16 B; the per-slot adjoints of the final pass, predict and gather, 7 x 16 + 4 B)."""
    b_step = 336.0 + 48.0 * (K - 1)
    forward = b_step * (2.0 * steps - min(kept * ckpt, steps)) / steps
    tape = 2.0 * ((2 * K + 6) * 16.0 + 17.0)
    reverse = 64.0 + 16.0 * K + 7 * 16.0 + 4.0
    return forward + tape + reverse


def bench_adjoint(P, steps=400, ckpt=20):
    """The adjoint on the 16 384-agent hall (80 m x 70 m, two 4 m exits, 128 x 128 lattice at 0.5 m, seed 0): the
    loss L = dt * sum_t sum_i D(p_i(t)) of 400 steps from the spawn and its gradient with respect to every agent's
    desired speed and radius and the relaxation time, checkpoints every 20 steps (the default tape budget keeps the
    last segments' tapes from the checkpoint pass; `pure_recompute`: budget 0, every other segment recomputed). Against
    the plain forward of the same 400 steps. Both timed with CUDA events on the handle's stream (inputs larger than L2 are not at stake: the
    working set, 16 384 agents, is L2-resident on both sides)."""
    import torch
    import swarm_gb300
    from swarm_gb300 import venues
    venue, (boids, r, v0) = venues.terrace_c4()
    n = boids.shape[0]
    stream = torch.cuda.Stream()
    sim = swarm_gb300.CrowdSim(P, venue, n)
    sim.set_stream(stream.cuda_stream)
    sim.set_agent_params(r, v0)
    # agent-steps: the agents active at the start of each of the 400 steps
    sim.set_state(boids)
    active = 0
    for _ in range(steps):
        active += int((sim.state()[:, 3] != 0).sum())
        sim.step(1)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    sim.set_state(boids)
    sim.step(3)
    sim.set_state(boids)
    torch.cuda.synchronize()
    e0.record(stream)
    sim.step(steps)
    e1.record(stream)
    e1.synchronize()
    fwd_ms = e0.elapsed_time(e1)
    out = {"workload": "hall 80x70 m, 2 exits of 4 m, 16384 agents (128x128 lattice, 0.5 m), 400 steps from the "
                       "spawn, loss dt*sum_t sum_i D(p_i(t)), gradient wrt v0_i, r_i, tau",
           "steps": steps, "agent_steps": active, "forward_ms_per_step": fwd_ms / steps}
    for c, budget in ((ckpt, None), (ckpt, 0), (steps, None)):
        sim.set_adjoint_tape_budget(1 << 30 if budget is None else budget)
        sim.set_state(boids)
        sim.adjoint(steps, c)   # allocation and warm-up
        torch.cuda.synchronize()
        e0.record(stream)
        L, gv, gr, gt, st = sim.adjoint(steps, c, stats=True)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        value = active / (ms * 1e-3)
        b = adjoint_bytes(P.proj_iterations, steps, c, st["kept_segments"])
        rec = {"ckpt_every": c, "segments": st["segments"], "kept_segments": st["kept_segments"],
               "tape_budget_bytes": 1 << 30 if budget is None else budget,
               "value": value, "unit": UNIT, "ms_per_step": ms / steps,
               "ratio_vs_forward": ms / fwd_ms, "loss": L, "dL_dtau": gt,
               "bytes_per_agent_step": b, "fraction_of_hbm_roofline": value * b / (peaks()[0] * 1e9),
               "tape_bytes": st["tape_bytes"], "launches": st["launches"],
               "ms": {k: round(st[k], 3) for k in ("ms_checkpoint", "ms_recompute", "ms_reverse", "ms_rev_final",
                                                   "ms_rev_sweeps", "ms_rev_predict", "ms_rev_gather")}}
        if c == ckpt and budget is None:
            out.update(rec)
        elif c == ckpt:
            out["pure_recompute"] = rec
        else:
            out["full_tape"] = rec
    sim.close()
    return out


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo), for the baseline's record."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.processor() or platform.machine()


CPU_SAMPLE_STEPS = 400   # the CPU sample: this many consecutive steps of the workload from its spawn


def cpu_baseline(warmup=2, steps=CPU_SAMPLE_STEPS):
    """The oracle port of the reference's CPU step (OpenMP, every host thread) on the same workload: `warmup` steps
    from the spawn, then `steps` consecutive steps timed one by one (wall clock), agent-steps counted per step. The
    workload is built by the oracle library's host build of the venue builders, so this process never loads the CUDA
    library."""
    import swarm_gb300
    from oracle import oracle as O
    O.build()
    swarm_gb300.use_generator(O.lib())
    venue, (boids, r, v0) = workload()
    sim = O.OracleSim(swarm_gb300.params_si(), venue.struct)
    sim.set_state(boids)
    sim.set_agent_params(r, v0)
    sim.step(warmup)
    agent_steps, t_total = 0, 0.0
    for _ in range(steps):
        active = int((sim.state()[:, 3] != 0).sum())
        t0 = time.perf_counter()
        sim.step(1)
        t_total += time.perf_counter() - t0
        agent_steps += active
    threads = O.lib().oracle_max_threads()
    return {"value": agent_steps / t_total, "unit": UNIT, "cores": threads, "cpu_model": cpu_model(), "kind": "port",
            "sample": f"{steps} consecutive steps of the 65536-agent hall after {warmup} warm-up steps from its spawn, "
                      f"{t_total:.1f} s of wall clock on {threads} OpenMP threads",
            "ms_per_step": t_total / steps * 1e3}


def bench_config(n, world):
    """The workload record both arms print (the same dict: the same workload)."""
    return {"workload": WORKLOAD, "agents": n, "sweeps": 8, "dt_s": 0.05,
            "l2": "GPU arm: flushed before every timed step (256 MiB write, outside the timed events)",
            "parallelism": f"replicas x{world}" if world > 1 else "1 GPU"}


def replica_totals(dist, device, ms, agent_steps):
    """The whole job over the ranks (replicas): the slowest rank's time and every rank's agent-steps. `dist` is
    torch.distributed (None: one process); `device` holds the reduction tensors ("cuda" for NCCL, "cpu" for gloo)."""
    if dist is None:
        return float(ms), float(agent_steps)
    import torch
    t = torch.tensor([float(ms)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    a = torch.tensor([float(agent_steps)], device=device, dtype=torch.float64)
    dist.all_reduce(a)
    return float(t.item()), float(a.item())


def run_reference(args, rank, world):
    """The reference arm: the reference's CPU step (the oracle port; the reference's own build needs its source tree,
    absent where the benchmark runs) on the host cores, the same workload, metric and unit. Each run times the same
    fixed sample (CPU_SAMPLE_STEPS steps after args.warmup warm-up steps), whatever --steps asks, so that its number
    does not depend on a short sample; rank 0 alone runs under torchrun."""
    if rank != 0:
        return 0
    base = cpu_baseline(warmup=args.warmup)
    line = {"impl": "reference", "metric": METRIC, "value": base["value"], "unit": UNIT, "n_gpus": args.gpus,
            "steps": CPU_SAMPLE_STEPS, "warmup": args.warmup, "ms_per_step": base["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (generated hall and lattice spawn, seed 0)",
            "config": bench_config(65536, world), "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--phase-kernels", action="store_true", help="one kernel per phase instead of the fused step")
    ap.add_argument("--no-batch", action="store_true", help="skip the 256-instance batched measurement")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint measurement")
    ap.add_argument("--no-bowl", action="store_true", help="skip the seated-bowl measurement")
    ap.add_argument("--adjoint-steps", type=int, default=400, help="steps of the adjoint measurement (400: the workload)")
    ap.add_argument("--only", choices=["adjoint", "bowl", "bowl_step", "batched", "navfield", "venue_l", "venue_s", "terrace"], default=None,
                    help="run only this sub-measurement and print its object (profiling runs)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    if args.only:   # one sub-measurement alone (a profiling run; not the benchmark line)
        import torch
        import __graft_entry__
        __graft_entry__._pkg_build().build()
        import swarm_gb300
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        P = swarm_gb300.params_si()
        fn = {"adjoint": lambda: bench_adjoint(P, steps=args.adjoint_steps), "bowl": lambda: bench_bowl(P),
              "batched": lambda: bench_batched(P),
              "navfield": lambda: bench_nav_field(bowl_venue()), "venue_l": lambda: bench_venue_l(),
              "venue_s": lambda: bench_venue_s(), "terrace": lambda: bench_terrace(),
              "bowl_step": lambda: bench_bowl(P, steps=10, evacuation=False)}[args.only]
        print(json.dumps({args.only: fn()}))
        return 0

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import numpy as np
    import torch
    import __graft_entry__
    __graft_entry__._pkg_build().build()
    import swarm_gb300

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    venue, (boids, r, v0) = workload()
    P = swarm_gb300.params_si()
    n = boids.shape[0]
    stream = torch.cuda.Stream()
    sim = swarm_gb300.CrowdSim(P, venue, n)
    sim.set_stream(stream.cuda_stream)
    sim.set_state(boids)
    sim.set_agent_params(r, v0)
    sim.set_graph(args.phase_kernels)   # the per-phase kernels replay graphs; the fused step is one launch either way
    sim.set_fused(not args.phase_kernels)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            sim.step(1)
    torch.cuda.synchronize()
    start_state = sim.state()

    # timed region: K steps, each bracketed by CUDA events on the simulation's stream, L2 flushed before each. Stage
    # timing is off here (its events and in-kernel stamps cost ~5 us a step); the fused step is one launch, so each
    # step's event pair is that launch's duration. The stage breakdown comes from a replay of the same steps below.
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(k & 0xFF)
                evs[k][0].record(stream)
                sim.step(1)
                evs[k][1].record(stream)
            stream.synchronize()
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    step_ms = [a.elapsed_time(b) for a, b in evs]
    total_ms = sum(step_ms)
    launches = sim.launch_count() * args.steps   # per-step launches of the last call x timed steps

    # the stage breakdown: the same steps again from the same state with stage timing on (untimed as a whole)
    stages = []
    sim.set_state(start_state)
    sim.set_timing(True)
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(k & 0xFF)
            sim.step(1)
        stream.synchronize()
        stages.append(sim.stage_times())
    sim.set_timing(False)

    # exact agent-steps: replay the timed steps (bit-identical) and count the agents active at each step's start
    sim.synchronize()   # raises if a device-side check or wait failed during the timed steps
    rep = swarm_gb300.CrowdSim(P, venue, n)
    rep.set_state(start_state)
    rep.set_agent_params(r, v0)
    agent_steps = 0
    for _ in range(args.steps):
        agent_steps += int((rep.state()[:, 3] != 0).sum())
        rep.step(1)
    rep.close()

    t_max, agent_steps_all = replica_totals(dist, "cuda", total_ms, agent_steps)
    value = agent_steps_all / (t_max * 1e-3)

    # roofline of the dominant kernel, from the library's events over the timed steps. The default path runs each
    # step as one persistent kernel (k_step_fused): its algorithmic bytes are the whole step's, B_step per agent.
    K = P.proj_iterations
    active_mean = agent_steps / args.steps
    if args.phase_kernels:
        per = {
            "k_predict": (statistics.mean(s["predict"] for s in stages), 1, BYTES["predict"]),
            "k_project": (statistics.mean(s["project"] for s in stages) / max(K - 1, 1), max(K - 1, 0), BYTES["sweep"]),
            "k_final": (statistics.mean(s["final_pass"] for s in stages), 1, BYTES["final"]),
            "sort (5 kernels)": (statistics.mean(s["sort"] for s in stages) / 5.0, 5, BYTES["sort"] / 5.0),
        }
    else:   # the fused kernel's launches: the timed steps' own events (one launch a step)
        per = {"k_step_fused": (total_ms / args.steps, 1, B_STEP)}
    dom = max(per, key=lambda k: per[k][0] * per[k][1])
    dom_ms, _, dom_bytes = per[dom]
    hbm, peak_kind = peaks()
    achieved = dom_bytes * active_mean / (dom_ms * 1e-3) / 1e9
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "traffic.txt")   # measured by ncu, one line per kernel: name bytes
    if os.path.exists(tfile):
        for line in open(tfile):
            parts = line.split()
            if len(parts) == 2 and not line.startswith("#") and parts[0] == dom:
                traffic = int(parts[1])

    # the same workload congested: stepped on (untimed) to 250 steps from the spawn -- the reference's own benchmark
    # states are the spawn and CONGESTED_STEPS = 250 -- then timed the same way
    congested = None
    if rank == 0 and world == 1:
        done = args.warmup + args.steps
        with torch.cuda.stream(stream):
            sim.step(max(0, CONGESTED_STEPS - done))
        torch.cuda.synchronize()
        c_ms, c_active = [], []
        for k in range(min(args.steps, 20)):
            c_active.append(int((sim.state()[:, 3] != 0).sum()))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                flush.fill_(k & 0xFF)
                e0.record(stream)
                sim.step(1)
                e1.record(stream)
            stream.synchronize()
            c_ms.append(e0.elapsed_time(e1))
        congested = {"after_steps": max(CONGESTED_STEPS, done), "steps": len(c_ms),
                     "value": sum(c_active) / (sum(c_ms) * 1e-3), "ms_per_step": statistics.mean(c_ms),
                     "active_per_step": statistics.mean(c_active)}

    # the same steps chained in one persistent launch (a grid barrier between steps, no launch per step): the state
    # stays L2-resident between steps here, as in a simulation run; the per-step figure above flushes L2 before each
    chained = None
    if rank == 0 and world == 1:
        ch = swarm_gb300.CrowdSim(P, venue, n)
        ch.set_stream(stream.cuda_stream)
        ch.set_state(start_state)
        ch.set_agent_params(r, v0)
        with torch.cuda.stream(stream):
            ch.step(args.warmup)
        ch.set_state(start_state)
        torch.cuda.synchronize()
        c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            flush.fill_(0)
            c0.record(stream)
            ch.step(args.steps)
            c1.record(stream)
        stream.synchronize()
        ch.synchronize()
        c_ms = c0.elapsed_time(c1)
        chained = {"value": agent_steps / (c_ms * 1e-3), "ms_per_step": c_ms / args.steps, "launches": ch.launch_count(),
                   "l2": "flushed once before the run, warm between its steps"}
        ch.close()

    # e2e through swarm_step_host with pinned host buffers
    e2e_sim = swarm_gb300.CrowdSim(P, venue, n)
    e2e_sim.set_agent_params(r, v0)
    e2e_sim.set_graph(True)
    e2e_sim.set_fused(not args.phase_kernels)
    h_in = torch.from_numpy(start_state.copy()).pin_memory()
    h_out = torch.empty_like(h_in).pin_memory()
    for _ in range(2):
        e2e_sim.step_host(h_in.data_ptr(), h_out.data_ptr(), n, 1)
    cur_in, cur_out = h_in, h_out
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_sim.step_host(cur_in.data_ptr(), cur_out.data_ptr(), n, 1)
        cur_in, cur_out = cur_out, cur_in
    e2e_ms, _ = replica_totals(dist, "cuda", (time.perf_counter() - t0) * 1e3, 0)   # the slowest rank's wall clock
    e2e_value = agent_steps_all / (e2e_ms * 1e-3)

    line = None
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (generated hall and lattice spawn, seed 0)",
            "config": bench_config(n, world),
            "details": {"active_per_step": active_mean,
                        "step_fraction_of_hbm_roofline": value * B_STEP / (hbm * 1e9),
                        "path": "one kernel per phase (CUDA graphs)" if args.phase_kernels else
                                "one persistent cooperative kernel per step",
                        "stage_ms_mean": {k: statistics.mean(s[k] for s in stages)
                                          for k in ("sort", "predict", "project", "final_pass", "total")}},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "peak_kind": peak_kind,
                         "bytes_per_agent": dom_bytes, "mean_launch_ms": dom_ms,
                         "traffic": traffic},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": n * 32, "d2h_bytes_per_step": n * 32,
                    "path": "swarm_step_host (C ABI), pinned host buffers"},
            "gpu_launches": launches,
        }
        if congested:
            line["details"]["congested"] = congested
        if chained:
            line["details"]["chained_steps"] = chained
        line["clocks"] = clk.summary()
        if not args.no_batch and world == 1:
            try:
                line["batched"] = bench_batched(P)
            except Exception as e:  # reported, not fatal
                line["batched"] = {"error": str(e)[:300]}
        if not args.no_bowl and world == 1:
            try:
                line["bowl"] = bench_bowl(P)
            except Exception as e:  # reported, not fatal
                line["bowl"] = {"error": str(e)[:300]}
        if not args.no_bowl and world == 1:
            try:
                line["reference_venue_L"] = bench_venue_l()
            except Exception as e:  # reported, not fatal
                line["reference_venue_L"] = {"error": str(e)[:300]}
            try:
                line["reference_venue_S"] = bench_venue_s()
            except Exception as e:  # reported, not fatal
                line["reference_venue_S"] = {"error": str(e)[:300]}
            try:
                line["reference_terrace"] = bench_terrace()
            except Exception as e:  # reported, not fatal
                line["reference_terrace"] = {"error": str(e)[:300]}
        if not args.no_adjoint and world == 1:
            try:
                line["adjoint"] = bench_adjoint(P, steps=args.adjoint_steps)
            except Exception as e:  # reported, not fatal
                line["adjoint"] = {"error": str(e)[:300]}
        if not args.no_cpu_baseline and world == 1:
            try:
                line["cpu_baseline"] = cpu_baseline()
            except Exception as e:  # reported, not fatal
                line["cpu_baseline"] = {"value": None, "error": str(e)[:200]}
        print(json.dumps(line))
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
