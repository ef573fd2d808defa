"""Python binding of libswarm_gb300.so (include/swarm_cuda.h): the GB300 crowd step behind a ctypes layer.

The class CrowdSim mirrors the reference's step/state API (DedovSergei/swarm-crowd-simulation
include/swarm/cpu_crowd_sim.hpp:30-169 and include/swarm/crowd_sim.hpp:53-194): set_state (setState / upload),
step, state, grid, cells, contacts, set_projection_iterations, set_drive_table. States are numpy float32 arrays of
shape (n, 8): the reference's GpuBoid (position.xyzw, velocity.xyzw).

There is no CPU fallback: if the library has not been built the import fails with the build command.
"""
import ctypes as C
import os

import numpy as np

from .abi import (METRIC_CELL_WORDS, SWARM_LOSS_NAV_DISTANCE, SWARM_OK, SWARM_VENUE_GRID, SWARM_VENUE_STADIUM,
                  SwarmAdjointStats, SwarmEvacuation, SwarmLossSpec, SwarmMetricCounters, SwarmNavFieldStats, SwarmParams,
                  SwarmStageTimes, SwarmTuning, SwarmVenue, SwarmExitChoiceSpec, SwarmSeatedChoiceSpec, CHOICE_NONE,
                  CHOICE_EMPTY, fptr)

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_DIR, "libswarm_gb300.so")
_lib = None


class SwarmError(RuntimeError):
    pass


_H = C.c_void_p
_SIG = {
    "swarm_params_reference": [C.POINTER(SwarmParams)],
    "swarm_params_si": [C.POINTER(SwarmParams)],
    "swarm_create": [C.POINTER(SwarmParams), C.POINTER(SwarmVenue), C.c_int, C.POINTER(_H)],
    "swarm_destroy": [_H],
    "swarm_batch_create": [C.POINTER(SwarmParams), C.c_void_p, C.c_void_p, C.c_int, C.POINTER(_H)],
    "swarm_set_stream": [_H, C.c_void_p],
    "swarm_last_error": [_H, C.c_char_p, C.c_int],
    "swarm_upload_state": [_H, C.POINTER(C.c_float), C.c_int],
    "swarm_download_state": [_H, C.POINTER(C.c_float), C.c_int],
    "swarm_upload_state_device": [_H, C.c_void_p, C.c_int],
    "swarm_download_state_device": [_H, C.c_void_p, C.c_int],
    "swarm_set_agent_params": [_H, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int],
    "swarm_step": [_H, C.c_int],
    "swarm_set_iterations": [_H, C.c_int],
    "swarm_step_host": [_H, C.c_void_p, C.c_void_p, C.c_int, C.c_int],
    "swarm_set_drive_table": [_H, C.POINTER(C.c_float), C.c_int],
    "swarm_set_graph": [_H, C.c_int],
    "swarm_set_fused": [_H, C.c_int],
    "swarm_set_tuning": [_H, C.POINTER(SwarmTuning)],
    "swarm_autotune": [_H, C.c_int, C.POINTER(SwarmTuning)],
    "swarm_test_barrier_timeout": [_H],
    "swarm_synchronize": [_H],
    "swarm_get_grid": [_H, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.c_int],
    "swarm_get_cells": [_H, C.POINTER(C.c_uint32), C.c_int],
    "swarm_get_contacts": [_H, C.POINTER(C.c_uint8), C.c_int],
    "swarm_set_timing": [_H, C.c_int],
    "swarm_stage_times": [_H, C.POINTER(SwarmStageTimes)],
    "swarm_launch_count": [_H, C.POINTER(C.c_int64)],
    "swarm_metrics_enable": [_H, C.c_int, C.c_void_p],
    "swarm_metrics_reset": [_H],
    "swarm_metrics_read": [_H, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int],
    "swarm_metric_thresholds_grid": [C.POINTER(SwarmVenue), C.c_int, C.c_void_p],
    "swarm_hall_layout": [C.c_void_p, C.POINTER(SwarmVenue)],
    "swarm_hall_fields": [C.c_void_p, C.POINTER(SwarmVenue), C.POINTER(C.c_float), C.POINTER(C.c_float),
                          C.POINTER(C.c_float)],
    "swarm_adjoint_run": [_H, C.POINTER(SwarmLossSpec), C.c_int, C.c_int, C.POINTER(C.c_double),
                          C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float),
                          C.POINTER(SwarmAdjointStats)],
    "swarm_adjoint_set_tape_budget": [_H, C.c_int64],
    "swarm_set_relaxation_time": [_H, C.c_float],
    "swarm_run_evacuation": [_H, C.c_int, C.c_void_p, C.POINTER(SwarmEvacuation)],
    "swarm_snapshot_write": [C.c_char_p, C.POINTER(C.c_float), C.c_int],
    "swarm_snapshot_read": [C.c_char_p, C.POINTER(C.c_float), C.c_int],
    "swarm_snapshot_count": [C.c_char_p],
    "swarm_sdf_read": [C.c_char_p, C.POINTER(C.c_float), C.c_int],
    "swarm_nav_cache_read": [C.c_char_p, C.c_uint64, C.c_void_p, C.c_int64, C.POINTER(C.c_int32), C.POINTER(C.c_float),
                             C.POINTER(C.c_float), C.POINTER(C.c_float)],
    "swarm_nav_field_gpu": [C.c_int, C.c_int, C.c_double, C.c_void_p, C.c_void_p, C.POINTER(C.c_float),
                            C.POINTER(SwarmNavFieldStats)],
    "swarm_nav_field_cpu": [C.c_int, C.c_int, C.c_double, C.c_void_p, C.c_void_p, C.POINTER(C.c_float)],
    "swarm_set_nav_solver": [C.c_int],
    "swarm_hall_exit_fields": [C.c_void_p, C.POINTER(SwarmVenue), C.POINTER(C.c_float), C.POINTER(C.c_float),
                               C.c_void_p],
    "swarm_bowl_exit_fields": [C.c_void_p, C.POINTER(SwarmVenue), C.POINTER(C.c_float), C.POINTER(C.c_float),
                               C.c_void_p],
    "swarm_exit_choice_table": [C.POINTER(SwarmVenue), C.POINTER(SwarmExitChoiceSpec), C.c_void_p,
                                C.POINTER(C.c_float)],
    "swarm_set_exit_choice": [_H, C.POINTER(SwarmExitChoiceSpec)],
    "swarm_get_exit_choice": [_H, C.c_void_p, C.c_int, C.c_void_p],
    "swarm_set_seated_choice": [_H, C.POINTER(SwarmSeatedChoiceSpec)],
    "swarm_choice_cache_read": [C.c_char_p, C.c_uint64, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p,
                                C.POINTER(C.c_int32), C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                C.POINTER(C.c_int32), C.POINTER(C.c_int64)],
    "swarm_bowl_layout": [C.c_void_p, C.POINTER(SwarmVenue)],
    "swarm_bowl_fields": [C.c_void_p, C.POINTER(SwarmVenue), C.POINTER(C.c_float), C.POINTER(C.c_float),
                          C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_void_p, C.POINTER(C.c_float)],
    "swarm_spawn_bowl": [C.c_void_p, C.c_float, C.c_uint64, C.c_float, C.c_float, C.c_float, C.c_float,
                         C.c_float, C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float)],
    "swarm_spawn_lattice": [C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_uint64,
                            C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float,
                            C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float)],
}


def bind(L):
    """Sets the C signatures of every entry point of _SIG that the library L exports (the CUDA library, or a host
    build of the venue builders) and returns L."""
    for name, args in _SIG.items():
        if hasattr(L, name):
            f = getattr(L, name)
            f.argtypes = args
            f.restype = C.c_int
    return L


def lib():
    """The loaded CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with `python swarm-crowd-simulation_gb300/build.py` "
                              "(or __graft_entry__.build()); there is no CPU fallback")
        _lib = bind(C.CDLL(LIB_PATH))
    return _lib


_gen = None


def use_generator(L):
    """The library the venue builders, spawns and parameter presets call from now on: a ctypes library exporting the
    host entry points of csrc/venues.cpp and csrc/params.cpp (None: the CUDA library). The builders are host code, so
    a host-only build of the same sources gives the same venues without loading the CUDA library."""
    global _gen
    _gen = None if L is None else bind(L)


def generator():
    return _gen if _gen is not None else lib()


def params_reference():
    """The reference's constants (model units, K = 32), folded as the reference folds them."""
    p = SwarmParams()
    _check(generator().swarm_params_reference(C.byref(p)), "swarm_params_reference")
    return p


def params_si():
    """The SI preset of the grid venues (dt 0.05 s, K = 8, tau 0.5 s, per-agent radius and v0)."""
    p = SwarmParams()
    _check(generator().swarm_params_si(C.byref(p)), "swarm_params_si")
    return p


def snapshot_write(path, boids):
    """A workload snapshot: the raw GpuBoid array (the reference's bench_common saveSnapshot format)."""
    b = np.ascontiguousarray(boids, dtype=np.float32).reshape(-1, 8)
    _check(lib().swarm_snapshot_write(os.fsencode(path), fptr(b), b.shape[0]), "swarm_snapshot_write")


def nav_cache_read(path, expected_key=0):
    """A seated venue's navigation-field cache file as the reference writes it, as the GPU table: (cells (res^2, 4)
    float32 -- anchor x, anchor y, distance, info bits --, (res, origin, cell, 1 / cell))."""
    res, o, c, ic = C.c_int32(), C.c_float(), C.c_float(), C.c_float()
    p = os.fsencode(path)
    _check(lib().swarm_nav_cache_read(p, expected_key, None, 0, C.byref(res), C.byref(o), C.byref(c), C.byref(ic)),
           "swarm_nav_cache_read")
    cells = np.empty((res.value * res.value, 4), np.float32)
    _check(lib().swarm_nav_cache_read(p, expected_key, cells.ctypes.data_as(C.c_void_p), cells.shape[0], C.byref(res),
                                      C.byref(o), C.byref(c), C.byref(ic)), "swarm_nav_cache_read")
    return cells, (res.value, o.value, c.value, ic.value)


def choice_cache_read(path, expected_key=0):
    """A seated venue's exit-choice cache file as the reference writes it: (index (res^2,) uint32, entries (n, 36)
    uint32 -- 24 slot words, 12 distance words --, clear widths (n_exits,) float64, (res, origin, cell, 1 / cell))."""
    res, o, c, ic = C.c_int32(), C.c_float(), C.c_float(), C.c_float()
    ne, nx = C.c_int64(), C.c_int32()
    p = os.fsencode(path)
    _check(lib().swarm_choice_cache_read(p, expected_key, None, 0, None, 0, None, C.byref(res), C.byref(o), C.byref(c),
                                         C.byref(ic), C.byref(nx), C.byref(ne)), "swarm_choice_cache_read")
    index = np.empty(res.value * res.value, np.uint32)
    entries = np.empty((max(ne.value, 1), 36), np.uint32)
    widths = np.empty(max(nx.value, 1), np.float64)
    _check(lib().swarm_choice_cache_read(p, expected_key, index.ctypes.data_as(C.c_void_p), index.shape[0],
                                         entries.ctypes.data_as(C.c_void_p), entries.shape[0],
                                         widths.ctypes.data_as(C.c_void_p), C.byref(res), C.byref(o), C.byref(c),
                                         C.byref(ic), C.byref(nx), C.byref(ne)), "swarm_choice_cache_read")
    return index, entries[:ne.value], widths[:nx.value], (res.value, o.value, c.value, ic.value)


def snapshot_read(path):
    n = lib().swarm_snapshot_count(os.fsencode(path))
    if n <= 0:
        raise SwarmError(f"{path}: not a GpuBoid snapshot")
    out = np.empty((n, 8), np.float32)
    _check(lib().swarm_snapshot_read(os.fsencode(path), fptr(out), n), "swarm_snapshot_read")
    return out


def sdf_read(path, res=130):
    """The reference's stadium.sdf: res^3 float32 ([x][y][z], z fastest)."""
    out = np.empty(res ** 3, np.float32)
    _check(lib().swarm_sdf_read(os.fsencode(path), fptr(out), int(res)), "swarm_sdf_read")
    return out


def _choice_spec(fields, widths, types, candidates):
    f = np.ascontiguousarray(fields, dtype=np.float32)
    w = np.ascontiguousarray(widths, dtype=np.float32)
    t = np.ascontiguousarray(types, dtype=np.uint8)
    spec = SwarmExitChoiceSpec(int(w.shape[0]), int(candidates), fptr(f), fptr(w),
                               t.ctypes.data_as(C.POINTER(C.c_uint8)))
    return spec, (f, w, t)


def exit_choice_table(venue, fields, widths, types, candidates=24):
    """swarm_exit_choice_table: the queue-aware choice's candidates per hash cell, (cells, K) exits and distances."""
    spec, keep = _choice_spec(fields, widths, types, candidates)
    v = venue.struct
    cells = v.grid_res_x * v.grid_res_y
    ex = np.empty((cells, candidates), np.uint8)
    di = np.empty((cells, candidates), np.float32)
    _check(lib().swarm_exit_choice_table(C.byref(v), C.byref(spec), ex.ctypes.data_as(C.c_void_p), fptr(di)),
           "swarm_exit_choice_table")
    return ex, di


def exit_inv_capacity(widths):
    """Seconds per queued agent of each exit, 60 / (w J) with J = 83.6 persons per metre per minute (float32, as the
    library computes it)."""
    return (60.0 / (np.asarray(widths, dtype=np.float32).astype(np.float64) * 83.6)).astype(np.float32)


def nav_field(kind, h, speed=None, solver="gpu"):
    """The fast-marching travel distance on a grid (kind: (ny, nx) uint8, 0 free, 1 source, 3 wall; speed: (ny, nx)
    float32 or None): (field (ny, nx) float32, stats dict or None). solver "gpu" or "cpu": the same floats."""
    kind = np.ascontiguousarray(kind, dtype=np.uint8)
    ny, nx = kind.shape
    sp = None if speed is None else np.ascontiguousarray(speed, dtype=np.float32).reshape(ny, nx)
    out = np.empty((ny, nx), np.float32)
    kp = kind.ctypes.data_as(C.c_void_p)
    spp = None if sp is None else sp.ctypes.data_as(C.c_void_p)
    if solver == "gpu":
        st = SwarmNavFieldStats()
        _check(lib().swarm_nav_field_gpu(nx, ny, float(h), kp, spp, fptr(out), C.byref(st)), "swarm_nav_field_gpu")
        return out, {k: getattr(st, k) for k, _ in SwarmNavFieldStats._fields_}
    if solver != "cpu":
        raise ValueError("solver: 'gpu' or 'cpu'")
    _check(lib().swarm_nav_field_cpu(nx, ny, float(h), kp, spp, fptr(out)), "swarm_nav_field_cpu")
    return out, None


def set_nav_solver(solver):
    """The solver the venue builders use from now on ("cpu" or "gpu"); returns the previous one."""
    if solver not in ("cpu", "gpu"):
        raise ValueError("solver: 'gpu' or 'cpu'")
    code = 1 if solver == "gpu" else 0
    prev = lib().swarm_set_nav_solver(code)
    if prev < 0:
        raise SwarmError("swarm_set_nav_solver failed")
    return "gpu" if prev == 1 else "cpu"


def _check(rc, what, h=None):
    if rc != SWARM_OK:
        msg = ""
        if h is not None:
            buf = C.create_string_buffer(512)
            lib().swarm_last_error(h, buf, 512)
            msg = buf.value.decode()
        raise SwarmError(f"{what} failed ({rc}): {msg}")


from .venues import Venue  # noqa: E402  (needs lib())


class CrowdSim:
    """One simulation on the current CUDA device (the reference's CrowdSim / CpuCrowdSim)."""

    def __init__(self, params, venue, capacity):
        self.params = params
        self.venue = venue
        self.capacity = int(capacity)
        h = C.c_void_p()
        _check(lib().swarm_create(C.byref(params), C.byref(venue.struct), self.capacity, C.byref(h)), "swarm_create")
        self._h = h
        self.n = 0

    def close(self):
        if getattr(self, "_h", None):
            lib().swarm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc, what):
        _check(rc, what, self._h)

    # ---- state ----
    def set_state(self, boids):
        """CpuCrowdSim::setState / CrowdSim::upload: (n, 8) float32 GpuBoid array."""
        b = np.ascontiguousarray(boids, dtype=np.float32).reshape(-1, 8)
        self._ck(lib().swarm_upload_state(self._h, fptr(b), b.shape[0]), "upload")
        self.n = b.shape[0]

    def set_agent_params(self, radius, v0):
        r = np.ascontiguousarray(radius, dtype=np.float32)
        v = np.ascontiguousarray(v0, dtype=np.float32)
        self._ck(lib().swarm_set_agent_params(self._h, fptr(r), fptr(v), r.shape[0]), "set_agent_params")

    def state(self):
        out = np.empty((self.n, 8), np.float32)
        self._ck(lib().swarm_download_state(self._h, fptr(out), self.n), "download")
        return out

    # ---- stepping ----
    def step(self, steps=1):
        self._ck(lib().swarm_step(self._h, int(steps)), "step")

    def step_host(self, in_ptr, out_ptr, n, steps=1):
        """swarm_step_host on raw host pointers (e.g. pinned buffers): upload, step, download, wait."""
        self._ck(lib().swarm_step_host(self._h, C.c_void_p(in_ptr), C.c_void_p(out_ptr), int(n), int(steps)), "step_host")
        self.n = int(n)

    def set_stream(self, stream_ptr):
        """Run on the caller's CUDA stream (a cudaStream_t as an int; 0 / None: the handle's own)."""
        self._ck(lib().swarm_set_stream(self._h, C.c_void_p(stream_ptr or None)), "set_stream")

    def synchronize(self):
        self._ck(lib().swarm_synchronize(self._h), "synchronize")

    def set_projection_iterations(self, k):
        self._ck(lib().swarm_set_iterations(self._h, int(k)), "set_iterations")

    def set_drive_table(self, dirs):
        if dirs is None:
            self._ck(lib().swarm_set_drive_table(self._h, None, 0), "set_drive_table")
            return
        d = np.ascontiguousarray(dirs, dtype=np.float32).reshape(-1, 2)
        self._ck(lib().swarm_set_drive_table(self._h, fptr(d), d.shape[0]), "set_drive_table")

    def set_graph(self, enabled=True):
        self._ck(lib().swarm_set_graph(self._h, int(bool(enabled))), "set_graph")

    def set_exit_choice(self, fields=None, widths=None, types=None, candidates=24):
        """The queue-aware exit choice (fields: (n_exits, nav nodes) per-exit distances, widths in metres, types 0
        avenue / 1 door); None: the nearest-exit field. Restarts the choice (no exit assigned)."""
        if fields is None:
            self._ck(lib().swarm_set_exit_choice(self._h, None), "set_exit_choice")
            return
        spec, _keep = _choice_spec(fields, widths, types, candidates)
        self._ck(lib().swarm_set_exit_choice(self._h, C.byref(spec)), "set_exit_choice")

    def set_seated_choice(self, index=None, entries=None, inv_cap_s=None, seconds_per_unit=0.0, dist_quantum=0.0,
                          choice_steps=17):
        """The queue-aware exit choice of a seated venue on the reference's own candidate table (index: res^2 words on
        the navigation grid; entries: (n, 36) uint32 GpuNavChoiceCell words; inv_cap_s: seconds per queued agent per
        exit); None: off. Restarts the choice (no exit assigned)."""
        if index is None:
            self._ck(lib().swarm_set_seated_choice(self._h, None), "set_seated_choice")
            return
        idx = np.ascontiguousarray(index, dtype=np.uint32)
        ent = np.ascontiguousarray(entries, dtype=np.uint32).reshape(-1, 36)
        cap = np.ascontiguousarray(inv_cap_s, dtype=np.float32)
        spec = SwarmSeatedChoiceSpec(int(cap.shape[0]), int(round(np.sqrt(idx.shape[0]))), idx.ctypes.data,
                                     ent.ctypes.data, int(ent.shape[0]), fptr(cap), float(seconds_per_unit),
                                     float(dist_quantum), int(choice_steps))
        self._ck(lib().swarm_set_seated_choice(self._h, C.byref(spec)), "set_seated_choice")

    def exit_choice(self):
        """(assigned exit per agent (CHOICE_NONE: none yet), counters: evaluations, eligible, switches, forced)"""
        a = np.empty(self.n, np.uint32)
        c = np.empty(4, np.uint32)
        self._ck(lib().swarm_get_exit_choice(self._h, a.ctypes.data_as(C.c_void_p), self.n, c.ctypes.data_as(C.c_void_p)),
                 "get_exit_choice")
        return a, c

    def set_fused(self, enabled=True):
        """One persistent kernel per step (True, the default) or one kernel per phase (False)."""
        self._ck(lib().swarm_set_fused(self._h, int(bool(enabled))), "set_fused")

    def set_tuning(self, fused=True, threads=0, blocks_per_sm=0, steps_per_launch=0):
        t = SwarmTuning(int(bool(fused)), int(threads), int(blocks_per_sm), 0.0, int(steps_per_launch))
        self._ck(lib().swarm_set_tuning(self._h, C.byref(t)), "set_tuning")

    def autotune(self, steps=3):
        """Times each launch configuration from the current state (restored), keeps the fastest; returns it."""
        t = SwarmTuning()
        self._ck(lib().swarm_autotune(self._h, int(steps), C.byref(t)), "autotune")
        return {"fused": bool(t.fused), "threads": t.threads, "blocks_per_sm": t.blocks_per_sm,
                "ms_per_step": t.ms_per_step, "steps_per_launch": t.steps_per_launch}

    def download_device(self, dst_ptr):
        """The state into device memory at dst_ptr (n x 8 floats)."""
        self._ck(lib().swarm_download_state_device(self._h, C.c_void_p(dst_ptr), self.n), "download_device")

    def set_timing(self, enabled=True):
        self._ck(lib().swarm_set_timing(self._h, int(bool(enabled))), "set_timing")

    def stage_times(self):
        t = SwarmStageTimes()
        self._ck(lib().swarm_stage_times(self._h, C.byref(t)), "stage_times")
        return {k: getattr(t, k) for k, _ in SwarmStageTimes._fields_}

    def launch_count(self):
        c = C.c_int64()
        self._ck(lib().swarm_launch_count(self._h, C.byref(c)), "launch_count")
        return c.value

    # ---- safety metrics ----
    def metrics_enable(self, res, threshold_mass):
        """Metrics after every step: res x res 1 m cells; threshold_mass (res*res, 4) uint32 (LoS E, LoS F, crush, -)."""
        t = np.ascontiguousarray(threshold_mass, dtype=np.uint32).reshape(-1, 4)
        assert t.shape[0] == res * res
        self._ck(lib().swarm_metrics_enable(self._h, int(res), t.ctypes.data_as(C.c_void_p)), "metrics_enable")
        self.metric_res = int(res)

    def metrics_reset(self):
        self._ck(lib().swarm_metrics_reset(self._h), "metrics_reset")

    def metrics(self):
        """(counters struct, cells (res*res, 16) uint32, evacuation step per agent)."""
        ctr = SwarmMetricCounters()
        cells = np.empty((self.metric_res * self.metric_res, METRIC_CELL_WORDS), np.uint32)
        evac = np.empty(self.n, np.uint32)
        self._ck(lib().swarm_metrics_read(self._h, C.byref(ctr), cells.ctypes.data_as(C.c_void_p),
                                          evac.ctypes.data_as(C.c_void_p), self.n), "metrics_read")
        return ctr, cells, evac

    # ---- headless evacuation ----
    def run_evacuation(self, max_steps):
        """Steps until no agent is active or max_steps: (stats dict: steps, initial_active, remaining, t50/t90/t100 in
        steps and seconds), active count after every step run (int32 array))."""
        e = SwarmEvacuation()
        active = np.zeros(int(max_steps), np.int32)
        self._ck(lib().swarm_run_evacuation(self._h, int(max_steps), active.ctypes.data_as(C.c_void_p), C.byref(e)),
                 "run_evacuation")
        return {k: getattr(e, k) for k, _ in SwarmEvacuation._fields_}, active[:e.steps]

    # ---- the adjoint ----
    def set_relaxation_time(self, tau):
        """tau_relax = tau, relax_step = exp(-dt / tau)."""
        self._ck(lib().swarm_set_relaxation_time(self._h, float(tau)), "set_relaxation_time")

    def set_adjoint_tape_budget(self, nbytes):
        """Device bytes the adjoint may keep as segment tapes beyond the last segment's (default 1 GiB; 0: recompute
        every other segment); the gradients are the same either way."""
        self._ck(lib().swarm_adjoint_set_tape_budget(self._h, int(nbytes)), "adjoint_set_tape_budget")

    def adjoint(self, steps, ckpt_every=20, stats=False):
        """The evacuation loss L = dt * sum_t sum_i D(p_i(t)) of `steps` steps from the current state (left as it is)
        and its gradient by the adjoint: (L, dL/dv0 (n,), dL/dr (n,), dL/dtau) [, stats dict]."""
        spec = SwarmLossSpec(SWARM_LOSS_NAV_DISTANCE, 0)
        loss = C.c_double()
        gv = np.empty(self.n, np.float32)
        gr = np.empty(self.n, np.float32)
        gt = np.empty(1, np.float32)
        st = SwarmAdjointStats()
        self._ck(lib().swarm_adjoint_run(self._h, C.byref(spec), int(steps), int(ckpt_every), C.byref(loss), fptr(gv),
                                         fptr(gr), fptr(gt), C.byref(st)), "adjoint_run")
        out = (loss.value, gv, gr, float(gt[0]))
        if stats:
            return out + ({k: getattr(st, k) for k, _ in SwarmAdjointStats._fields_},)
        return out

    # ---- inspection ----
    def grid(self):
        """CpuCrowdSim::grid(): the last step's sorted (gridID, boidID) pairs."""
        g = np.empty(self.n, np.uint32)
        b = np.empty(self.n, np.uint32)
        self._ck(lib().swarm_get_grid(self._h, g.ctypes.data_as(C.POINTER(C.c_uint32)),
                                      b.ctypes.data_as(C.POINTER(C.c_uint32)), self.n), "get_grid")
        return g, b

    def cells(self):
        """CpuCrowdSim::cells(): (startIndex, agentCount) per cell, shape (ncells, 2)."""
        nc = lib().swarm_get_cells(self._h, None, 0)
        out = np.empty((nc, 2), np.uint32)
        self._ck(lib().swarm_get_cells(self._h, out.ctypes.data_as(C.POINTER(C.c_uint32)), nc), "get_cells")
        return out

    def contacts(self):
        out = np.empty(self.n, np.uint8)
        self._ck(lib().swarm_get_contacts(self._h, out.ctypes.data_as(C.POINTER(C.c_uint8)), self.n), "get_contacts")
        return out


class BatchSim(CrowdSim):
    """Many independent grid venues packed into one simulation (swarm_batch_create): the state is every instance's
    agents one after another; instance i occupies [starts[i], starts[i + 1])."""

    def __init__(self, params, venues, counts):
        self.params = params
        self.venue = None
        self.venues = list(venues)
        counts = np.ascontiguousarray(counts, dtype=np.int32)
        arr = (SwarmVenue * len(self.venues))(*[v.struct for v in self.venues])
        self._arr = arr
        h = C.c_void_p()
        _check(lib().swarm_batch_create(C.byref(params), C.cast(arr, C.c_void_p), counts.ctypes.data_as(C.c_void_p),
                                        len(self.venues), C.byref(h)), "swarm_batch_create")
        self._h = h
        self.capacity = int(counts.sum())
        self.starts = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
        self.n = 0


__all__ = ["CrowdSim", "BatchSim", "Venue", "SwarmError", "lib", "params_reference", "params_si", "SwarmParams", "SwarmVenue",
           "SWARM_VENUE_GRID", "SWARM_VENUE_STADIUM"]
