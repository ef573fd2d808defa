"""ORACLE -- test infrastructure only: ctypes wrapper of liboracle.so (the CPU restatement, swarm_oracle.cpp) and of
_ref/libswarm_ref.so (the unmodified reference CPU step, built in this container only; see Makefile).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module, as the checker.
"""
import ctypes as C
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", platform.machine(), "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libswarm_ref.so")
_o = None
_r = None


def build(ref=False):
    """make -C oracle (and the reference's own CPU step when ref and the Makefile finds the reference tree)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if ref and subprocess.run(["make", "-s", "-C", HERE, "has-ref"], capture_output=True).returncode == 0:
        subprocess.run(["make", "-s", "-j8", "-C", HERE, "ref"], check=True)


def ref_dir():
    """The reference tree that _ref/libswarm_ref.so was built from (recorded by `make ref`), or None."""
    rec = os.path.join(HERE, "_ref", "ref_dir.txt")
    if not os.path.exists(rec):
        return None
    d = open(rec).read().strip()
    return d if os.path.isdir(d) else None


def lib():
    global _o
    if _o is None:
        if not os.path.exists(ORACLE_SO):
            build()
        L = C.CDLL(ORACLE_SO)
        V = C.c_void_p
        L.oracle_create.restype = V
        L.oracle_create.argtypes = [V, V, C.c_int]
        L.oracle_last_error.restype = C.c_char_p
        for name in ["oracle_destroy", "oracle_set_state", "oracle_set_agent_params", "oracle_set_iterations",
                     "oracle_set_threads", "oracle_set_drive_table", "oracle_step", "oracle_get_state",
                     "oracle_get_grid", "oracle_get_cells", "oracle_get_contacts", "oracle_set_exit_choice",
                     "oracle_get_exit_choice"]:
            getattr(L, name).restype = C.c_int
        L.oracle_destroy.argtypes = [V]
        L.oracle_set_state.argtypes = [V, V, C.c_int]
        L.oracle_set_agent_params.argtypes = [V, V, V, C.c_int]
        L.oracle_set_iterations.argtypes = [V, C.c_int]
        L.oracle_set_threads.argtypes = [V, C.c_int]
        L.oracle_set_drive_table.argtypes = [V, V, C.c_int]
        L.oracle_step.argtypes = [V, C.c_int]
        L.oracle_get_state.argtypes = [V, V]
        L.oracle_get_grid.argtypes = [V, V, V]
        L.oracle_get_cells.argtypes = [V, V, C.c_int]
        L.oracle_get_contacts.argtypes = [V, V]
        L.oracle_set_exit_choice.argtypes = [V, C.c_int, C.c_int, V, V, V, V]
        L.oracle_get_exit_choice.argtypes = [V, V, V]
        L.grad_eval.restype = C.c_int
        L.grad_eval.argtypes = [C.c_int, V, V, V, C.c_int, V, V, C.c_double, C.c_int, C.c_int, C.c_int, V, V, V, V, V, V, V]
        L.grad_last_error.restype = C.c_char_p
        _o = L
    return _o


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class OracleSim:
    """The CPU restatement, with CpuCrowdSim's API (same method names as swarm_gb300.CrowdSim)."""

    def __init__(self, params, venue_struct, threads=0):
        self._h = lib().oracle_create(C.byref(params), C.byref(venue_struct), threads)
        if not self._h:
            raise RuntimeError("oracle_create: " + lib().oracle_last_error().decode())
        self.ncells = venue_struct.grid_res_x * venue_struct.grid_res_y
        self.n = 0

    def __del__(self):
        if getattr(self, "_h", None):
            lib().oracle_destroy(self._h)
            self._h = None

    def set_state(self, boids):
        b = np.ascontiguousarray(boids, dtype=np.float32).reshape(-1, 8)
        assert lib().oracle_set_state(self._h, _p(b), b.shape[0]) == 0
        self.n = b.shape[0]

    def set_agent_params(self, radius, v0):
        r = np.ascontiguousarray(radius, dtype=np.float32)
        v = np.ascontiguousarray(v0, dtype=np.float32)
        assert lib().oracle_set_agent_params(self._h, _p(r), _p(v), r.shape[0]) == 0

    def set_projection_iterations(self, k):
        if lib().oracle_set_iterations(self._h, int(k)) != 0:
            raise ValueError(lib().oracle_last_error().decode())

    def set_threads(self, t):
        return lib().oracle_set_threads(self._h, int(t))

    def set_drive_table(self, dirs):
        if dirs is None:
            lib().oracle_set_drive_table(self._h, None, 0)
            return
        d = np.ascontiguousarray(dirs, dtype=np.float32).reshape(-1, 2)
        lib().oracle_set_drive_table(self._h, _p(d), d.shape[0])

    def set_exit_choice(self, fields, inv_cap, table_exits, table_dists):
        """The queue-aware exit choice: per-exit fields (n_exits, nav nodes), seconds per queued agent per exit, and
        the candidate table (cells, K) of exits and distances (as the library builds it); fields None: off."""
        if fields is None:
            lib().oracle_set_exit_choice(self._h, 0, 0, None, None, None, None)
            return
        f = np.ascontiguousarray(fields, dtype=np.float32)
        ic = np.ascontiguousarray(inv_cap, dtype=np.float32)
        te = np.ascontiguousarray(table_exits, dtype=np.uint8)
        td = np.ascontiguousarray(table_dists, dtype=np.float32)
        self._choice = (f, ic, te, td)
        lib().oracle_set_exit_choice(self._h, int(ic.shape[0]), int(te.shape[1]), _p(f), _p(ic), _p(te), _p(td))

    def exit_choice(self):
        """(assigned exit per agent, counters: evaluations, eligible, switches, forced)"""
        a = np.empty(self.n, np.uint32)
        c = np.empty(4, np.uint32)
        lib().oracle_get_exit_choice(self._h, _p(a), _p(c))
        return a, c

    def step(self, steps=1):
        assert lib().oracle_step(self._h, int(steps)) == 0, lib().oracle_last_error().decode()

    def state(self):
        out = np.empty((self.n, 8), np.float32)
        lib().oracle_get_state(self._h, _p(out))
        return out

    def grid(self):
        g = np.empty(self.n, np.uint32)
        b = np.empty(self.n, np.uint32)
        lib().oracle_get_grid(self._h, _p(g), _p(b))
        return g, b

    def cells(self):
        out = np.empty((self.ncells, 2), np.uint32)
        lib().oracle_get_cells(self._h, _p(out), self.ncells)
        return out

    def contacts(self):
        out = np.empty(self.n, np.uint8)
        lib().oracle_get_contacts(self._h, _p(out))
        return out


def grad_eval(prec, params, venue_struct, state, radius, v0, tau, steps, dirs=None, threads=0, want_state=False):
    """The loss L = dt * sum_t sum_i D(p_i(t)) of `steps` steps from `state` (swarm_grad.cpp), its derivatives along
    directions and the run's branch signature.

    prec 32: float arithmetic (bit-exact with the step); prec 64: double. dirs: None, or (dr, dv0, dtau) with dr, dv0
    of shape (k, n) and dtau of shape (k,), k <= 8 (tangents in double). Returns (loss, dloss (k,) or None, signature,
    end state (n, 8) float32 or None).
    """
    b = np.ascontiguousarray(state, dtype=np.float32).reshape(-1, 8)
    n = b.shape[0]
    r = np.ascontiguousarray(radius, dtype=np.float64)
    v = np.ascontiguousarray(v0, dtype=np.float64)
    loss = np.zeros(1, np.float64)
    sig = np.zeros(1, np.uint64)
    out = np.empty((n, 8), np.float32) if want_state else None
    nt = 0
    dr = dv = dt = dl = None
    if dirs is not None:
        dr = np.ascontiguousarray(np.atleast_2d(dirs[0]), dtype=np.float64)
        dv = np.ascontiguousarray(np.atleast_2d(dirs[1]), dtype=np.float64)
        dt = np.ascontiguousarray(np.atleast_1d(dirs[2]), dtype=np.float64)
        nt = dt.shape[0]
        assert dr.shape == (nt, n) and dv.shape == (nt, n) and 1 <= nt <= 8
        dl = np.zeros(nt, np.float64)
    pp = lambda a: None if a is None else _p(a)
    rc = lib().grad_eval(int(prec), C.byref(params), C.byref(venue_struct), _p(b), n, _p(r), _p(v), float(tau), int(steps),
                         int(threads), nt, pp(dr), pp(dv), pp(dt), _p(loss), pp(dl), _p(sig), pp(out))
    if rc != 0:
        raise RuntimeError("grad_eval: " + lib().grad_last_error().decode())
    return float(loss[0]), dl, int(sig[0]), out


class OracleMetrics:
    """The metrics restatement (MetricsReference::record): record(prev, cur) after each step."""

    def __init__(self, params, venue_struct, res, threshold_mass, n):
        L = lib()
        L.oracle_metrics_create.restype = C.c_void_p
        L.oracle_metrics_create.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int]
        L.oracle_metrics_record.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        L.oracle_metrics_read.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_metrics_destroy.argtypes = [C.c_void_p]
        self.thr = np.ascontiguousarray(threshold_mass, dtype=np.uint32)
        self._h = L.oracle_metrics_create(C.byref(params), C.byref(venue_struct), res, _p(self.thr), n)
        self.res, self.n = res, n

    def __del__(self):
        if getattr(self, "_h", None):
            lib().oracle_metrics_destroy(self._h)

    def record(self, prev, cur):
        a = np.ascontiguousarray(prev, dtype=np.float32)
        b = np.ascontiguousarray(cur, dtype=np.float32)
        lib().oracle_metrics_record(self._h, _p(a), _p(b), self.n)

    def read(self):
        ctr = np.zeros(196, np.uint32)   # SwarmMetricCounters, 784 bytes
        cells = np.zeros((self.res * self.res, 16), np.uint32)
        evac = np.zeros(self.n, np.uint32)
        lib().oracle_metrics_read(self._h, _p(ctr), _p(cells), _p(evac))
        return ctr, cells, evac


# ---- the unmodified reference (this container only) ----
def ref_available():
    return os.path.exists(REF_SO)


def ref_lib():
    global _r
    if _r is None:
        L = C.CDLL(REF_SO)
        V = C.c_void_p
        L.ref_create.restype = V
        L.ref_create.argtypes = [C.c_char_p, C.c_int, C.c_int]
        L.ref_last_error.restype = C.c_char_p
        L.ref_set_state.argtypes = [V, V, C.c_int]
        L.ref_step.argtypes = [V, C.c_int]
        L.ref_get_state.argtypes = [V, V]
        L.ref_get_grid.argtypes = [V, V, V]
        L.ref_get_cells.argtypes = [V, V, C.c_int]
        L.ref_get_contacts.argtypes = [V, V]
        L.ref_set_iterations.argtypes = [V, C.c_int]
        L.ref_destroy.argtypes = [V]
        L.ref_spawn_terrace.argtypes = [C.c_int, C.c_uint, V]
        L.ref_spawn_seated.argtypes = [C.c_char_p, C.c_int, C.c_double, C.c_uint, V]
        L.ref_load_sdf.argtypes = [C.c_char_p]
        L.ref_timings.argtypes = [V, V]
        _r = L
    return _r


class RefSim:
    """swarm::CpuCrowdSim itself (counting sort), on venue 'terrace' | 'S' | 'M' | 'L'."""

    def __init__(self, venue="terrace", threads=0):
        self._h = ref_lib().ref_create(venue.encode(), 0, threads)
        if not self._h:
            raise RuntimeError(ref_lib().ref_last_error().decode())
        self.n = 0

    def __del__(self):
        if getattr(self, "_h", None):
            ref_lib().ref_destroy(self._h)

    def set_state(self, boids):
        b = np.ascontiguousarray(boids, dtype=np.float32).reshape(-1, 8)
        assert ref_lib().ref_set_state(self._h, _p(b), b.shape[0]) == 0
        self.n = b.shape[0]

    def set_projection_iterations(self, k):
        assert ref_lib().ref_set_iterations(self._h, int(k)) == 0

    def step(self, steps=1):
        assert ref_lib().ref_step(self._h, int(steps)) == 0

    def state(self):
        out = np.empty((self.n, 8), np.float32)
        ref_lib().ref_get_state(self._h, _p(out))
        return out

    def grid(self):
        g = np.empty(self.n, np.uint32)
        b = np.empty(self.n, np.uint32)
        ref_lib().ref_get_grid(self._h, _p(g), _p(b))
        return g, b

    def cells(self, ncells=1600):
        out = np.empty((ncells, 2), np.uint32)
        ref_lib().ref_get_cells(self._h, _p(out), ncells)
        return out

    def contacts(self):
        out = np.empty(self.n, np.uint8)
        ref_lib().ref_get_contacts(self._h, _p(out))
        return out


class RefMetrics:
    """swarm::metrics::MetricsReference itself (the terrace's exits)."""

    def __init__(self, n, threshold_mass):
        L = ref_lib()
        L.ref_metrics_create.restype = C.c_void_p
        L.ref_metrics_create.argtypes = [C.c_int, C.c_void_p, C.c_int]
        L.ref_metrics_record.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        L.ref_metrics_read.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.ref_metrics_destroy.argtypes = [C.c_void_p]
        self.thr = np.ascontiguousarray(threshold_mass, dtype=np.uint32)
        self.cells = self.thr.size // 4
        self._h = L.ref_metrics_create(n, _p(self.thr), self.cells)
        self.n = n

    def __del__(self):
        if getattr(self, "_h", None):
            ref_lib().ref_metrics_destroy(self._h)

    def record(self, prev, cur):
        a = np.ascontiguousarray(prev, dtype=np.float32)
        b = np.ascontiguousarray(cur, dtype=np.float32)
        assert ref_lib().ref_metrics_record(self._h, _p(a), _p(b), self.n) == 0

    def read(self):
        ctr = np.zeros(196, np.uint32)
        cells = np.zeros((self.cells, 16), np.uint32)
        evac = np.zeros(self.n, np.uint32)
        ref_lib().ref_metrics_read(self._h, _p(ctr), _p(cells), _p(evac))
        return ctr, cells, evac


def ref_terrace_metric_cells():
    """computeMetricVenue(stadium.sdf).cellInfo(): (threshold_mass (4096, 4), walkable m^2 (4096,))."""
    L = ref_lib()
    L.ref_metrics_terrace_cells.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    thr = np.zeros((4096, 4), np.uint32)
    area = np.zeros(4096, np.float32)
    assert L.ref_metrics_terrace_cells(_p(thr), _p(area), 4096) == 4096
    return thr, area


def ref_load_sdf(path):
    return ref_lib().ref_load_sdf(path.encode()) == 0


def ref_spawn_terrace(n, seed=1337):
    out = np.empty((n, 8), np.float32)
    assert ref_lib().ref_spawn_terrace(n, seed, _p(out)) == 0
    return out


def state_hash(state):
    """FNV-1a 64 of the raw state bytes (the reference's golden::stateHash, tools/golden_state.hpp:121-126)."""
    h = 0xcbf29ce484222325
    for byte in np.ascontiguousarray(state, dtype=np.float32).tobytes():
        h ^= byte
        h = (h * 0x100000001b3) & 0xFFFFFFFFFFFFFFFF
    return h
