"""Writes tests/golden/seated_S.npz: the reference's seated venue S and runs of its unmodified CPU step (oracle/_ref,
built from the reference's own sources by oracle/Makefile), for the GPU tests of the seated venue.

    python tests/golden/make_seated_golden.py      (needs the reference tree: REF_DIR=<tree> make -C oracle ref)

Contents:
  layout            venue S's swarm::SeatedLayout in the C ABI's SwarmSeatedLayout bytes; grid = (gridRes, domainMin,
                    domainSpan, exitDepth, exitMaxZ); incline = sim_params.hpp's V_STAIR_UP, V_STAIR_DOWN,
                    INCLINE_INV_REF_SLOPE, T_HEADWAY, T_HEADWAY_STAIR_UP/_DOWN (EMPIRICAL, CONSERVATIVE)
  nav_*             the navigation field's GPU table (nav::gpuCells of nav::forVenue) in a compact form: per cell the
                    anchor cell's index (delta-coded along the row-major order) and the info word; the anchor's
                    position is its cell centre (nav::Grid::centre, double arithmetic rounded once; an unreachable
                    cell's own centre), checked here against the table; the distance is not kept (the step reads only
                    the anchor and the info bits)
  dense_*           the dense forced scenario of the reference's venue tests (tools/venue_s.hpp denseSetup: every seat
                    occupied, each agent along its row to the nearer gangway, down it and out): the spawn, the drive
                    table of each of the first 250 steps (XOR-delta coded across steps; the drive table is a function of
                    the state, so a bit-exact step meets exactly these tables), the state, sorted pairs, cell table and
                    contact bits after step 1, and the state after 250 steps, whose FNV-1a hash is the reference's own
                    pin "CPU counting venue S dense" (tools/golden_state.hpp:45)
  nearest_*         spawnSeatedCrowd(venueS(), 4096, 1.0, 1337) under ModelOptions{} (nearest exit, level speed): the
                    spawn, the state etc. after step 1, the states after 10, 50 and 250 steps; the last is the pin
                    "CPU counting venue S nearest exit, level speed" (golden_state.hpp:62)
  incline_*         the same spawn under {nearest exit, incline speed, stair spacing EMPIRICAL}: states after 1, 50 and
                    250 steps (the reference's output; the reference pins this model only with the queue-aware choice)

tests/golden/seated_S_choice.npz: venue S's queue-aware exit choice as the reference builds it (nav::choiceForVenue) in
a compact form -- per exit its anchor and its 16-bit distance at every entry (delta-coded along the entries, lzma), the
exit of every slot (lzma), the capacity terms; the index words follow from the navigation table's FIT and REACHABLE
bits (checked here), the empty slots are constant (checked) -- and the reference's routed runs of the seat spawn
under its default model {queue-aware, incline speed, stair spacing EMPIRICAL}: the assignments and counters after
steps 1, 17 and 18 (the first evaluation), the states after 1 and 18 steps, the state hashes after 50 and 250 steps
(the last: the pin "CPU counting venue S routed", golden_state.hpp:55), and the 250-step hash with the level spacing
(pin golden_state.hpp:69). Written alone by `python tests/golden/make_seated_golden.py choice`.

and tests/golden/seated_M.npz, seated_L.npz: the generated venues M (15 832 seats, N = 16 384) and L (63 424 seats,
N = 65 536) -- several straight gangways, doors per gangway head, corner doors, merged corner gangways -- with the
layout, grid, compact navigation table as above, the full seat spawn spawnSeatedCrowd(venue, N, 1.0, 1337) (zlib), and
the FNV-1a hashes of the reference's states after 1, 10, 50 and 250 steps under {nearest exit, level speed} and after
10 and 250 steps under {nearest exit, incline speed, stair spacing EMPIRICAL}. Written alone by
`python tests/golden/make_seated_golden.py generated`.

tests/golden/seated_S_evac.npz: the active count after every step of venue S's full seat spawn run by the reference's
CPU step to its last agent out, routed (its default model) and at the nearest exit and level speed. Written alone by
`python tests/golden/make_seated_golden.py evacuation`; tests/golden/seated_M_evac.npz, seated_L_evac.npz: the same for
M and L at the nearest exit, at the level speed and with the incline speed and stair spacing
(`python tests/golden/make_seated_golden.py generated_evacuation M L`).
"""
import ctypes as C
import lzma
import os
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.join(HERE, "..", "..")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "swarm-crowd-simulation_gb300"))
from oracle import oracle as O  # noqa: E402
from swarm_gb300.abi import SwarmSeatedLayout  # noqa: E402
sys.path.insert(0, HERE)
from seated_choice import EMPTY_SLOT, choice_index, decode_choice_entries  # noqa: E402

PIN_DENSE = 0xa2abaea7c0139b09     # golden_state.hpp:45  CPU counting venue S dense
PIN_NEAREST = 0xb1d6dac42f5dcd09   # golden_state.hpp:62  CPU counting venue S nearest exit, level speed
PIN_ROUTED = 0x434356ac8d65471d    # golden_state.hpp:55  CPU counting venue S routed
PIN_ROUTED_LEVEL = 0x22ad15f59ee18632   # golden_state.hpp:69  CPU counting venue S routed, level spacing
STEPS = 250                        # golden_state.hpp:19  GOLDEN_STEPS
CHOICE_STEPS = 17                  # sim_params.hpp:417-418


def fnv1a(a):
    """The reference's golden::stateHash (golden_state.hpp:121-126): 64-bit FNV-1a over the raw state bytes."""
    h = 0xcbf29ce484222325
    for x in np.ascontiguousarray(a).view(np.uint8).tobytes():
        h = ((h ^ x) * 0x100000001b3) & 0xFFFFFFFFFFFFFFFF
    return h


def _bind(L):
    V = C.c_void_p
    L.ref_create_opts.restype = V
    L.ref_create_opts.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
    L.ref_set_drive.argtypes = [V, V, C.c_int]
    L.ref_dense_setup.argtypes = [C.c_char_p, V, C.c_int]
    L.ref_dense_drive.argtypes = [C.c_char_p, V, C.c_int, V]
    L.ref_seated_layout.argtypes = [C.c_char_p, V, V, V, V, V, V]
    L.ref_incline_constants.argtypes = [V]
    L.ref_nav_table.argtypes = [C.c_char_p, V, C.c_int, V, V, V]
    return L


def _sim(L, venue, incline=0, stair=0):
    s = O.RefSim.__new__(O.RefSim)
    s._h = L.ref_create_opts(venue, 0, 0, 0, incline, stair)
    assert s._h, L.ref_last_error()
    s.n = 0
    return s


def _one_step_record(prefix, sim, out):
    out[prefix + "state1"] = sim.state()
    g, b = sim.grid()
    out[prefix + "grid1_key"], out[prefix + "grid1_id"] = g, b
    out[prefix + "cells1"] = sim.cells(40 * 40)
    out[prefix + "contacts1"] = sim.contacts()


def _venue_records(L, venue, out):
    """The layout, grid, incline constants and compact navigation table of a seated venue into out."""
    lay = SwarmSeatedLayout()
    res, dmin, dspan, edep, emaxz = C.c_int(), C.c_float(), C.c_float(), C.c_float(), C.c_float()
    assert L.ref_seated_layout(venue, C.byref(lay), C.byref(res), C.byref(dmin), C.byref(dspan), C.byref(edep), C.byref(emaxz)) == 0
    out["layout"] = np.frombuffer(bytes(lay), np.uint8)
    out["grid"] = np.array([res.value, dmin.value, dspan.value, edep.value, emaxz.value], np.float64)
    inc = np.empty(8, np.float32)
    L.ref_incline_constants(inc.ctypes.data)
    out["incline"] = inc

    # the navigation field, compact
    org, cell, inv = C.c_float(), C.c_float(), C.c_float()
    nres = L.ref_nav_table(venue, None, 0, C.byref(org), C.byref(cell), C.byref(inv))
    nav = np.empty((nres * nres, 4), np.float32)
    L.ref_nav_table(venue, nav.ctypes.data, nres * nres, C.byref(org), C.byref(cell), C.byref(inv))
    info = nav[:, 3].view(np.uint32).copy()
    centre = (np.float64(org.value) + (np.arange(nres, dtype=np.float64) + 0.5) * np.float64(cell.value)).astype(np.float32)
    cx = np.searchsorted(centre, nav[:, 0])
    cy = np.searchsorted(centre, nav[:, 1])
    assert (cx < nres).all() and (cy < nres).all()
    anchor = (cx + cy * nres).astype(np.int64)
    assert np.array_equal(centre[cx], nav[:, 0]) and np.array_equal(centre[cy], nav[:, 1]), "anchors are cell centres"
    reach = (info & 0x200) != 0
    assert np.array_equal(np.isfinite(nav[:, 2]), reach)
    own = np.arange(nres * nres)
    assert np.array_equal(anchor[~reach], own[~reach]), "an unreachable cell's anchor is its own centre"
    delta = np.diff(anchor, prepend=0).astype(np.int32)
    out["nav_grid"] = np.array([nres, org.value, cell.value, inv.value], np.float64)
    out["nav_anchor_delta_z"] = np.frombuffer(zlib.compress(delta.tobytes(), 9), np.uint8)
    out["nav_info_z"] = np.frombuffer(zlib.compress(info.tobytes(), 9), np.uint8)
    return res.value


def generated_venue(L, name, n):
    """seated_M.npz / seated_L.npz: the venue, its full seat spawn and the reference's state hashes."""
    out = {}
    _venue_records(L, name, out)
    spawn = np.empty((n, 8), np.float32)
    assert L.ref_spawn_seated(name, n, 1.0, 1337, spawn.ctypes.data) == 0
    out["spawn_z"] = np.frombuffer(zlib.compress(spawn.tobytes(), 9), np.uint8)
    out["n"] = np.array([n, int((spawn[:, 3] != 0).sum())], np.int64)
    for prefix, incline, stair, keep in (("nearest_", 0, 0, (1, 10, 50, 250)), ("incline_", 1, 1, (10, 250))):
        sim = _sim(L, name, incline, stair)
        sim.set_state(spawn)
        done = 0
        for k in keep:
            sim.step(k - done)
            done = k
            out[prefix + "hash%d" % k] = np.array([fnv1a(sim.state())], np.uint64)
    path = os.path.join(HERE, "seated_%s.npz" % name.decode())
    np.savez_compressed(path, **out)
    print("wrote", os.path.basename(path), os.path.getsize(path), "bytes")


def evacuation_records(L):
    """seated_S_evac.npz: the reference's CPU step on venue S from the full seat spawn run to its last agent out, under
    its default model (queue-aware exit choice, incline speed, stair spacing EMPIRICAL), the same with the level
    spacing, at the nearest exit and level speed, and at the nearest exit with the incline speed and stair spacing:
    the active count after every step (the routed run empties at step 1361, as the reference's own validation output
    records for its CPU counting sort)."""
    g = np.load(os.path.join(HERE, "seated_S.npz"))
    spawn = g["nearest_spawn"]
    out = {}
    for prefix, opts in (("routed_", (0, 0, 1, 1, 1)), ("nearest_", (0, 0, 0, 0, 0)), ("routed_level_", (0, 0, 1, 1, 0)),
                         ("incline_", (0, 0, 0, 1, 1))):
        sim = O.RefSim.__new__(O.RefSim)
        sim._h = L.ref_create_opts(b"S", *opts)
        sim.n = 0
        sim.set_state(spawn)
        active = []
        while not active or (active[-1] > 0 and len(active) < 5000):
            sim.step(1)
            active.append(int((sim.state()[:, 3] != 0).sum()))
        assert active[-1] == 0
        out[prefix + "active"] = np.array(active, np.int32)
    assert out["routed_active"].shape[0] == 1361, out["routed_active"].shape
    path = os.path.join(HERE, "seated_S_evac.npz")
    np.savez_compressed(path, **out)
    print("wrote seated_S_evac.npz:", os.path.getsize(path), "bytes")


def generated_evacuation(L, name):
    """seated_<name>_evac.npz: the reference's CPU step on a generated venue (M or L) from its full seat spawn (the
    fixture's) run to its last agent out at the nearest exit, at the level speed and with the incline speed and stair
    spacing: the active count after every step."""
    g = np.load(os.path.join(HERE, "seated_%s.npz" % name.decode()))
    spawn = np.frombuffer(zlib.decompress(g["spawn_z"].tobytes()), np.float32).reshape(-1, 8).copy()
    out = {}
    for prefix, incline in (("nearest_", 0), ("incline_", 1)):
        sim = _sim(L, name, incline, incline)
        sim.set_state(spawn)
        active = []
        while not active or (active[-1] > 0 and len(active) < 40000):
            sim.step(1)
            active.append(int((sim.state()[:, 3] != 0).sum()))
        assert active[-1] == 0
        out[prefix + "active"] = np.array(active, np.int32)
    path = os.path.join(HERE, "seated_%s_evac.npz" % name.decode())
    np.savez_compressed(path, **out)
    print("wrote", os.path.basename(path), os.path.getsize(path), "bytes,", {k: v.shape[0] for k, v in out.items()}, "steps")


def _lz(a):
    return np.frombuffer(lzma.compress(np.ascontiguousarray(a).tobytes(), preset=9 | lzma.PRESET_EXTREME), np.uint8)


def choice_records(L):
    """seated_S_choice.npz (see the module docstring)."""
    V = C.c_void_p
    L.ref_choice_table.restype = C.c_longlong
    L.ref_choice_table.argtypes = [C.c_char_p, V, C.c_longlong, V, C.c_longlong, V, V]
    L.ref_choice_state.argtypes = [V, V, C.c_int, V, V]
    meta = np.zeros(3 + 64, np.float32)
    res = C.c_int()
    ne = L.ref_choice_table(b"S", None, 0, None, 0, meta.ctypes.data, C.byref(res))
    assert ne > 0, L.ref_last_error()
    cells = res.value * res.value
    index = np.empty(cells, np.uint32)
    entries = np.empty((ne, 36), np.uint32)
    assert L.ref_choice_table(b"S", index.ctypes.data, cells, entries.ctypes.data, ne, meta.ctypes.data, C.byref(res)) == ne
    E = int(meta[0])
    # the index from the navigation table: the class bit, and entries numbered in grid order over FIT + REACHABLE cells
    g = np.load(os.path.join(HERE, "seated_S.npz"))
    info = np.frombuffer(zlib.decompress(g["nav_info_z"].tobytes()), np.uint32)
    assert int(g["nav_grid"][0]) == res.value
    assert np.array_equal(choice_index(info), index), "the index follows from the navigation table"
    slot, dist = entries[:, :24], entries[:, 24:]
    ex = ((slot >> 25) & 63).astype(np.uint8)
    q = np.stack([(dist[:, k >> 1] >> ((k & 1) * 16)) & 0xFFFF for k in range(24)], 1)
    assert np.all(slot[ex == 63] == EMPTY_SLOT) and np.all(q[ex == 63] == 0xFFFF) and np.all(slot >> 31 == 1)
    rows = np.arange(ne)
    anchor = np.zeros((E, ne), np.int64)
    dq = np.zeros((E, ne), np.int64)
    seen = np.zeros((E, ne), bool)
    for k in range(24):
        m = ex[:, k] != 63
        e = ex[m, k].astype(np.int64)
        anchor[e, rows[m]] = slot[m, k] & 0x1FFFFFF
        dq[e, rows[m]] = q[m, k]
        seen[e, rows[m]] = True
    assert seen.all(), "every exit is a candidate of every entry (the venue has fewer exits than slots)"
    out = {"choice_meta": meta[:3 + E].copy(), "choice_grid": np.array([res.value, ne, CHOICE_STEPS], np.int64),
           "choice_order_lz": _lz(ex),
           "choice_anchor_lz": _lz(np.diff(anchor, axis=1, prepend=0).astype(np.int32)),
           "choice_q_lz": _lz(np.diff(dq, axis=1, prepend=0).astype(np.int32))}
    # the decoding the tests use gives the reference's words back
    assert np.array_equal(decode_choice_entries(out), entries)

    spawn = np.empty((4096, 8), np.float32)
    assert L.ref_spawn_seated(b"S", 4096, 1.0, 1337, spawn.ctypes.data) == 0
    sim = O.RefSim.__new__(O.RefSim)
    sim._h = L.ref_create_opts(b"S", 0, 0, 1, 1, 1)
    sim.n = 0
    sim.set_state(spawn)
    assign = np.empty(4096, np.uint32)
    counters = np.empty(132, np.uint32)
    cstep = C.c_uint32()
    for s in range(1, STEPS + 1):
        sim.step(1)
        if s in (1, 17, 18):
            L.ref_choice_state(sim._h, assign.ctypes.data, 4096, counters.ctypes.data, C.byref(cstep))
            assert cstep.value == s
            out["routed_assign%d" % s] = assign.copy()
            out["routed_counters%d" % s] = counters.copy()
        if s in (1, 18):
            out["routed_state%d" % s] = sim.state()
        if s in (50, STEPS):
            out["routed_hash%d" % s] = np.array([fnv1a(sim.state())], np.uint64)
    assert int(out["routed_hash250"][0]) == PIN_ROUTED, "%016x" % int(out["routed_hash250"][0])
    sim = O.RefSim.__new__(O.RefSim)
    sim._h = L.ref_create_opts(b"S", 0, 0, 1, 1, 0)
    sim.n = 0
    sim.set_state(spawn)
    sim.step(STEPS)
    out["level_hash250"] = np.array([fnv1a(sim.state())], np.uint64)
    assert int(out["level_hash250"][0]) == PIN_ROUTED_LEVEL, "%016x" % int(out["level_hash250"][0])
    path = os.path.join(HERE, "seated_S_choice.npz")
    np.savez_compressed(path, **out)
    print("wrote seated_S_choice.npz:", os.path.getsize(path), "bytes")


def main():
    os.environ.setdefault("SWARM_NAV_CACHE", os.path.join("/tmp", "swarm_navcache"))
    O.build(ref=True)
    assert O.ref_available(), "the reference tree is needed: REF_DIR=<tree> make -C oracle ref"
    L = _bind(O.ref_lib())
    if sys.argv[1:] == ["choice"]:
        choice_records(L)
        return
    if sys.argv[1:] == ["evacuation"]:
        evacuation_records(L)
        return
    if sys.argv[1:2] == ["generated_evacuation"]:
        for name in sys.argv[2:] or ["M", "L"]:
            generated_evacuation(L, name.encode())
        return
    if sys.argv[1:] == ["generated"]:
        generated_venue(L, b"M", 16384)
        generated_venue(L, b"L", 65536)
        return
    out = {}
    assert _venue_records(L, b"S", out) == 40

    # the dense forced scenario
    n = L.ref_dense_setup(b"S", None, 0)
    spawn = np.empty((n, 8), np.float32)
    L.ref_dense_setup(b"S", spawn.ctypes.data, n)
    sim = _sim(L, b"S")
    sim.set_state(spawn)
    cur = spawn
    tables = []
    for s in range(STEPS):
        d = np.empty((n, 2), np.float32)
        L.ref_dense_drive(b"S", cur.ctypes.data, n, d.ctypes.data)
        tables.append(d)
        L.ref_set_drive(sim._h, d.ctypes.data, n)
        sim.step(1)
        cur = sim.state()
        if s == 0:
            _one_step_record("dense_", sim, out)
    assert fnv1a(cur) == PIN_DENSE, "%016x" % fnv1a(cur)
    U = np.stack(tables).view(np.uint32)
    X = U.copy()
    X[1:] ^= U[:-1]
    out["dense_spawn"] = spawn
    out["dense_drive_xor_z"] = np.frombuffer(zlib.compress(X.tobytes(), 9), np.uint8)
    out["dense_state250"] = cur

    # nearest exit, level speed; then the incline speed and stair spacing
    spawn = np.empty((4096, 8), np.float32)
    assert L.ref_spawn_seated(b"S", 4096, 1.0, 1337, spawn.ctypes.data) == 0
    out["nearest_spawn"] = spawn
    for prefix, incline, stair, keep in (("nearest_", 0, 0, (10, 50, 250)), ("incline_", 1, 1, (50, 250))):
        sim = _sim(L, b"S", incline, stair)
        sim.set_state(spawn)
        for s in range(1, STEPS + 1):
            sim.step(1)
            if s == 1:
                _one_step_record(prefix, sim, out)
            if s in keep:
                out[prefix + "state%d" % s] = sim.state()
        if prefix == "nearest_":
            assert fnv1a(out["nearest_state250"]) == PIN_NEAREST, "%016x" % fnv1a(out["nearest_state250"])
    out["incline_hash250"] = np.array([fnv1a(out["incline_state250"])], np.uint64)
    np.savez_compressed(os.path.join(HERE, "seated_S.npz"), **out)
    print("wrote seated_S.npz:", os.path.getsize(os.path.join(HERE, "seated_S.npz")), "bytes")
    choice_records(L)
    generated_venue(L, b"M", 16384)
    generated_venue(L, b"L", 65536)
    evacuation_records(L)
    generated_evacuation(L, b"M")
    generated_evacuation(L, b"L")


if __name__ == "__main__":
    main()
