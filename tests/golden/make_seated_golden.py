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

and tests/golden/seated_M.npz, seated_L.npz: the generated venues M (15 832 seats, N = 16 384) and L (63 424 seats,
N = 65 536) -- several straight gangways, doors per gangway head, corner doors, merged corner gangways -- with the
layout, grid, compact navigation table as above, the full seat spawn spawnSeatedCrowd(venue, N, 1.0, 1337) (zlib), and
the FNV-1a hashes of the reference's states after 1, 10 and 50 steps under {nearest exit, level speed} and after 10
steps under {nearest exit, incline speed, stair spacing EMPIRICAL}.
"""
import ctypes as C
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

PIN_DENSE = 0xa2abaea7c0139b09     # golden_state.hpp:45  CPU counting venue S dense
PIN_NEAREST = 0xb1d6dac42f5dcd09   # golden_state.hpp:62  CPU counting venue S nearest exit, level speed
STEPS = 250                        # golden_state.hpp:19  GOLDEN_STEPS


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
    for prefix, incline, stair, keep in (("nearest_", 0, 0, (1, 10, 50)), ("incline_", 1, 1, (10,))):
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


def main():
    os.environ.setdefault("SWARM_NAV_CACHE", os.path.join("/tmp", "swarm_navcache"))
    O.build(ref=True)
    assert O.ref_available(), "the reference tree is needed: REF_DIR=<tree> make -C oracle ref"
    L = _bind(O.ref_lib())
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
    generated_venue(L, b"M", 16384)
    generated_venue(L, b"L", 65536)


if __name__ == "__main__":
    main()
