"""The on-disk formats behind the C ABI: workload snapshots (raw GpuBoid arrays, the reference's
tools/benchmark/bench_common.hpp saveSnapshot / loadSnapshot) and the baked terrace volume (stadium.sdf, raw float32
130^3, the reference's src/sdf.cpp loadSDFVolume) and the navigation-field cache files of the seated venues (nav::save /
nav::load, src/nav_field.cpp:554-656). Host code only: no GPU."""
import os

import numpy as np
import pytest


def test_snapshot_round_trip_is_bit_exact(built, terrace_golden, tmp_path):
    import swarm_gb300
    st = terrace_golden["spawn"]
    path = tmp_path / "terrace_spawn.bin"
    swarm_gb300.snapshot_write(path, st)
    assert path.stat().st_size == st.shape[0] * 32
    back = swarm_gb300.snapshot_read(path)
    assert back.shape == st.shape
    assert np.array_equal(back.view(np.uint32), np.ascontiguousarray(st, np.float32).view(np.uint32))


def test_snapshot_file_is_the_raw_gpuboid_array(built, tmp_path):
    """Byte layout: 8 float32 per agent (pos.xyz, active, vel.xyz, padding), little-endian, no header."""
    import swarm_gb300
    st = np.arange(5 * 8, dtype=np.float32).reshape(5, 8)
    path = tmp_path / "s.bin"
    swarm_gb300.snapshot_write(path, st)
    assert path.read_bytes() == st.astype("<f4").tobytes()


def test_snapshot_size_checks(built, tmp_path):
    import swarm_gb300
    from swarm_gb300 import lib
    from swarm_gb300.abi import SWARM_E_INVALID
    ragged = tmp_path / "ragged.bin"
    ragged.write_bytes(b"\0" * 33)
    assert lib().swarm_snapshot_count(bytes(ragged)) == -1
    with pytest.raises(swarm_gb300.SwarmError):
        swarm_gb300.snapshot_read(ragged)
    empty = tmp_path / "empty.bin"
    empty.write_bytes(b"")
    assert lib().swarm_snapshot_count(bytes(empty)) == -1
    assert lib().swarm_snapshot_count(bytes(tmp_path / "missing.bin")) == -1
    four = tmp_path / "four.bin"
    four.write_bytes(b"\0" * 128)
    out = np.empty((3, 8), np.float32)
    # the reader wants exactly n agents, as the reference's loadSnapshot does
    assert lib().swarm_snapshot_read(bytes(four), swarm_gb300.fptr(out), 3) == SWARM_E_INVALID
    assert lib().swarm_snapshot_write(bytes(tmp_path / "x.bin"), swarm_gb300.fptr(out), 0) == SWARM_E_INVALID


def test_sdf_read_round_trip(built, stadium_sdf, tmp_path):
    import swarm_gb300
    path = tmp_path / "stadium.sdf"
    path.write_bytes(np.ascontiguousarray(stadium_sdf, "<f4").tobytes())
    assert path.stat().st_size == 130 ** 3 * 4
    back = swarm_gb300.sdf_read(path)
    assert np.array_equal(back.view(np.uint32), np.ascontiguousarray(stadium_sdf, np.float32).reshape(-1).view(np.uint32))
    short = tmp_path / "short.sdf"
    short.write_bytes(path.read_bytes()[:-4])
    with pytest.raises(swarm_gb300.SwarmError):
        swarm_gb300.sdf_read(short)
    with pytest.raises(swarm_gb300.SwarmError):
        swarm_gb300.sdf_read(path, res=129)


def _nav_cache_bytes(res, origin, cell, anchor, cls, dist, exit_id, names, key=0x1234, version=2):
    """A navigation-field cache file in the reference's format (nav::save, src/nav_field.cpp:554-595)."""
    import struct
    n = res * res
    payload = struct.pack("<IIfffIQ", version, res, origin, cell, np.float32(res / (res * cell)), len(names), key)
    payload += np.zeros(n, np.float32).tobytes() + np.asarray(cls, np.uint8).tobytes() + np.zeros(n, np.uint8).tobytes()
    payload += np.full(n, -1, np.int8).tobytes() + np.asarray(dist, np.float32).tobytes()
    payload += np.asarray(anchor, np.int32).tobytes() + np.asarray(exit_id, np.uint8).tobytes()
    for nm in names:
        payload += struct.pack("<I", len(nm)) + nm
    h = 0xcbf29ce484222325
    for b in payload:
        h = ((h ^ b) * 0x100000001b3) & 0xFFFFFFFFFFFFFFFF
    return b"SWNAVF01" + payload + struct.pack("<Q", h)


def test_nav_cache_file_reads_into_the_gpu_table(built, tmp_path):
    """swarm_nav_cache_read on a small cache file written to the reference's format: anchors to cell centres (an
    unreachable cell's own), the info bits (exit id, FIT, reachable); a damaged checksum, another version or another
    key are refused."""
    import swarm_gb300
    res, origin, cell = 5, -1.0, 0.4
    rng = np.random.default_rng(3)
    n = res * res
    anchor = rng.integers(0, n, n).astype(np.int32)
    dist = rng.uniform(0.0, 3.0, n).astype(np.float32)
    dist[[3, 7]] = np.inf
    anchor[[3, 7]] = -1
    cls = rng.integers(0, 2, n).astype(np.uint8)
    exit_id = rng.integers(0, 12, n).astype(np.uint8)
    p = tmp_path / "nav_T.bin"
    p.write_bytes(_nav_cache_bytes(res, origin, cell, anchor, cls, dist, exit_id, [b"avenue +x", b"door"]))
    cells, grid = swarm_gb300.nav_cache_read(str(p))
    assert grid[0] == res and grid[1] == np.float32(origin) and grid[2] == np.float32(cell)
    a = np.where(anchor >= 0, anchor, np.arange(n))
    centre = (np.float64(np.float32(origin)) + (np.arange(res) + 0.5) * np.float64(np.float32(cell))).astype(np.float32)
    assert np.array_equal(cells[:, 0], centre[a % res]) and np.array_equal(cells[:, 1], centre[a // res])
    assert np.array_equal(cells[:, 2], dist)
    info = exit_id.astype(np.uint32) | np.where(cls == 0, 0x100, 0) | np.where(np.isfinite(dist), 0x200, 0)
    assert np.array_equal(cells[:, 3].view(np.uint32), info.astype(np.uint32))
    assert swarm_gb300.nav_cache_read(str(p), expected_key=0x1234)[1][0] == res
    bad = bytearray(p.read_bytes())
    bad[-1] ^= 1
    q = tmp_path / "bad.bin"
    q.write_bytes(bytes(bad))
    for path, key in ((q, 0), (p, 0x999)):
        with pytest.raises(swarm_gb300.SwarmError):
            swarm_gb300.nav_cache_read(str(path), expected_key=key)
    q.write_bytes(_nav_cache_bytes(res, origin, cell, anchor, cls, dist, exit_id, [], version=3))
    with pytest.raises(swarm_gb300.SwarmError):
        swarm_gb300.nav_cache_read(str(q))


def test_nav_cache_file_of_the_reference_equals_its_gpu_table(built, tmp_path):
    """The cache file the reference writes for venue S (nav::forVenue builds and saves it), read by
    swarm_nav_cache_read, equals the reference's own GPU table (nav::gpuCells) bit for bit. Needs the reference's CPU
    build (this container)."""
    import ctypes as C
    import glob
    from oracle import oracle as O
    import swarm_gb300
    if not O.ref_available():
        pytest.skip("the reference's CPU build is not here")
    cache = os.environ.get("SWARM_NAV_CACHE") or str(tmp_path / "navcache")
    os.environ["SWARM_NAV_CACHE"] = cache
    L = O.ref_lib()
    V = C.c_void_p
    L.ref_nav_table.argtypes = [C.c_char_p, V, C.c_int, V, V, V]
    o, c, ic = C.c_float(), C.c_float(), C.c_float()
    res = L.ref_nav_table(b"S", None, 0, C.byref(o), C.byref(c), C.byref(ic))
    want = np.empty((res * res, 4), np.float32)
    assert L.ref_nav_table(b"S", want.ctypes.data, res * res, C.byref(o), C.byref(c), C.byref(ic)) == res
    files = glob.glob(os.path.join(cache, "nav_S_*.bin"))
    assert len(files) == 1
    key = int(os.path.basename(files[0])[6:-4], 16)
    cells, grid = swarm_gb300.nav_cache_read(files[0], expected_key=key)
    assert grid == (res, o.value, c.value, ic.value)
    assert np.array_equal(cells.view(np.uint32), want.view(np.uint32))
