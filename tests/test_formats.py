"""The on-disk formats behind the C ABI: workload snapshots (raw GpuBoid arrays, the reference's
tools/benchmark/bench_common.hpp saveSnapshot / loadSnapshot) and the baked terrace volume (stadium.sdf, raw float32
130^3, the reference's src/sdf.cpp loadSDFVolume). Host code only: no GPU."""
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
