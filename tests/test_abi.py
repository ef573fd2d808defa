"""The C ABI: the library loads on a machine without a GPU, exports every entry point include/*.h declares, and its
structs have the header's layout. No compute call here."""
import ctypes as C
import os
import re
import subprocess

import pytest

from conftest import ROOT


def _declared():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            text = open(os.path.join(inc, f)).read()
            names |= set(re.findall(r"^\s*(?:int|void|const char\*)\s+(swarm_\w+)\s*\(", text, re.M))
    return names


def test_library_exports_every_declared_symbol(built):
    import swarm_gb300
    names = _declared()
    assert len(names) >= 20
    lib = C.CDLL(swarm_gb300.LIB_PATH)
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_layouts_match_header(tmp_path):
    from swarm_gb300.abi import SwarmParams, SwarmStageTimes, SwarmVenue
    from swarm_gb300.venues import HallSpec
    src = tmp_path / "sz.c"
    src.write_text('#include "swarm_cuda.h"\n#include <stdio.h>\n#include <stddef.h>\n'
                   'int main(void){printf("%zu %zu %zu %zu %zu %zu\\n", sizeof(SwarmParams), sizeof(SwarmVenue),'
                   ' sizeof(SwarmStageTimes), sizeof(SwarmHallSpec), offsetof(SwarmVenue, wall_sdf),'
                   ' offsetof(SwarmParams, park_coord)); return 0;}\n')
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    want = [C.sizeof(SwarmParams), C.sizeof(SwarmVenue), C.sizeof(SwarmStageTimes), C.sizeof(HallSpec),
            SwarmVenue.wall_sdf.offset, SwarmParams.park_coord.offset]
    assert got == want


def test_reference_constants_are_the_folded_ones(built):
    """sim_params.hpp's static_asserts and folds (include/swarm/sim_params.hpp:90-92, 118, 272, 418)."""
    import numpy as np
    import swarm_gb300
    p = swarm_gb300.params_reference()
    f32 = np.float32
    assert p.body_diam == f32(0.0128) and p.r_sep == f32(0.016)
    assert 96.0 < p.gravity_dt / f32(0.01) < 96.1
    assert 0.0095 < p.max_step_up < 0.0097
    assert p.perc_ring == 1 and p.proj_iterations == 32
    # GLSL-style folding: 1.25 * 0.0064 folded in double from the decimals, rounded once
    assert p.feeler_reach == f32(0.008)
    assert p.hash_to_radians == f32(6.28318530718 / 4294967296.0)
    assert p.feeler_off[1][0] == f32(f32(0.92387953) * p.feeler_reach)


def test_invalid_arguments_are_rejected_without_a_gpu(built):
    import swarm_gb300
    from swarm_gb300.abi import SwarmVenue, SWARM_E_INVALID
    L = swarm_gb300.lib()
    h = C.c_void_p()
    p = swarm_gb300.params_reference()
    v = SwarmVenue()   # kind 0 without an SDF
    assert L.swarm_create(C.byref(p), C.byref(v), 16, C.byref(h)) == SWARM_E_INVALID
    assert L.swarm_create(C.byref(p), C.byref(v), 0, C.byref(h)) == SWARM_E_INVALID
    assert L.swarm_step(None, 1) == SWARM_E_INVALID
    assert L.swarm_params_si(None) == SWARM_E_INVALID


def test_product_has_no_cpu_fallback():
    """The package never imports or loads the oracle."""
    pkg = os.path.join(ROOT, "swarm-crowd-simulation_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".cpp", ".h")):
                text = open(os.path.join(dirpath, f)).read()
                for needle in ("import oracle", "from oracle", "liboracle", "oracle_create", "libswarm_ref"):
                    assert needle not in text, (f, needle)


def _mirrors():
    """Every ctypes mirror of a header struct, with the header's name."""
    from swarm_gb300 import abi, venues
    out = {name: cls for name, cls in vars(abi).items()
           if isinstance(cls, type) and issubclass(cls, C.Structure) and name.startswith("Swarm")}
    out["SwarmHallSpec"] = venues.HallSpec
    out["SwarmBowlSpec"] = venues.BowlSpec
    return out


def test_every_struct_mirror_has_the_header_layout(tmp_path):
    """Size and every field's offset of each ctypes mirror, against the header compiled by gcc."""
    mirrors = _mirrors()
    assert len(mirrors) >= 12
    lines, want = [], []
    for name, cls in sorted(mirrors.items()):
        lines.append(f'printf("%zu\\n", sizeof({name}));')
        want.append(C.sizeof(cls))
        for field in cls._fields_:
            lines.append(f'printf("%zu\\n", offsetof({name}, {field[0]}));')
            want.append(getattr(cls, field[0]).offset)
    src = tmp_path / "layout.c"
    src.write_text('#include "swarm_cuda.h"\n#include <stdio.h>\n#include <stddef.h>\nint main(void){\n' +
                   "\n".join(lines) + "\nreturn 0;}\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert got == want
