"""Builds libswarm_gb300.so in-tree: the CUDA kernels for sm_103a and the host C++ of the C ABI.

    python swarm-crowd-simulation_gb300/build.py [--force]

Every .cu is compiled with -fmad=false and without fast math: the step's float arithmetic must round exactly as the
reference's CPU arithmetic (no fused multiply-adds). Objects compile in parallel; only changed sources recompile.
"""
import concurrent.futures as cf
import os
import platform
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build", platform.machine())
LIB = os.path.join(PKG, "libswarm_gb300.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
                  "-Xcompiler", "-fPIC,-ffp-contract=off", "-Xptxas", "-warn-spills"]
CXXFLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off"]


def _sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cu, cpp


def _headers_mtime():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h", ".hpp"))]
    hs.append(os.path.join(PKG, "..", "include", "swarm_cuda.h"))
    return max(os.path.getmtime(h) for h in hs)


def _compile(src, force, hdr_mtime):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if not force and os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), hdr_mtime):
        return obj, None
    if src.endswith(".cu"):
        cmd = [NVCC] + NVFLAGS + ["-c", src, "-o", obj]
    else:
        cmd = ["g++"] + CXXFLAGS + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, "FAILED: " + " ".join(cmd) + "\n" + r.stdout + r.stderr
    return obj, (r.stdout + r.stderr).strip() or None


def _elf_machine(path):
    """The ELF e_machine of a shared object (62: x86-64, 183: aarch64), None if unreadable."""
    try:
        with open(path, "rb") as f:
            head = f.read(20)
        return int.from_bytes(head[18:20], "little") if head[:4] == b"\x7fELF" else None
    except OSError:
        return None


_MACHINE = {"x86_64": 62, "aarch64": 183, "arm64": 183}.get(platform.machine())


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    cu, cpp = _sources()
    srcs = [os.path.join(CSRC, f) for f in cu + cpp]
    hdr = _headers_mtime()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, force, hdr), srcs))
    errs = [m for _, m in results if m and m.startswith("FAILED")]
    if errs:
        raise RuntimeError("\n".join(errs))
    if verbose:
        for _, m in results:
            if m:
                print(m)
    objs = [o for o, _ in results]
    stale = not os.path.exists(LIB) or _elf_machine(LIB) != _MACHINE or \
        os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs)
    if force or stale:
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
