"""Build libvx_cuda.so in-tree for sm_103a (no cmake; a few translation units in parallel).

FP64 kernel files (``*64.cu``) are compiled with ``--fmad=false`` so that every double
expression keeps the reference's separate IEEE multiply/add rounding; host code uses
``-ffp-contract=off`` for the same reason on aarch64, where GCC would otherwise fuse.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIB = HERE / "libvx_cuda.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def build(force: bool = False, verbose: bool = False) -> Path:
    srcs = sources()
    deps = srcs + list(CSRC.glob("*.hpp")) + list(CSRC.glob("*.cuh")) + [HERE.parent / "include" / "vx.h", HERE.parent / "include" / "veritas_gb300.hpp",
                                              HERE / "driver" / "veritas_gb300_run.cpp", Path(__file__)]
    if LIB.exists() and (HERE / "veritas_gb300_run").exists() and not force:
        t = LIB.stat().st_mtime
        if all(p.stat().st_mtime <= t for p in deps):
            return LIB
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    host_flags = ["-O2", "-fPIC", "-ffp-contract=off", "-std=c++17"]
    jobs = []
    for s in srcs:
        obj = BUILD / (s.name + ".o")
        if s.suffix == ".cu":
            cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                   "-I", str(CSRC), "-c", str(s), "-o", str(obj)]
            if s.stem.endswith("64"):
                cmd.insert(1, "--fmad=false")
            if s.name == "fct64.cu":  # the FP64 FCT kernels once more, contracted (fast form)
                fast = BUILD / "fct64_fast.cu.o"
                jobs.append(([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-DVX_FP64_FAST", "-Xcompiler",
                              "-fPIC", "-I", str(CSRC), "-c", str(s), "-o", str(fast)], fast))
        else:
            cmd = [nvcc, "-x", "cu", *ARCH, "-O3", "-std=c++17", "-Xcompiler", ",".join(host_flags),
                   "-I", str(CSRC), "-c", str(s), "-o", str(obj)]
        jobs.append((cmd, obj))
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        futs = [ex.submit(_run, c) for c, _ in jobs]
        for f in futs:
            f.result()
    tmp = LIB.with_suffix(".so.tmp")
    _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *[str(o) for _, o in jobs], "-lcudart", "-lpthread",
          "-Xlinker", "--no-undefined"])
    os.replace(tmp, LIB)
    # the stand-alone C++ driver over include/veritas_gb300.hpp, found next to the library
    drv = HERE / "veritas_gb300_run"
    _run(["g++", "-O2", "-std=c++17", "-I", str(HERE.parent / "include"), str(HERE / "driver" / "veritas_gb300_run.cpp"),
          "-L", str(HERE), "-lvx_cuda", "-Wl,-rpath,$ORIGIN", "-o", str(drv)])
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
