"""Build libheatflow_gb300.so in-tree with nvcc for sm_103a (GB300).

Translation units compile in parallel; the set-up and RHS kernels are compiled with -fmad=false
(they restate the reference's arithmetic bit for bit), the solver kernels with FMA.
build_library(checked=True) builds the index-checked variant (-DHF_CHECKED, every global access
of the step kernels checked against its array's extent) into _build/checked/, for tests.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libheatflow_gb300.so")
OUT_CHECKED = os.path.join(OUT, "checked")
LIB_CHECKED = os.path.join(OUT_CHECKED, "libheatflow_gb300_checked.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
          "--expt-relaxed-constexpr", "-Xptxas", "-v"]
# unit -> extra flags
UNITS = {
    "hf_assemble.cu": ["-fmad=false"],
    "hf_rhs.cu": ["-fmad=false"],
    "hf_solve.cu": [],
    "hf_abi.cu": ["-fmad=false"],
    "hf_probe.cu": [],
    "hf_noalloc.cu": [],
}


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(unit: str, flags: list[str], verbose: bool, out: str = OUT) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(out, unit.replace(".cu", ".o"))
    cmd = [nvcc(), *ARCH, *COMMON, *flags, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{r.stderr}")
    with open(obj + ".ptxas.txt", "w") as f:
        f.write(r.stderr)
    if verbose:
        print(r.stderr)
    return obj


def _stale(lib: str = LIB) -> bool:
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "heatflow_gb300.h"))
    deps.append(__file__)
    return any(os.path.getmtime(p) > t for p in deps)


HOST = os.path.join(HERE, "host")
DRIVER = os.path.join(OUT, "heatflow_gb300")
HOST_SOURCES = ["deck.cpp", "heatflow_main.cpp"]


def build_driver(force: bool = False) -> str:
    """The C++ host program (HeatFlow's main program over the C ABI), linked against the library
    with an $ORIGIN run path so it runs from the build folder."""
    deps = [os.path.join(HOST, f) for f in os.listdir(HOST)] + [LIB, __file__]
    if not force and os.path.exists(DRIVER) and all(os.path.getmtime(p) <= os.path.getmtime(DRIVER)
                                                     for p in deps):
        return DRIVER
    gxx = shutil.which("g++") or "g++"
    inc = os.path.join(os.path.dirname(HERE), "include")
    cmd = [gxx, "-O2", "-std=c++17", "-Wall", "-Wextra", "-I", inc,
           *[os.path.join(HOST, f) for f in HOST_SOURCES],
           "-L", OUT, "-lheatflow_gb300", "-Wl,-rpath,$ORIGIN", "-o", DRIVER + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed for the host program:\n{r.stderr}")
    os.replace(DRIVER + ".tmp", DRIVER)
    return DRIVER


def build_library(force: bool = False, verbose: bool = False, checked: bool = False) -> str:
    lib, out = (LIB_CHECKED, OUT_CHECKED) if checked else (LIB, OUT)
    extra = ["-DHF_CHECKED"] if checked else []
    if not force and not _stale(lib):
        return lib
    os.makedirs(out, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1] + extra, verbose, out), UNITS.items()))
    tmp = lib + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build_library(force=True, verbose=False))
    print(build_library(force=True, verbose=False, checked=True))
    print(build_driver(force=True))
