"""In-tree build of the GB300 stepping-loop library (sm_103a).

Compiles the CUDA translation units in parallel with nvcc and links
``celeritas_gb300/_build/libceleritas_gb300.so``. Only ``-gencode
arch=compute_103a,code=sm_103a`` is generated: the library targets GB300.

The FP64 build compiles device code with ``-fmad=false`` so that no multiply
and add are contracted into an fma that the reference's expressions do not
spell out; explicit fma calls (interpolation, axpy, dot products) remain.

The mixed-precision build (``libceleritas_gb300_mixed.so``) compiles the
same sources with ``-DGBX_PHYS_REAL=float``: energies, cross sections, step
limits, multiple scattering, energy loss and the interactors compute in FP32,
while positions, directions, geometry distances, time, the field integrator
and the energy-deposition tally stay FP64. It may contract multiply-adds.
"""

from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_NAMES = {"double": "libceleritas_gb300.so", "mixed": "libceleritas_gb300_mixed.so"}
PRECISIONS = tuple(LIB_NAMES)

SOURCES = [
    "csrc/device/Kernels.cu",
    "csrc/device/Core.cu",
    "csrc/capi.cu",
    "csrc/host/HostParams.cc",
]

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def common_flags(precision: str = "double") -> list[str]:
    flags = ARCH_FLAGS + [
        "-O3",
        "-lineinfo",
        "-std=c++17",
        "-Xcompiler",
        "-fPIC",
        # Host code (table set-up, the elementary functions' host copies)
        # without contraction, as the CPU oracle programs are compiled
        "-Xcompiler",
        "-ffp-contract=off",
        "--expt-relaxed-constexpr",
        "-Xptxas",
        "-v" if os.environ.get("GBX_PTXAS_VERBOSE") else "-O3",
    ]
    if precision == "double":
        flags.append("-fmad=false")
    else:
        flags += ["-fmad=true", "-DGBX_PHYS_REAL=float"]
    return flags


def lib_path(precision: str = "double") -> str:
    return os.path.join(BUILD_DIR, LIB_NAMES[precision])


def _newest_mtime(paths):
    return max(os.path.getmtime(p) for p in paths)


def _deps():
    deps = []
    for root, _dirs, files in os.walk(os.path.join(HERE, "csrc")):
        for f in files:
            if f.endswith((".hh", ".cuh", ".cu", ".cc", ".h")):
                deps.append(os.path.join(root, f))
    deps.append(os.path.join(HERE, "..", "include", "celeritas_gb300.h"))
    deps.append(os.path.abspath(__file__))
    return deps


def build(force: bool = False, verbose: bool = False, precision: str = "double") -> str:
    """Compile and link one library if any source changed; return its path."""
    obj_dir = os.path.join(BUILD_DIR, precision)
    os.makedirs(obj_dir, exist_ok=True)
    out = lib_path(precision)
    if not force and os.path.exists(out) and os.path.getmtime(out) >= _newest_mtime(_deps()):
        return out
    nvcc = nvcc_path()
    flags = common_flags(precision)

    def compile_one(src):
        obj = os.path.join(obj_dir, os.path.basename(src) + ".o")
        cmd = [nvcc] + flags + ["-x", "cu", "-c", os.path.join(HERE, src), "-o", obj]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{res.stderr[-6000:]}")
        if verbose and res.stderr:
            print(res.stderr)
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as pool:
        objs = list(pool.map(compile_one, SOURCES))
    tmp = out + ".tmp"
    cmd = [nvcc] + ARCH_FLAGS + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr[-6000:]}")
    os.replace(tmp, out)
    return out


def build_all(force: bool = False) -> dict[str, str]:
    """Build the FP64 and the mixed-precision libraries concurrently."""
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(PRECISIONS)) as pool:
        futs = {p: pool.submit(build, force, False, p) for p in PRECISIONS}
        return {p: f.result() for p, f in futs.items()}


if __name__ == "__main__":
    print(build_all(force=True))
