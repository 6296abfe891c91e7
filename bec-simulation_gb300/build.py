"""Build recipe for libsbec.so (the C-ABI engine) — in-tree, sm_103a only.

Each translation unit is compiled by its own nvcc / g++ process in parallel and
linked into ``bec-simulation_gb300/lib/libsbec.so``.  Used by
``__graft_entry__.build()`` and by the tests; no cmake.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
LIB_DIR = PKG / "lib"
BUILD_DIR = PKG / "_build"
LIB = LIB_DIR / "libsbec.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["sbec_engine_f64.cu", "sbec_engine_f32.cu", "sbec_lines_f64.cu", "sbec_lines_f32_v0.cu",
              "sbec_lines_f32_v1.cu", "sbec_lines_f32_v2.cu", "sbec_lines_f32_v3.cu", "sbec_lines_f32_v4.cu",
              "sbec_lines_f32_v5.cu", "sbec_lines_f32_v6.cu", "sbec_lines_f32_v7.cu", "sbec_rows_f32_v12.cu",
              "sbec_rows_f32_v13.cu", "sbec_rows_f32_v14.cu", "sbec_rows_f32_v15.cu", "sbec_segment_f32.cu",
              "sbec_noalloc.cu", "sbec_peaks.cu", "sbec_itp_steps_f32.cu", "sbec_itp_steps_f64.cu"]
CPP_SOURCES = ["sbec_setup.cpp", "sbec_api.cpp"]


def _cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def _run(cmd: list) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(map(str, cmd)) + "\n" + r.stdout + r.stderr)


def _stale(obj: Path, deps: list) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, ptxas_verbose: bool = False, jobs: int | None = None) -> Path:
    """Compile every translation unit and link ``lib/libsbec.so``; returns its path."""
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    BUILD_DIR.mkdir(exist_ok=True)
    LIB_DIR.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + [INCLUDE / "sbec.h"]
    common = ["-O3", "-std=c++17", "-I", str(INCLUDE), "-I", str(CSRC)]
    jobs_list = []
    objs = []
    for src in CU_SOURCES:
        obj = BUILD_DIR / (src + ".o")
        objs.append(obj)
        if _stale(obj, [CSRC / src] + headers):
            cmd = [nvcc, *ARCH, "-lineinfo", *common, "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
                   "-c", str(CSRC / src), "-o", str(obj)]
            if ptxas_verbose:
                cmd += ["-Xptxas", "-v"]
            jobs_list.append(cmd)
    for src in CPP_SOURCES:
        obj = BUILD_DIR / (src + ".o")
        objs.append(obj)
        if _stale(obj, [CSRC / src] + headers):
            jobs_list.append(["g++", *common, "-fPIC", "-I", str(cuda / "include"), "-c", str(CSRC / src),
                              "-o", str(obj)])
    if jobs_list:
        with ThreadPoolExecutor(max_workers=jobs or max(1, min(len(jobs_list), os.cpu_count() or 1))) as ex:
            for cmd in jobs_list:
                if verbose:
                    print(" ".join(cmd), file=sys.stderr)
            list(ex.map(_run, jobs_list))
    if _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-Xcompiler", "-fPIC",
              "-L", str(cuda / "lib64"), "-lcudart"])
    return LIB


if __name__ == "__main__":
    p = build(verbose=True, ptxas_verbose="-v" in sys.argv)
    print(p)
