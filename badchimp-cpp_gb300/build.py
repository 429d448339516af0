"""Builds libbclbm.so in-tree with nvcc for sm_103a (GB300).

Translation units are compiled in parallel:
  csrc/bclbm_exact.cu    FP64 kernels in the reference's expression order,
                         compiled with -fmad=false (no FMA contraction)
  csrc/bclbm_kernels.cu  FP64 (FMA) and FP32-compute kernels, the staged
                         (TMA table-tile) single-phase kernels, reductions
  csrc/bclbm_api.cu      the C ABI of include/bclbm.h (host code)
  csrc/bclbm_static.cu   bclbm_moments_static, the entry point that allocates nothing
  csrc/bclbm_batch.cu    the multi-instance batch (persistent kernel, CUDA graph)
  csrc/bclbm_geometry.cu the host-side lattice builder (voxel mask to node tables)
  csrc/bclbm_vtklb.cu    the .vtklb geometry-file reader (host)
  csrc/bclbm_vtu.cu      the VTU/PVTU writer of the output step (host)
  csrc/bclbm_links.cu    the std_one_phase step: tag resolution, FMA kernel instances
Host code is compiled with -ffp-contract=off so that host-side arithmetic is
the same on x86-64 and aarch64.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
CSRC = HERE / "csrc"
BUILD = CSRC / "_build"
OUT = HERE / "libbclbm.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

UNITS = {
    "bclbm_exact.cu": ["-fmad=false"],
    "bclbm_kernels.cu": [],
    "bclbm_api.cu": [],
    "bclbm_static.cu": [],
    "bclbm_batch.cu": [],
    "bclbm_geometry.cu": [],
    "bclbm_vtklb.cu": [],
    "bclbm_vtu.cu": [],
    "bclbm_links.cu": [],
}


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found")
    return exe


def common_flags():
    return ARCH + ["-lineinfo", "-O3", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
                   "-Xcompiler", "-ffp-contract=off", f"-I{REPO / 'include'}", f"-I{CSRC}"]


def _stale() -> bool:
    if not OUT.exists():
        return True
    t = OUT.stat().st_mtime
    deps = list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + \
        list((REPO / "include").glob("*.h")) + [Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose: bool = False, extra_flags=None) -> Path:
    if not force and not _stale():
        return OUT
    BUILD.mkdir(parents=True, exist_ok=True)
    procs = []
    objs = []
    for src, flags in UNITS.items():
        obj = BUILD / (Path(src).stem + ".o")
        cmd = [nvcc(), "-c", str(CSRC / src), "-o", str(obj)] + common_flags() + flags + list(extra_flags or [])
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
        objs.append(str(obj))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append(f"{src}:\n{out}")
        elif verbose and out.strip():
            print(out, file=sys.stderr)
    if failed:
        raise RuntimeError("nvcc failed\n" + "\n".join(failed))
    tmp = OUT.with_suffix(".so.tmp")
    cmd = [nvcc(), "-shared", "-o", str(tmp)] + objs + ARCH + ["-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed\n" + res.stdout + res.stderr)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(OUT)
