"""Build the CUDA library in-tree: insta_gb300/_lib/libinsta_gb300.so (sm_103a only).

Each translation unit compiles in parallel with nvcc; the objects link into one
shared library exporting the C ABI of include/insta_gb300.h.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT_DIR = HERE / "_lib"
LIB = OUT_DIR / "libinsta_gb300.so"
SOURCES = ["insta_abi.cu", "frame_kernels.cu", "render_kernels.cu", "static_scratch.cu", "train_kernels.cu", "train_mlp.cu", "mlp_slots.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found")
    return cand


def flags(extra=()) -> list:
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC,-O3",
                   "-I", str(CSRC), "-I", str(HERE.parent / "include")] + list(extra)


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False, ptxas_info: bool = False) -> Path:
    OUT_DIR.mkdir(exist_ok=True)
    headers = [p for p in CSRC.iterdir() if p.suffix in (".h", ".cuh")] + [HERE.parent / "include" / "insta_gb300.h"]
    objs = []
    jobs = []
    for src in SOURCES:
        obj = OUT_DIR / (Path(src).stem + ".o")
        objs.append(obj)
        if force or ptxas_info or _stale(obj, [CSRC / src] + headers):
            extra = ["-Xptxas", "-v"] if ptxas_info else []
            jobs.append([nvcc()] + flags(extra) + ["-c", str(CSRC / src), "-o", str(obj)])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or ptxas_info or r.returncode:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode:
                raise RuntimeError(f"nvcc failed: {' '.join(cmd)}")
    if force or _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", str(LIB)] + [str(o) for o in objs] + ["-lcudart", "-lcublas"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
