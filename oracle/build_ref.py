"""Build oracle/_ref/libinsta_ref.so: the reference's own hot-path headers compiled for the host.

TEST INFRASTRUCTURE ONLY.  Compiles oracle/ref_probe.cpp, which includes the INSTA headers
where they lie (the INSTA tree at $INSTA_REFERENCE, default /root/reference), against the
Eigen subset and tiny-cuda-nn stand-ins in oracle/ref_shim.  Nothing from the reference tree is
copied; the output goes only to oracle/_ref/.  Where the tree is absent (the GPU hosts) this
build is skipped and the committed golden vectors in tests/golden/ carry the pin instead.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
LIB = OUT / "libinsta_ref.so"


def reference_root() -> Path:
    return Path(os.environ.get("INSTA_REFERENCE", "/root/reference"))


def available() -> bool:
    r = reference_root()
    return (r / "instant-ngp" / "include" / "neural-graphics-primitives" / "bvh.cuh").exists() and (r / "include" / "rta" / "affine.cuh").exists()


def build(quiet: bool = False) -> Path:
    if not available():
        raise FileNotFoundError(f"INSTA sources not found under {reference_root()}")
    OUT.mkdir(exist_ok=True)
    src = HERE / "ref_probe.cpp"
    shim = HERE / "ref_shim"
    deps = [src] + list(shim.rglob("*"))
    if LIB.exists() and all(d.stat().st_mtime <= LIB.stat().st_mtime for d in deps if d.is_file()):
        return LIB
    r = reference_root()
    tmp = OUT / f"libinsta_ref.{os.getpid()}.so"
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-w",
           "-I", str(shim), "-I", str(r / "instant-ngp" / "include"), "-I", str(r / "include"),
           str(src), "-o", str(tmp)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode:
        raise RuntimeError("reference host build failed:\n" + res.stderr[-4000:])
    os.replace(tmp, LIB)
    if not quiet:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build()
