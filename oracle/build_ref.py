"""Build oracle/_ref/libinsta_ref.so: the reference's own hot-path headers compiled for the host.

TEST INFRASTRUCTURE ONLY.  Compiles oracle/ref_probe.cpp, which includes the INSTA headers
where they lie (the INSTA tree at $INSTA_REFERENCE, default /root/reference), against the
Eigen subset and tiny-cuda-nn stand-ins in oracle/ref_shim.  Nothing from the reference tree is
copied; the output goes only to oracle/_ref/.  Where the tree is absent (the GPU hosts) this
build is skipped and the committed golden vectors in tests/golden/ carry the pin instead.
"""
from __future__ import annotations

import os
import re
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


# The march helpers of instant-ngp/src/testbed_nerf.cu (inline __host__ __device__ or small
# __device__ functions inside a .cu file that cannot be compiled whole): their text is taken from
# the reference file at build time, in file order, into oracle/_ref/march_helpers.inc, which
# oracle/ref_march_probe.cpp includes.  Nothing is copied into the repository.
MARCH_FILE = ("instant-ngp", "src", "testbed_nerf.cu")
MARCH_FUNCS = ["NERF_RENDERING_NEAR_DISTANCE", "NERF_STEPS", "NERF_CASCADES", "SQRT3", "STEPSIZE", "MIN_CONE_STEPSIZE",
               "MAX_CONE_STEPSIZE", "grid_mip_offset", "calc_cone_angle", "calc_dt", "distance_to_next_voxel",
               "advance_to_next_voxel", "warp_dt", "unwarp_dt", "cascaded_grid_idx_at", "density_grid_occupied_at",
               "mip_from_pos", "mip_from_dt"]


def extract_functions(text: str, names) -> str:
    """The source text of each named top-level function definition (signature line to its
    matching closing brace), in file order."""
    lines = text.splitlines()
    found = []
    for name in names:
        pat = re.compile(r"^(inline|__device__|__host__|static|constexpr|\s)*[\w:<>&* ]*\b" + re.escape(name) + r"\s*\(")
        start = next((i for i, ln in enumerate(lines) if pat.match(ln) and not ln.rstrip().endswith(";")), None)
        if start is None:
            raise RuntimeError(f"{name} not found in the reference march source")
        depth, end, opened = 0, start, False
        for j in range(start, len(lines)):
            for ch in lines[j]:
                if ch == "{":
                    depth += 1
                    opened = True
                elif ch == "}":
                    depth -= 1
            if opened and depth == 0:
                end = j
                break
        found.append((start, "\n".join(lines[start:end + 1])))
    found.sort()
    return "\n\n".join(t for _, t in found) + "\n"


def build(quiet: bool = False) -> Path:
    if not available():
        raise FileNotFoundError(f"INSTA sources not found under {reference_root()}")
    OUT.mkdir(exist_ok=True)
    src = HERE / "ref_probe.cpp"
    src_march = HERE / "ref_march_probe.cpp"
    shim = HERE / "ref_shim"
    deps = [src, src_march, Path(__file__)] + list(shim.rglob("*"))
    if LIB.exists() and all(d.stat().st_mtime <= LIB.stat().st_mtime for d in deps if d.is_file()):
        return LIB
    r = reference_root()
    inc = OUT / "march_helpers.inc"
    inc.write_text(extract_functions(r.joinpath(*MARCH_FILE).read_text(), MARCH_FUNCS))
    tmp = OUT / f"libinsta_ref.{os.getpid()}.so"
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-w",
           "-I", str(shim), "-I", str(r / "instant-ngp" / "include"), "-I", str(r / "include"), "-I", str(OUT),
           str(src), str(src_march), "-o", str(tmp)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode:
        raise RuntimeError("reference host build failed:\n" + res.stderr[-4000:])
    os.replace(tmp, LIB)
    if not quiet:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build()
