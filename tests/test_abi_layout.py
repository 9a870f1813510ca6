"""The ctypes mirrors in insta_gb300/abi.py against the C structs of include/insta_gb300.h: a small
C program (gcc, no GPU) prints sizeof and every field's offsetof, which must equal the ctypes
layout, so a binding never passes a shifted field through the C ABI."""
import ctypes as C
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

STRUCTS = {
    "insta_field_desc": "FieldDesc",
    "insta_render_desc": "RenderDesc",
    "insta_stats": "Stats",
    "insta_pcg32": "Pcg32State",
    "insta_density_update_desc": "DensityUpdateDesc",
    "insta_adam_config": "AdamConfig",
    "insta_train_loss_desc": "TrainLossDesc",
    "insta_server_config": "ServerConfig",
    "insta_tuning": "Tuning",
    "insta_training_pixels_desc": "TrainingPixelsDesc",
}


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    from insta_gb300 import abi
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "insta_gb300.h"', "int main(void) {"]
    for cname, pyname in STRUCTS.items():
        lines.append(f'    printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for fname, *_ in getattr(abi, pyname)._fields_:
            lines.append(f'    printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["    return 0;", "}"]
    d = tmp_path_factory.mktemp("abi_layout")
    src, exe = d / "layout.c", d / "layout"
    src.write_text("\n".join(lines) + "\n")
    subprocess.run(["gcc", "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    table = {}
    for line in out.splitlines():
        cname, field, value = line.split()
        table[(cname, field)] = int(value)
    return table


@pytest.mark.parametrize("cname", sorted(STRUCTS))
def test_ctypes_mirror_matches_header(c_layout, cname):
    from insta_gb300 import abi
    cls = getattr(abi, STRUCTS[cname])
    assert C.sizeof(cls) == c_layout[(cname, "sizeof")], cname
    for fname, *_ in cls._fields_:
        assert getattr(cls, fname).offset == c_layout[(cname, fname)], (cname, fname)
