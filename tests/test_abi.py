"""The C ABI library: it builds, loads without a GPU, exports every function that
include/rocketsim_gb300.h declares, and its ctypes mirrors match the C layouts."""
import ctypes as C
import os
import re
import shutil
import subprocess
import tempfile

import pytest

from rocketsim_gb300 import abi
from rocketsim_gb300.build import build

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "rocketsim_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(rsg_[a-z0-9_]+)\s*\(", text)
    return sorted(set(n for n in names if not n.endswith("_fn")))


def test_library_builds_and_exports_every_declared_function():
    path = build()
    assert os.path.exists(path)
    lib = C.CDLL(path)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"
    assert set(declared_functions()) == set(abi.PROTOTYPES), "ctypes prototypes differ from the header"


def test_struct_layouts_match_header():
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    structs = {"rsg_car_state": abi.CarState, "rsg_ball_state": abi.BallState, "rsg_pad_state": abi.PadState,
               "rsg_car_controls": abi.CarControls, "rsg_car_config": abi.CarConfig,
               "rsg_ball_hit_info": abi.BallHitInfo, "rsg_rotmat": abi.RotMat,
               "rsg_heatseeker_info": abi.HeatseekerInfo}
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', 'int main(void) {']
    for cname, ct in structs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in ct._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0; }")
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "l.c"), os.path.join(d, "l")
        open(src, "w").write("\n".join(lines))
        subprocess.run([gcc, "-std=c99", src, "-o", exe], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {}
    for ln in out:
        if ln:
            a, b, v = ln.split()
            got[(a, b)] = int(v)
    for cname, ct in structs.items():
        assert got[(cname, "size")] == C.sizeof(ct), cname
        for fname, _ in ct._fields_:
            assert got[(cname, fname)] == getattr(ct, fname).offset, f"{cname}.{fname}"


def test_preset_configs_without_gpu():
    import rocketsim_gb300 as rsg
    c = rsg.car_config(rsg.CAR_OCTANE)
    assert abs(c.hitbox_size.x - 120.507) < 1e-4 and c.dodge_deadzone == 0.5
    with pytest.raises(abi.RSGError):
        rsg.car_config(9)
