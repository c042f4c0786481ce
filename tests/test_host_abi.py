"""Host-side checks of the GPU library (no GPU needed): it loads, exports
every entry point of include/cannon_gpu.h, and its Shape/Body constructor
arithmetic matches the oracle's bit for bit."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from cannon_physics_gb300 import _abi as A
from cannon_physics_gb300 import engine, scenes
from cannon_physics_gb300 import serve as S
from oracle import oracle_py as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from cannon_physics_gb300 import build as B
    B.build()
    return engine.lib()


def header_functions():
    src = open(os.path.join(ROOT, "include", "cannon_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w]+\**\s+\**(cp_\w+)\s*\(", src, flags=re.M)))


def test_library_exports_every_header_entry_point(lib):
    names = header_functions()
    assert len(names) >= 18
    for n in names:
        assert hasattr(lib, n), f"libcannon_gpu.so does not export {n}"
    assert lib.cp_abi_version() == 4


def test_ctypes_layouts_match_the_c_header(tmp_path):
    """The Python and Dart bindings mirror the C structs; a C probe compiled
    against the header must agree on every size and field offset."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = [("cp_body_desc", A.BodyDesc), ("cp_body_state", A.BodyState), ("cp_body_shape", A.BodyShape), ("cp_ray", A.Ray), ("cp_ray_hit", A.RayHit), ("cp_shape_desc", A.ShapeDesc), ("cp_world_desc", A.WorldDesc),
               ("cp_contact", A.Contact), ("cp_row", A.Row), ("cp_constraint_desc", A.ConstraintDesc),
               ("cp_contact_material", A.ContactMaterial), ("cp_step_info", A.StepInfo), ("cp_config", A.Config),
               ("cp_serve_config", S.ServeConfig), ("cp_serve_stats", S.ServeStats)]
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "cannon_gpu.h"', "int main(void) {"]
    expect = []
    for cname, py in structs:
        lines.append(f'printf("%zu\\n", sizeof({cname}));')
        expect.append(C.sizeof(py))
        for fname, _ in py._fields_:
            cf = {"lambda_": "lambda", "from_": "from"}.get(fname, fname)
            lines.append(f'printf("%zu\\n", offsetof({cname}, {cf}));')
            expect.append(getattr(py, fname).offset)
    lines.append("return 0; }")
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "probe"
    subprocess.check_call([cc, "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = [int(x) for x in subprocess.check_output([str(exe)]).split()]
    assert got == expect


def _bytes(arr):
    return arr.view(np.uint8).reshape(len(arr), -1)


@pytest.mark.parametrize("make", [scenes.spheres_on_plane, lambda: scenes.box_pile(8, 8, 4),
                                  lambda: scenes.mixed_chains(8, 8, 4, chains=4, chain_len=8),
                                  lambda: scenes.column_world(300, 9, "mixed"), scenes.compound_pile,
                                  scenes.joints_and_hulls])
def test_body_setup_matches_oracle_bitwise(lib, make):
    a, b = make(), make()
    O.setup_scene(a)
    engine.setup_scene(b)
    assert np.array_equal(a.shapes["bounding_sphere_radius"], b.shapes["bounding_sphere_radius"])
    assert np.array_equal(_bytes(a.bodies), _bytes(b.bodies))


def test_invalid_inputs_are_rejected(lib):
    s = A.default_shapes(1)
    s[0]["type"] = A.SHAPE_SPHERE
    s[0]["radius"] = -1.0
    assert lib.cp_shape_setup(s.ctypes.data) == A.CP_ERR_ARG
    assert b"negative" in lib.cp_last_error()
    s[0]["type"] = A.SHAPE_CYLINDER
    s[0]["radius_top"] = 0.5
    s[0]["radius_bottom"] = 0.5
    s[0]["num_segments"] = 40  # hull over the device table limit
    assert lib.cp_shape_setup(s.ctypes.data) == A.CP_ERR_UNSUPPORTED
    b = A.default_bodies(1)
    b[0]["shape"] = 3
    assert lib.cp_body_setup(s.ctypes.data, 1, None, 0, b.ctypes.data, 1) == A.CP_ERR_ARG


def test_compound_bodies_are_checked(lib):
    """Extra shapes must lie inside the table, name existing shapes and
    belong to a body with a first shape; the oracle takes the same view."""
    from oracle import oracle_py as Op
    s = A.default_shapes(2)
    s["type"] = A.SHAPE_SPHERE
    s["radius"] = 0.5
    t = A.body_shapes(2)
    t["shape"] = (1, 0)
    OL = Op.lib()
    cases = [(0, 3, 0), (1, 2, 0), (-1, 1, 0), (0, 1, -1), (0, 2, 5), (0, 65535, 0)]
    for first, count, shape in cases:
        b = A.default_bodies(1)
        b[0]["shape"] = shape
        b[0]["mass"] = 1.0
        b[0]["extra_shapes_first"] = first
        b[0]["extra_shapes_count"] = count
        t2 = t.copy()
        if (first, count, shape) == (0, 2, 5):
            b[0]["shape"] = 0
            t2["shape"][1] = 5
        assert lib.cp_body_setup(s.ctypes.data, 2, t2.ctypes.data, 2, b.ctypes.data, 1) == A.CP_ERR_ARG, (first, count, shape)
        assert OL.orc_body_setup(s.ctypes.data, 2, t2.ctypes.data, 2, b.ctypes.data, 1) == A.CP_ERR_ARG, (first, count, shape)
    b = A.default_bodies(1)
    b[0]["shape"] = 0
    b[0]["mass"] = 1.0
    b[0]["extra_shapes_count"] = 2
    assert lib.cp_body_setup(s.ctypes.data, 2, t.ctypes.data, 2, b.ctypes.data, 1) == A.CP_OK
