"""The C-ABI library loads, exports every function include/gb2d.h declares,
and its record layouts match the numpy/ctypes mirrors (no GPU needed)."""
import ctypes
import os
import re

import numpy as np
import pytest

from pypybox2d_gb300 import abi

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(REPO, "include", "gb2d.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gb_[a-z_0-9]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from pypybox2d_gb300 import build
    build.build()
    return abi.load_library()


def test_library_exports_every_declared_function(lib):
    names = declared_functions()
    assert "gb_batch_step" in names and len(names) >= 10
    for n in names:
        assert hasattr(lib, n), f"libgb2d.so does not export {n}"
    assert set(names) <= set(abi.EXPORTED) | {"gb_version", "gb_last_error"}


def test_record_layouts_match(lib):
    sizes = (ctypes.c_int32 * 6)()
    assert lib.gb_struct_sizes(sizes) == 0
    assert sizes[0] == abi.BODY.itemsize
    assert sizes[1] == abi.FIXTURE.itemsize
    assert sizes[2] == abi.CONTACT.itemsize
    assert sizes[3] == abi.WORLD.itemsize
    assert sizes[4] == ctypes.sizeof(abi.Scene)
    assert sizes[5] == ctypes.sizeof(abi.StepOpts)
    assert lib.gb_joint_size() == abi.JOINT.itemsize
    assert lib.gb_controller_size() == abi.CONTROLLER.itemsize
    assert lib.gb_body_state_size() == abi.BODY_STATE.itemsize == 152


def test_errors_are_reported_not_silent(lib):
    h = ctypes.c_void_p()
    assert lib.gb_batch_create(None, 0, ctypes.byref(h)) == -1
    assert b"NULL" in lib.gb_last_error()
    assert lib.gb_batch_step(None, None, None) == -1


def test_bad_scene_is_rejected_before_any_device_call(lib):
    from pypybox2d_gb300 import scenes
    W, B, F, M = scenes.pyramid_world(rows=2)
    W = W.copy()
    W["body_count"] = len(B) + 5     # range outside the body array
    s, keep = abi.make_scene(W, B, F, None, M)
    h = ctypes.c_void_p()
    assert lib.gb_batch_create(ctypes.byref(s), 0, ctypes.byref(h)) == -1
    assert b"outside" in lib.gb_last_error()


def test_launch_config_layout():
    text = open(os.path.join(REPO, "include", "gb2d.h")).read()
    m = re.search(r"#define GB_LAUNCH_CONFIG_BYTES (\d+)", text)
    assert m and int(m.group(1)) == ctypes.sizeof(abi.LaunchConfig) == abi.LAUNCH_CONFIG_BYTES
