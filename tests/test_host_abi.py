"""CPU tests of the product's host side and its C ABI (no GPU needed).

Checks that librc.so loads and exports every function include/rc.h declares,
that its host-only helpers agree with the oracle, and that GPU entry points
fail with a status (never abort) when no device is present.
"""
import ctypes as C
import math
import os
import re

import numpy as np
import pytest

import radiancecascade_gb300 as R
from radiancecascade_gb300 import _ffi as F
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header_functions():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            src = open(os.path.join(ROOT, "include", h)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(rc_[a-z0-9_]+)\s*\(", src))
    return names


def test_library_exports_every_declared_symbol():
    names = _header_functions()
    assert len(names) >= 20
    lib = C.CDLL(F.LIB_PATH)
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    # every declared function is also bound by the Python layer
    assert names <= set(F.SIGNATURES), sorted(names - set(F.SIGNATURES))


def test_abi_version_and_status_strings():
    assert F.lib().rc_abi_version() == 1
    assert F.status_name(F.RC_ERR_TIMEOUT) == "RC_ERR_TIMEOUT"


def test_params_validation():
    p = R.make_params(64, 5)
    assert tuple(p.grid) == (64, 64, 64)
    with pytest.raises(R.RCError) as e:
        R.make_params(60, 5)  # not a multiple of the top spacing (32)
    assert e.value.status == F.RC_ERR_INVALID_ARG
    with pytest.raises(R.RCError):
        R.make_params(64, 5, dir_res0=3)
    bad = R.make_params(64, 5)
    bad.reserved[0] = 1
    assert F.lib().rc_params_validate(C.byref(bad)) == F.RC_ERR_INVALID_ARG
    assert "reserved" in F.last_error()


def test_level_shapes():
    p = R.make_params(256, 6)
    infos = [R.level_info(p, i) for i in range(6)]
    assert [i.probes[0] for i in infos] == [128, 64, 32, 16, 8, 4]
    assert [i.num_dirs for i in infos] == [16, 64, 256, 1024, 4096, 16384]
    assert [(i.interval_lo, i.interval_hi) for i in infos] == [(0, 1), (1, 5), (5, 21), (21, 85), (85, 341),
                                                                (341, 1365)]
    rays = sum(i.num_dirs * i.probes[0] ** 3 for i in infos)
    assert rays == 66060288
    assert F.lib().rc_fluence_elems(C.byref(p)) == 3 * 128 ** 3


@pytest.mark.parametrize("n", [2, 4, 8, 16, 32])
def test_directions_and_solid_angles_match_oracle(n):
    assert np.array_equal(R.directions(n), O.directions(n))
    assert np.abs(np.abs(R.directions(n)).sum(1) - n).max() == 0
    om = R.solid_angles(n)
    assert abs(om.sum() - 4 * math.pi) < 1e-12
    assert np.abs(om - O.solid_angles(n)).max() < 1e-13


@pytest.mark.parametrize("name,frames", [("c64", 0), ("c64", 17), ("c256", 0), ("c256", 239)])
def test_generator_motion_and_voxeliser_match_oracle(name, frames):
    b, s = R.workload_scene(name, frame=frames)
    ob, os_ = O.config_scene(name, frame=frames)
    assert b.tobytes() == ob.tobytes()
    assert s.tobytes() == os_.tobytes()
    if name == "c64":
        v = R.voxelise_host(64, b, s)
        assert v.tobytes() == O.voxelise(64, ob, os_).tobytes()


def test_half_rounding_matches_oracle():
    # emission draws pass through the library's float->binary16 rounding
    spec = R.scene_spec(64, 0, (4, 20), 500, (2.0, 5.0), (0.0001, 60000.0))
    _, s = R.generate_scene(spec, 99)
    ospec = O.scene_spec(64, 0, 4, 20, 500, 2.0, 5.0, 0.0001, 60000.0)
    _, os_ = O.generate(ospec, 99)
    assert s.tobytes() == os_.tobytes()
    vals = np.array([0.0, 1e-8, 5.96e-8, 2.98e-8, 6.1e-5, 1.0, 1.0009765625, 65504.0, 65519.0, 65520.0, 3.14159],
                    np.float32)
    for v in vals:
        assert O.float_to_half(float(v)) == int(np.float16(v).view(np.uint16))


def test_gpu_entry_points_fail_cleanly_without_a_device():
    if os.environ.get("CUDA_VISIBLE_DEVICES") is None and _has_gpu():
        pytest.skip("a GPU is visible; covered by the gpu tests")
    p = R.make_params(32, 4)
    h = C.c_void_p()
    st = F.lib().rc_create(C.byref(p), 0, C.byref(h))
    assert st == F.RC_ERR_CUDA
    assert h.value is None
    assert "device" in F.last_error().lower()
    assert F.lib().rc_destroy(None) == F.RC_OK
    assert F.lib().rc_solve(None, None) == F.RC_ERR_INVALID_ARG


def test_batch_entry_points_check_arguments_before_the_device():
    p = (F.Params * 1)(R.make_params(32, 3))
    h = C.c_void_p()
    assert F.lib().rc_batch_create(p, 0, 0, C.byref(h)) == F.RC_ERR_INVALID_ARG
    assert F.lib().rc_batch_create(p, 1, 0, None) == F.RC_ERR_INVALID_ARG
    bad = (F.Params * 1)(R.make_params(32, 3))
    bad[0].num_cascades = 0
    assert F.lib().rc_batch_create(bad, 1, 0, C.byref(h)) == F.RC_ERR_INVALID_ARG
    assert "scene 0" in F.last_error()
    assert F.lib().rc_batch_destroy(None) == F.RC_OK
    assert F.lib().rc_batch_solve(None, None) == F.RC_ERR_INVALID_ARG
    assert F.lib().rc_batch_synchronize(None) == F.RC_ERR_INVALID_ARG
    assert F.lib().rc_batch_set_tiles(None, None) == F.RC_ERR_INVALID_ARG


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_nrc_defaults_and_argument_checks():
    p = F.NrcParams()
    assert F.lib().rc_nrc_params_default(C.byref(p)) == F.RC_OK
    assert (p.first_level, p.hash_log2_entries, p.base_resolution, p.max_resolution) == (2, 19, 16, 512)
    assert abs(p.learning_rate - 1e-2) < 1e-9 and p.train_fraction_log2 == 4 and p.fallback_tile == 8
    assert F.lib().rc_nrc_param_count() == 4 * (64 * 64 + 64) + 16 * 64 + 16
    assert F.lib().rc_nrc_enable(None, C.byref(p)) == F.RC_ERR_INVALID_ARG
    assert F.lib().rc_nrc_disable(None) == F.RC_ERR_INVALID_ARG
    assert F.lib().rc_nrc_params_default(None) == F.RC_ERR_INVALID_ARG



def test_cpp_driver_host_calls(tmp_path):
    """The C ABI driven from C++ (as a native renderer would), host-only calls."""
    import subprocess
    from tests.helpers import build_abi_driver
    exe = build_abi_driver(tmp_path)
    r = subprocess.run([exe, "host"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "host ok" in r.stdout


def test_rc_log_prints_errors_to_stderr():
    """RC_LOG=1 prints every error as it is set; unset, the library is silent."""
    import subprocess
    import sys
    code = ("import ctypes as C, radiancecascade_gb300 as R\n"
            "from radiancecascade_gb300 import _ffi as F\n"
            "p = R.make_params(64, 5); p.num_cascades = 0\n"
            "assert F.lib().rc_params_validate(C.byref(p)) == F.RC_ERR_INVALID_ARG\n")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, RC_LOG="1", PYTHONPATH=root)
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, cwd=root)
    assert r.returncode == 0, r.stderr
    assert "rc[error]" in r.stderr and "num_cascades" in r.stderr
    env.pop("RC_LOG")
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, cwd=root)
    assert r.returncode == 0 and "rc[error]" not in r.stderr


def test_ordinary_library_has_no_checked_words():
    """rc_check_status answers RC_ERR_UNSUPPORTED in the ordinary library (the
    checked one is librc_checked.so); it needs no GPU to say so."""
    first, count = C.c_uint64(7), C.c_uint32(7)
    assert F.lib().rc_check_status(0, C.byref(first), C.byref(count)) == F.RC_ERR_UNSUPPORTED
    assert first.value == 0 and count.value == 0
    assert "RC_CHECKED" in F.last_error()
