"""The checked build (librc_checked.so: the same sources compiled with
RC_CHECKED, every instrumented buffer access tested before it is made) on
small scenes -- 8^3, 16^3, 48^3, a non-cubic 16x32x48 and 64^3, FP32 and
FP16, an incremental emitter update, the batched solve and the learned form:
no access may fail the test, and the results still match the FP64 oracle
(FP32: relative L2 <= 1e-4; FP16 and the learned form: <= 1e-2).  The
checked library runs in a process of its own (RC_LIBRARY)."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_checked_build_finds_no_out_of_range_access():
    sys.path.insert(0, os.path.join(ROOT, "radiancecascade_gb300"))
    import importlib.util
    spec = importlib.util.spec_from_file_location("_rc_build", os.path.join(ROOT, "radiancecascade_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    lib = mod.build(checked=True)
    env = dict(os.environ, RC_LIBRARY=lib, PYTHONPATH=ROOT)
    r = subprocess.run([sys.executable, os.path.join(ROOT, "tests", "checked_run.py")], env=env,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 12, r.stdout
    for x in lines:
        print(x)
        assert x["status"] == 0 and x["failures"] == 0, x
        bound = 1e-4 if x["case"].endswith("fp32") or x["case"] == "batch" else 1e-2
        assert x["rel_l2"] <= bound, x
    assert lines[-1]["finite_query"]
