"""GPU test of rc_solve_noalloc, the entry point that allocates no memory.

Some callers cannot call cudaMalloc (a renderer that fixes its device-memory
budget at start-up, a plugin host that owns every allocation).  They pass
device buffers for the scene and the results, and the library works inside
its own statically sized device array.  This test drives that entry point
through the C ABI and checks it against the ordinary context path
(rc_create / rc_scene_upload / rc_solve) on two calls in a row, with the same
tolerance as the other FP32 parity tests, and the fluence directly against
the FP64 oracle.  A third call runs with host-side allocation failures
injected (RC_FAULT=alloc makes every allocation inside the library fail) and
must still succeed, since the entry point allocates nothing.  The file is
collected last on purpose; it also passes on its own in a fresh process.
"""
import ctypes as C
import os

import numpy as np
import pytest

import radiancecascade_gb300 as R
from oracle import oracle as O
from radiancecascade_gb300 import _ffi as F
from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu
FP32_REL_L2 = 1e-4
FP32_MAX_REL = 1e-5
FP16_VS_FP64 = 1e-2


def _context_path(params, vox):
    with R.Engine(params) as e:
        e.upload(vox)
        e.solve()
        e.synchronize()
        return e.fluence().copy(), [e.radiance(i).copy() for i in range(params.num_cascades)]


def _split_levels(params, flat):
    out, off = [], 0
    for i in range(params.num_cascades):
        info = R.level_info(params, i)
        n = info.radiance_elems
        px, py, pz = info.probes
        out.append(flat[off:off + n].reshape(3, info.num_dirs, pz, py, px))
        off += n
    return out


@pytest.mark.parametrize("precision", ["fp32", "fp16"])
def test_noalloc_matches_context_path_on_two_calls_in_a_row(precision):
    torch = pytest.importorskip("torch")
    params = R.make_params(64, 5, precision=precision)
    n_flu = 3 * int(np.prod(R.level_info(params, 0).probes))
    rad_bytes = sum(R.level_info(params, i).radiance_bytes for i in range(params.num_cascades))
    elem = np.float16 if precision == "fp16" else np.float32
    d_flu = torch.empty(n_flu, dtype=torch.float32, device="cuda")
    d_rad = torch.empty(rad_bytes, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    results = []
    for frame in (0, 7, 11):
        boxes, spheres = R.workload_scene("c64", frame=frame)
        vox = R.voxelise_host(64, boxes, spheres)
        d_vox = torch.from_numpy(vox.view(np.uint16).reshape(-1, 4).copy()).cuda()
        d_flu.fill_(float("nan"))
        inject = frame == 11  # the library's allocations fail; this call makes none
        if inject:
            os.environ["RC_FAULT"] = "alloc"
        try:
            st = F.lib().rc_solve_noalloc(C.byref(params), C.c_void_p(d_vox.data_ptr()),
                                          C.c_void_p(d_flu.data_ptr()), C.c_void_p(d_rad.data_ptr()),
                                          C.c_void_p(stream.cuda_stream))
        finally:
            if inject:
                del os.environ["RC_FAULT"]
        assert st == F.RC_OK, F.last_error()
        torch.cuda.synchronize()
        flu = d_flu.cpu().numpy().reshape(-1, 3).astype(np.float64)
        levels = _split_levels(params, d_rad.cpu().numpy().view(elem))
        ref64, _ = O.solve(O.params(64, 5), vox)
        assert rel_l2(flu, ref64) <= (FP16_VS_FP64 if precision == "fp16" else FP32_REL_L2)
        ref_flu, ref_levels = _context_path(params, vox)
        assert rel_l2(flu, ref_flu) <= FP32_REL_L2
        assert np.abs(flu - ref_flu).max() <= FP32_MAX_REL * max(1.0, np.abs(ref_flu).max())
        for g, r in zip(levels, ref_levels):
            g = g.astype(np.float64)
            r = r.astype(np.float64)
            assert rel_l2(g, r) <= FP32_REL_L2
            assert np.abs(g - r).max() <= FP32_MAX_REL * max(1.0, np.abs(r).max())
        results.append(flu)
    assert not np.array_equal(results[0], results[1])  # the second call really recomputed
    assert not np.array_equal(results[1], results[2])


def test_noalloc_rejects_oversize_and_null_buffers():
    params = R.make_params(256, 6)
    dummy = C.c_void_p(16)  # never dereferenced: both calls fail before any GPU work
    st = F.lib().rc_solve_noalloc(C.byref(params), dummy, dummy, dummy, None)
    assert st == F.RC_ERR_UNSUPPORTED
    assert "static maximum" in F.last_error()
    small = R.make_params(32, 4)
    st = F.lib().rc_solve_noalloc(C.byref(small), None, dummy, dummy, None)
    assert st == F.RC_ERR_INVALID_ARG
    st = F.lib().rc_solve_noalloc(C.byref(small), dummy, C.c_void_p(24), dummy, None)
    assert st == F.RC_ERR_INVALID_ARG
    assert "16-byte aligned" in F.last_error()
