"""Headless raster + Blinn-Phong shading on the GPU against the oracle's FP32
restatement.  Both rasterise the same way; they differ only in FP32
rounding (the GPU contracts multiply-adds), so a pixel on a triangle edge or
at a texture-filter switch may go either way: at most 0.5% of pixels may
differ by more than 2e-3 (absolute, or relative above 1)."""
import numpy as np
import pytest

import radiancecascade_gb300 as R
from radiancecascade_gb300 import _ffi as F
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _checker(n, c0, c1):
    y, x = np.mgrid[0:n, 0:n]
    img = np.where(((x // 4 + y // 4) % 2)[..., None] == 0, c0, c1).astype(np.uint8)
    return np.concatenate([img, np.full((n, n, 1), 255, np.uint8)], 2)


def _normal_map(n):
    y, x = np.mgrid[0:n, 0:n] / n
    nx, ny = 0.3 * np.sin(6 * x), 0.3 * np.cos(5 * y)
    nz = np.sqrt(1 - nx ** 2 - ny ** 2)
    rgb = ((np.stack([nx, ny, nz], 2) * 0.5 + 0.5) * 255).round().astype(np.uint8)
    return np.concatenate([rgb, np.full((n, n, 1), 255, np.uint8)], 2)


def _scene(g):
    pos, idx, tm, vox_mats = R.room_mesh(g, boxes=4, seed=3)
    uv = np.stack([pos[:, 0] / g + pos[:, 2] / (2 * g), pos[:, 1] / g], 1).astype(np.float32)
    verts = R.shade_vertices(pos, idx, texcoords=uv)
    assert not np.isnan(verts).any()
    mats = [R.shade_material(ambient=(1, 1, 1), diffuse=(0.6, 0.6, 0.6), specular=(0.5, 0.5, 0.5), shininess=32),
            R.shade_material(ambient=(1, 1, 1), diffuse=(0.8, 0.8, 0.8), specular=(0.2, 0.2, 0.2), shininess=8,
                             color_texture=0, normal_texture=1),
            R.shade_material()]  # no material: the predicate path
    tex = [dict(rgba=_checker(16, (200, 40, 40), (30, 160, 220)), srgb=1), dict(rgba=_normal_map(32), srgb=0)]
    return pos, idx, tm, vox_mats, verts, mats, tex


def _view(g, W, H, gi):
    v = F.ShadeView()
    v.view_proj[:] = R.camera_view_proj((g / 2, g / 2, 2.0), np.pi / 2, -0.1, W, H, fovy_deg=70, znear=0.1,
                                        zfar=4.0 * g)
    v.eye[:] = (g / 2, g / 2, 2.0)
    v.light[:] = (g * 0.3, g * 0.8, g * 0.4)
    v.width, v.height = W, H
    v.world_to_grid[:] = [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0]
    v.gi_scale = gi
    return v


def _compare(got, want):
    d = np.abs(got - want) / np.maximum(1.0, np.abs(want))
    bad = (d > 2e-3).any(-1)
    assert bad.mean() <= 5e-3, bad.mean()
    assert (want[..., :3] > 0).any(-1).mean() > 0.5  # most of the image is lit geometry


@pytest.mark.parametrize("gi", [0.0, 1.0])
def test_shading_matches_oracle(gi):
    g, W, H = 32, 160, 120
    pos, idx, tm, vox_mats, verts, mats, tex = _scene(g)
    with R.Engine(R.make_params(g, 4)) as e:
        e.set_mesh(pos, idx, vox_mats, tm)
        e.solve()
        flu = e.fluence()
        view = _view(g, W, H, gi)
        got = e.shade(view, verts, idx, mats, tm, tex)
    keep = [np.ascontiguousarray(t["rgba"]) for t in tex]
    ctex = (F.Texture * 2)()
    for k, t in enumerate(keep):
        ctex[k].rgba, ctex[k].width, ctex[k].height, ctex[k].srgb = t.ctypes.data, t.shape[1], t.shape[0], tex[k]["srgb"]
    cmats = (F.ShadeMaterial * 3)(*mats)
    want = O.shade(view, verts, idx, tm, cmats, ctex, flu, (g // 2,) * 3, 2)
    _compare(got, want)
    if gi > 0:
        base = O.shade(_view(g, W, H, 0.0), verts, idx, tm, cmats, ctex, None)
        assert (want[..., :3] - base[..., :3]).max() > 0  # the fluence term lights the scene


def test_shading_argument_checks():
    with R.Engine(R.make_params(16, 2)) as e:
        v = _view(16, 8, 8, 0.0)
        verts = np.zeros((3, 17), np.float32)
        with pytest.raises(R.RCError):
            e.shade(v, verts, np.array([[0, 1, 5]], np.uint32), [R.shade_material()])
        with pytest.raises(R.RCError):
            e.shade(v, verts, np.array([[0, 1, 2]], np.uint32), [R.shade_material(color_texture=0)])
        img = e.shade(v, verts, np.array([[0, 1, 2]], np.uint32), [R.shade_material()])
        assert np.array_equal(img[..., 3], np.ones((8, 8))) and not img[..., :3].any()


def test_set_mesh_then_draw_matches_one_call_shading():
    """rc_shade_set_mesh + rc_shade_draw give rc_shade's image bit for bit, for
    several views of one upload, into host memory and into a device buffer."""
    torch = pytest.importorskip("torch")
    g, W, H = 32, 96, 72
    pos, idx, tm, vox_mats, verts, mats, tex = _scene(g)
    with R.Engine(R.make_params(g, 4)) as e:
        e.set_mesh(pos, idx, vox_mats, tm)
        e.solve()
        views = [_view(g, W, H, 1.0), _view(g, W, H, 0.0)]
        views[1].eye[:] = (g / 3, g / 2, 3.0)
        views[1].view_proj[:] = R.camera_view_proj((g / 3, g / 2, 3.0), np.pi / 3, 0.0, W, H, fovy_deg=60,
                                                   znear=0.1, zfar=4.0 * g)
        want = [e.shade(v, verts, idx, mats, tm, tex) for v in views]
        with pytest.raises(R.RCError):  # a fresh context has no mesh to draw
            with R.Engine(R.make_params(16, 2)) as e2:
                e2.shade_draw(_view(16, 8, 8, 0.0))
        e.shade_set_mesh(verts, idx, mats, tm, tex)
        for v, w in zip(views, want):
            assert np.array_equal(e.shade_draw(v), w)
            d = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
            e.shade_draw(v, d)
            e.synchronize()
            assert np.array_equal(d.cpu().numpy(), w)
