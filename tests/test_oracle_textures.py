"""The oracle's TextureView::sample (Core/Texture.cu:15-35) pinned against an
independent numpy restatement and known answers: bilinear weights over texel
centres at uv * (size - 1), the last texel repeated beyond the far edge, and
the reference's extrapolation below 0 (the device's float -> uint32
conversion saturates a negative coordinate to texel 0 while the fraction
stays negative)."""
import numpy as np

import oracle
from craystal_gb300 import scenes
from craystal_gb300.api import MaterialFlags, flatten_scene, texture_texels


def numpy_sample(tex, uv):
    h, w = tex.shape[:2]
    out = np.zeros((len(uv), 4), np.float32)
    for i, (u, v) in enumerate(uv.astype(np.float32)):
        px = np.float32(u) * np.float32(w - 1)
        py = np.float32(v) * np.float32(h - 1)
        fx0, fy0 = np.floor(px), np.floor(py)
        x0 = 0 if not fx0 > 0 else int(fx0)
        y0 = 0 if not fy0 > 0 else int(fy0)
        x1, y1 = min(x0 + 1, w - 1), min(y0 + 1, h - 1)
        fx, fy = np.float32(px - np.float32(x0)), np.float32(py - np.float32(y0))
        t = lambda x, y: tex[min(y, h - 1), min(x, w - 1)]
        c0 = t(x0, y0) * (np.float32(1) - fx) + t(x1, y0) * fx
        c1 = t(x0, y1) * (np.float32(1) - fx) + t(x1, y1) * fx
        out[i] = c0 * (np.float32(1) - fy) + c1 * fy
    return out


def scene_with(tex):
    data, _ = scenes.cornell_box(width=8, height=8)
    data.textureImages = [tex]
    data.materials[0].flags |= int(MaterialFlags.hasDiffuseTexture)
    return oracle.OracleScene(flatten_scene(data))


def test_texture_sample_matches_numpy_restatement():
    rng = np.random.default_rng(3)
    tex = texture_texels(rng.random((9, 13, 3)))
    uv = np.concatenate([rng.uniform(-0.3, 1.3, (400, 2)), [[0, 0], [1, 1], [1, 0], [0, 1], [0.5, 0.5]]])
    got = scene_with(tex).texture_sample(0, uv)
    np.testing.assert_array_equal(got, numpy_sample(tex, uv))


def test_texture_known_answers():
    tex = np.zeros((2, 2, 4), np.float32)
    tex[0, 0, 0], tex[0, 1, 0], tex[1, 0, 0], tex[1, 1, 0] = 1.0, 2.0, 3.0, 4.0
    got = scene_with(tex).texture_sample(0, np.array([[0, 0], [1, 0], [0, 1], [1, 1], [0.5, 0.5], [2.0, 2.0],
                                                      [-0.5, 0.0]], np.float32))[:, 0]
    # corners, the centre average, the far-edge clamp, and 1 + (2 - 1) * -0.5
    np.testing.assert_array_equal(got, [1.0, 2.0, 3.0, 4.0, 2.5, 4.0, 0.5])


def test_texture_channels_fill_with_zero():
    t = texture_texels(np.full((3, 3), 0.25, np.float32))
    assert t.shape == (3, 3, 4) and (t[..., 0] == 0.25).all() and not t[..., 1:].any()
