"""Pins the CPU oracle against the known answers the reference's own tests hold
for this path: Tests/CameraTest.cpp:10-51 (camera ray directions) and
Tests/CoreTest.cpp:130-280 (sampler range, seeding and statistics).  Each
case keeps the reference test's inputs and tolerances."""
import numpy as np
import pytest

import oracle


def default_camera(w=512, h=512):
    # CameraProxy defaults, Core/CameraProxy.h:12-23
    return oracle.make_camera((0, 0, 0), (0, 0, -1), (0, 1, 0), 60.0, w, h)


@pytest.mark.parametrize("pos,expect,tol", [
    ((256, 256), (0.0, 0.0, -1.0), 1e-5),                             # CameraTest.cpp:16-24
    ((0, 0), (-0.44721359, 0.44721359, -0.774596691), 1e-4),           # :26-37
    ((511, 511), (0.446162969, -0.446162969, -0.77580744), 1e-4),     # :39-50
])
def test_camera_known_answers(pos, expect, tol):
    r = oracle.camera_rays(default_camera(), [pos])[0]
    assert tuple(r["o"]) == (0.0, 0.0, 0.0)
    np.testing.assert_allclose(r["d"], expect, atol=tol, rtol=0)
    assert r["tmin"] == 0.0 and np.isinf(r["tmax"])


def test_sampler_range():  # CoreTest.cpp:130-153
    d = oracle.sampler_draws(123, 456, 0, 3000)
    assert (d >= 0.0).all() and (d < 1.0).all()


def test_sampler_pixel_and_index_seeds():  # CoreTest.cpp:155-170, 219-243
    a = oracle.sampler_draws(0, 0, 0, 100)
    b = oracle.sampler_draws(0, 1, 0, 100)
    assert (a != b).any()
    c = oracle.sampler_draws(123, 456, 0, 100)
    assert np.array_equal(c, oracle.sampler_draws(123, 456, 0, 100))
    assert (c != oracle.sampler_draws(123, 456, 1, 100)).any()


def test_sampler_histogram():  # CoreTest.cpp:172-195
    d = oracle.sampler_draws(123, 456, 0, 10000)
    bins = np.bincount(np.minimum((d * 10).astype(int), 9), minlength=10)
    assert ((bins > 800) & (bins < 1200)).all()


def test_sampler_quadrants():  # CoreTest.cpp:197-216
    d = oracle.sampler_draws(123, 456, 0, 2000).reshape(-1, 2)
    q = set(zip(d[:, 0] >= 0.5, d[:, 1] >= 0.5))
    assert len(q) == 4


def test_sampler_moments():  # CoreTest.cpp:245-280
    d = oracle.sampler_draws(123, 456, 0, 10000).astype(np.float64)
    assert abs(d.mean() - 0.5) < 0.05
    assert abs(d.var(ddof=1) - 1.0 / 12.0) < 0.01


def test_sampler_state_recurrence():
    """Core/Sampler.cu:4-31 restated in numpy uint32 arithmetic."""
    def seq(px, py, si, n):
        m = np.uint32
        with np.errstate(over="ignore"):
            s = m(px) * m(2654435761) + m(py) * m(1597334677) + m(si)
            inc = m(px) * m(1234567891) + m(py) * m(987654321) + m(1)

            def step(s):
                old = s
                s = old * m(747796405) + inc
                old = ((old >> ((old >> m(28)) + m(4))) ^ old) * m(277803737)
                return s, (old >> m(22)) ^ old

            for _ in range(4):
                s, _ = step(s)
            out = []
            for _ in range(n):
                s, v = step(s)
                out.append(v)
        return np.array(out, np.uint32)

    for px, py, si in [(0, 0, 0), (123, 456, 7), (65535, 3, 1 << 20)]:
        assert np.array_equal(oracle.sampler_raw(px, py, si, 64), seq(px, py, si, 64))
        raw = seq(px, py, si, 64)
        np.testing.assert_array_equal(oracle.sampler_draws(px, py, si, 64),
                                      raw.astype(np.float32) * np.float32(1.0 / 4294967296.0))
