"""Camera models of the oracle (the per-pixel pinhole32 / equi62_lut1d
unproject and project the path's raygen and reprojection use), against the
cases of the reference's tests/test_camera_models.cpp:112-236. That file
checks the double-precision host models to 1e-12 ... 5e-6; the path runs
them in float (programs.cu:335-497), so the bounds here are float ones:
directions to 1e-6, pixels to 1e-4. The equi LUT comes from
rtgb_make_equi62_lut1d (camera_models.cpp:228-248)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from ray_tracing_gb300 import abi

DIR_TOL = 1e-6
PIX_TOL = 1e-4


@pytest.fixture(scope="module")
def orc():
    from oracle.binding import load
    return load()


def _identity_pose(c: abi.Camera):
    for i in range(3):
        c.rotation[4 * i] = 1.0


def _pinhole(w, h, fx, fy, cx, cy, k=(0.0, 0.0, 0.0), p=(0.0, 0.0)) -> abi.Camera:
    c = abi.Camera()
    c.enabled, c.width, c.height, c.model = 1, w, h, 0
    c.pinhole = abi.Pinhole32(fx, fy, cx, cy, k[0], k[1], k[2], p[0], p[1])
    _identity_pose(c)
    return c


def _equi(w, h, fx, fy, cx, cy, radial, tangential) -> abi.Camera:
    c = abi.Camera()
    c.enabled, c.width, c.height, c.model = 1, w, h, 1
    r = (C.c_double * 6)(*radial)
    t = (C.c_double * 2)(*tangential)
    assert abi.load().rtgb_make_equi62_lut1d(w, h, fx, fy, cx, cy, r, t, C.byref(c.equi)) == 0
    _identity_pose(c)
    return c


def _unit(v):
    v = np.asarray(v, np.float64)
    return v / np.linalg.norm(v)


def _unproject(orc, c, x, y):
    out = (C.c_float * 3)()
    orc.orc_unproject(C.byref(c), x, y, out)
    return _unit(out[:])


def _project(orc, c, d):
    d = _unit(d)
    out = (C.c_float * 2)()
    orc.orc_project(C.byref(c), (C.c_float * 3)(*d), out)
    return np.array(out[:], np.float64)


def test_pinhole_roundtrips(orc):
    mild = _pinhole(320, 240, 300.0, 300.0, 160.0, 120.0, (0.02, -0.01, 0.003), (0.001, -0.0015))
    assert np.array_equal(_unproject(orc, mild, 160.0, 120.0), [0.0, 0.0, 1.0])
    assert np.abs(_project(orc, mild, [0.0, 0.0, 1.0]) - (160.0, 120.0)).max() <= PIX_TOL
    d = [0.23, -0.17, 1.0]
    assert np.abs(_unproject(orc, mild, *_project(orc, mild, d)) - _unit(d)).max() <= DIR_TOL
    assert np.abs(_project(orc, mild, _unproject(orc, mild, 200.0, 80.0)) - (200.0, 80.0)).max() <= PIX_TOL
    # pinhole_hard of the reference test: strong radial and tangential terms
    hard = _pinhole(320, 240, 300.0, 315.0, 158.0, 121.0, (0.8, -0.7, 0.25), (0.03, -0.025))
    d = [1.28, -0.96, 1.0]
    assert np.abs(_unproject(orc, hard, *_project(orc, hard, d)) - _unit(d)).max() <= DIR_TOL


def test_equi_roundtrips_and_lut_edges(orc):
    e = _equi(640, 480, 280.0, 282.0, 320.0, 240.0, (0.02, -0.005, 0.001, -0.0002, 0.00005, -0.00001), (0.0012, -0.0009))
    assert np.abs(_unproject(orc, e, 320.0, 240.0) - (0.0, 0.0, 1.0)).max() <= DIR_TOL
    d = [0.21, 0.08, 1.0]
    assert np.abs(_unproject(orc, e, *_project(orc, e, d)) - _unit(d)).max() <= DIR_TOL
    assert np.abs(_project(orc, e, _unproject(orc, e, 360.0, 180.0)) - (360.0, 180.0)).max() <= PIX_TOL
    # no distortion: theta = r / f exactly
    ident = _equi(640, 480, 280.0, 280.0, 320.0, 240.0, (0.0,) * 6, (0.0, 0.0))
    theta = 0.3
    assert np.abs(_unproject(orc, ident, 320.0 + 280.0 * theta, 240.0) - (np.sin(theta), 0.0, np.cos(theta))).max() <= DIR_TOL
    # beyond the LUT's range the model falls back to the undistorted ray (x, y, 1)
    assert np.abs(_unproject(orc, ident, 320.0 + 280.0 * 5.0, 240.0 - 280.0 * 1.5) - _unit([5.0, -1.5, 1.0])).max() <= DIR_TOL
