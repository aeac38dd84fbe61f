"""Host-side parts of the boundary, no GPU: the camera controls of
Core/camera.h:36-78 (MoveRight / MoveUp / Pitch / Yaw / Roll, GLM quaternion
semantics) and the PPM / PFM writers that replace the GL display."""
import math

import numpy as np
import pytest


def _rodrigues(v, axis, deg):
    v = np.asarray(v, np.float64)
    k = np.asarray(axis, np.float64)
    k = k / np.linalg.norm(k)
    a = math.radians(deg)
    return v * math.cos(a) + np.cross(k, v) * math.sin(a) + k * np.dot(k, v) * (1 - math.cos(a))


def _rotate(venu, fwd, axis, deg):
    from venusaur_gb300._lib import ptr

    f = np.ascontiguousarray(fwd, np.float32)
    a = np.ascontiguousarray(axis, np.float32)
    out = np.zeros(3, np.float32)
    venu.lib().venu_camera_rotate(ptr(f), ptr(a), float(deg), ptr(out))
    return out


@pytest.mark.parametrize("deg", [0.0, 1.0, -2.5, 30.0, 90.0, 179.0, -360.0])
def test_rotate_matches_axis_angle(venu, deg):
    """forward * rotate(identity, radians(d), axis) rotates by -d about axis
    (vec3 * quat applies the inverse rotation), then normalises."""
    rng = np.random.default_rng(int(abs(deg) * 10) + 1)
    for _ in range(20):
        fwd = rng.normal(size=3)
        fwd /= np.linalg.norm(fwd)
        axis = rng.normal(size=3) * rng.uniform(0.1, 30.0)  # not unit: normalised inside
        got = _rotate(venu, fwd.astype(np.float32), axis, deg)
        want = _rodrigues(fwd.astype(np.float32), axis.astype(np.float32), -deg)
        want /= np.linalg.norm(want)
        assert np.abs(got - want).max() < 2e-6
        assert abs(float(np.linalg.norm(got.astype(np.float64))) - 1.0) < 1e-6


def test_rotate_unit_axis_not_renormalised(venu):
    """GLM rotate() leaves an axis within 0.001 of unit length as it is."""
    fwd = np.array([0.0, 0.0, -1.0], np.float32)
    axis = np.array([0.0, 1.0005, 0.0], np.float32)
    got = _rotate(venu, fwd, axis, 90.0)
    # unnormalised axis: the quaternion is not unit; inverse() divides by
    # dot(q, q), so the direction is still a rotation about y, then normalised
    want = _rodrigues(fwd, (0, 1, 0), -90.0)
    assert np.abs(got - want).max() < 1e-3


def test_camera_controls(venu):
    cam = venu.Camera((13.0, 2.0, 3.0), 20.0, 16 / 9, 0.1, 10.0)
    cam.SetForward((-13.0, -2.0, -3.0))
    assert cam.Changed() and not cam.Changed()
    U, V, W = cam.UVWFrame()
    f0 = cam.m_forward.copy()
    cam.Pitch(10.0)
    assert cam.Changed()
    assert abs(float(np.dot(cam.m_forward, U / np.linalg.norm(U)))) < 1e-6  # rotation about u keeps f . u = 0
    cam.Pitch(-10.0)
    assert np.abs(cam.m_forward - f0).max() < 1e-6
    cam.Yaw(15.0)
    cam.Yaw(-15.0)
    cam.Roll(5.0)  # about w, parallel to forward: forward unchanged
    assert np.abs(cam.m_forward - f0).max() < 1e-6
    p0 = cam.GetPosition()
    cam.MoveRight(2.0)
    assert np.allclose(cam.GetPosition() - p0, 2.0 * U / np.linalg.norm(U), atol=1e-5)
    p1 = cam.GetPosition()
    cam.MoveUp(-1.0)
    assert np.allclose(cam.GetPosition() - p1, -V / np.linalg.norm(V), atol=1e-5)
    p2 = cam.GetPosition()
    cam.MoveForward(0.5)
    assert np.allclose(cam.GetPosition() - p2, 0.5 * cam.m_forward, atol=1e-6)


def test_axes_are_those_of_the_last_frame(venu):
    """As in the reference, Pitch/MoveRight use the u/v/w of the last
    UVWFrame, not of the current forward vector."""
    cam = venu.Camera((0.0, 0.0, 0.0), 45.0, 1.0, 0.0, 1.0)
    U0, _, _ = cam.UVWFrame()
    cam.Yaw(30.0)
    cam.MoveRight(1.0)  # stale u: the one before the yaw
    assert np.allclose(cam.GetPosition(), U0 / np.linalg.norm(U0), atol=1e-6)
    U1, _, _ = cam.UVWFrame()
    assert not np.allclose(U0 / np.linalg.norm(U0), U1 / np.linalg.norm(U1), atol=1e-3)


def test_write_ppm(venu, tmp_path):
    W, H = 5, 3
    rng = np.random.default_rng(0)
    img = rng.integers(0, 256, size=(H, W, 4), dtype=np.uint8)
    p = tmp_path / "a.ppm"
    venu.write_ppm(str(p), img, W, H)
    data = p.read_bytes()
    head = b"P6\n5 3\n255\n"
    assert data[: len(head)] == head
    body = np.frombuffer(data[len(head):], np.uint8).reshape(H, W, 3)
    assert np.array_equal(body, img[::-1, :, :3])  # top row first


def test_write_pfm(venu, tmp_path):
    W, H = 4, 3
    rng = np.random.default_rng(1)
    img = rng.normal(size=(H, W, 4)).astype(np.float32)
    p = tmp_path / "a.pfm"
    venu.write_pfm(str(p), img, W, H)
    data = p.read_bytes()
    head = b"PF\n4 3\n-1.0\n"
    assert data[: len(head)] == head
    body = np.frombuffer(data[len(head):], "<f4").reshape(H, W, 3)
    assert np.array_equal(body, img[:, :, :3])  # bottom row first, as stored


def test_write_errors(venu, tmp_path):
    with pytest.raises(venu.VenuError):
        venu.write_ppm(str(tmp_path / "no" / "such" / "dir.ppm"), np.zeros(16, np.uint8), 2, 2)
    with pytest.raises(ValueError):
        venu.write_pfm(str(tmp_path / "x.pfm"), np.zeros(3, np.float32), 2, 2)
