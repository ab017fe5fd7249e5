"""Checkpoint directory layout of SaveCheckpoint / LoadCheckpoint (no GPU)."""
import os

import numpy as np

from amressif_gb300 import checkpoint as ck


def state(n, seed=0):
    r = np.random.default_rng(seed)
    u = [r.standard_normal((n, n + 1)), r.standard_normal((n + 1, n))]
    up = [r.standard_normal((n, n + 1)), r.standard_normal((n + 1, n))]
    return u, up, r.standard_normal((n, n))


def test_round_trip_uneven_boxes(tmp_path):
    n = 10
    u, up, p = state(n)
    path = ck.write_checkpoint(str(tmp_path), 7, u, up, p, 0.123456789012345678, (4, 3))
    assert os.path.basename(path) == "checkpoint00007"
    u2, up2, p2, t = ck.read_checkpoint(path)
    assert t == float("%.15g" % 0.123456789012345678)
    np.testing.assert_array_equal(p2, p)
    for a, b in zip(u + up, u2 + up2):
        np.testing.assert_array_equal(a, b)


def test_header_and_boxes(tmp_path):
    n = 8
    u, up, p = state(n, 1)
    path = ck.write_checkpoint(str(tmp_path), 0, u, up, p, 2.5, (4, 8))
    lines = open(os.path.join(path, "Header")).read().splitlines()
    assert lines[:5] == ["Checkpoint file for AMRESSIF", "2.5", "(2 0", "((0,0) (3,7) (0,0))", "((4,0) (7,7) (0,0))"]
    h = open(os.path.join(path, "Level_0", "vel_xCont_H")).read()
    assert "((0,0) (4,7) (1,0))" in h and "((4,0) (8,7) (1,0))" in h  # face boxes share the face between boxes
    with open(os.path.join(path, "Level_0", "vel_xCont_D_00000"), "rb") as f:
        head = f.readline().decode()
    assert head.startswith("FAB ((8, (64 11 52 0 1 12 0 1023)),(8, (8 7 6 5 4 3 2 1)))((0,0) (4,7) (1,0)) 1")


def test_chop_covers_domain():
    boxes = ck.chop(13, (5, 4))
    cover = np.zeros((13, 13), int)
    for (x0, y0), (x1, y1) in boxes:
        cover[y0:y1 + 1, x0:x1 + 1] += 1
    assert (cover == 1).all()


def test_plotfile_round_trip(tmp_path):
    n = 12
    u, up, p = state(n, 2)
    path = ck.write_plotfile(str(tmp_path), "plt", 42, u, p, 0.75, (8, 5))
    assert os.path.basename(path) == "plt00042"
    fields, t, step = ck.read_plotfile(path)
    assert t == 0.75 and step == 42
    cu, cv = ck.cell_velocity(u)
    np.testing.assert_array_equal(fields["pressure"], p)
    np.testing.assert_array_equal(fields["U"], cu)
    np.testing.assert_array_equal(fields["V"], cv)
    head = open(os.path.join(path, "Header")).read().splitlines()
    assert head[:6] == ["HyperCLaw-V1.1", "3", "pressure", "U", "V", "2"]
    assert head[-1] == "Level_0/Cell"


def state3(n, seed=0):
    r = np.random.default_rng(seed)
    shapes = [(n, n, n + 1), (n, n + 1, n), (n + 1, n, n)]
    return ([r.standard_normal(s) for s in shapes], [r.standard_normal(s) for s in shapes],
            r.standard_normal((n, n, n)))


def test_round_trip_3d(tmp_path):
    """vel_zCont / vel_zContPrev of the 3D build (utilities.cpp:821-822, 888-889)"""
    n = 6
    u, up, p = state3(n)
    path = ck.write_checkpoint(str(tmp_path), 3, u, up, p, 1.25, (4, 3, 5))
    names = sorted(f for f in os.listdir(os.path.join(path, "Level_0")) if f.endswith("_H"))
    assert names == sorted(x + "_H" for x in ck.fields(3))
    u2, up2, p2, t = ck.read_checkpoint(path)
    assert t == 1.25
    np.testing.assert_array_equal(p2, p)
    for a, b in zip(u + up, u2 + up2):
        np.testing.assert_array_equal(a, b)
    lines = open(os.path.join(path, "Header")).read().splitlines()
    assert lines[2] == "(8 0" and lines[3] == "((0,0,0) (3,2,4) (0,0,0))"
    h = open(os.path.join(path, "Level_0", "vel_zCont_H")).read()
    assert "((0,0,0) (3,2,5) (0,0,1))" in h and "((4,3,5) (5,5,6) (0,0,1))" in h


def test_plotfile_3d_has_w(tmp_path):
    n = 5
    u, _, p = state3(n, 4)
    path = ck.write_plotfile(str(tmp_path), "plt", 7, u, p, 0.5, (3, 4, 2), prob_hi=(2.0, 2.0, 2.0))
    fields, t, step = ck.read_plotfile(path)
    assert t == 0.5 and step == 7 and sorted(fields) == ["U", "V", "W", "pressure"]
    cart = ck.cell_velocity(u)
    np.testing.assert_array_equal(fields["W"], 0.5 * (u[2][:-1] + u[2][1:]))
    for name, c in zip("UVW", cart):
        np.testing.assert_array_equal(fields[name], c)
    np.testing.assert_array_equal(fields["pressure"], p)
    head = open(os.path.join(path, "Header")).read().splitlines()
    assert head[:7] == ["HyperCLaw-V1.1", "4", "pressure", "U", "V", "W", "3"]
