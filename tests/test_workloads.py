"""Host-side inputs of the benchmark configurations (no GPU)."""
import math

import numpy as np

from amressif_gb300 import workloads as wl


def test_perturbation_is_divergence_free_and_scaled():
    n = 64
    du, dv = wl.divfree_perturbation(n, amp=1e-3, seed=0)
    assert du.shape == (n, n + 1) and dv.shape == (n + 1, n)
    assert math.isclose(max(np.abs(du).max(), np.abs(dv).max()), 1e-3, rel_tol=1e-14)
    assert np.abs(wl.mac_divergence(du, dv)).max() <= 1e-15 * n
    np.testing.assert_array_equal(du[:, n], du[:, 0])
    np.testing.assert_array_equal(dv[n, :], dv[0, :])


def test_perturbation_is_seeded():
    a = wl.divfree_perturbation(32, seed=0)
    b = wl.divfree_perturbation(32, seed=0)
    c = wl.divfree_perturbation(32, seed=1)
    np.testing.assert_array_equal(a[0], b[0])
    assert not np.array_equal(a[0], c[0])


def test_tgv_fields_match_the_analytic_field():
    n = 16
    u, v, p = wl.tgv_fields(n)
    h = 2 * math.pi / n
    assert math.isclose(u[3, 5], math.sin(5 * h) * math.cos(3.5 * h), rel_tol=1e-15)
    assert math.isclose(v[3, 5], -math.cos(5.5 * h) * math.sin(3 * h), rel_tol=1e-15)
    assert math.isclose(p[3, 5], 0.25 * (math.cos(2 * 5.5 * h) + math.cos(2 * 3.5 * h)), rel_tol=1e-15)
    assert np.abs(wl.mac_divergence(u, v)).max() <= 1e-12
    assert math.isclose(wl.tgv_amplitude(u, v), 1.0, rel_tol=1e-14)


def test_lid_controls():
    c = wl.lid_controls(256, seed=0)
    assert c.shape == (256,)
    assert abs(c.mean() - 1.0) < 0.02 and 0.03 < c.std() < 0.07


def test_3d_perturbation_is_divergence_free():
    n = 16
    du = wl.divfree_perturbation3d(n, amp=1e-3, seed=0)
    assert [a.shape for a in du] == [(n, n, n + 1), (n, n + 1, n), (n + 1, n, n)]
    assert math.isclose(max(np.abs(a).max() for a in du), 1e-3, rel_tol=1e-14)
    assert np.abs(wl.mac_divergence3d(du)).max() <= 1e-14 * n
    u, p = wl.tgv3d_fields(n)
    assert np.abs(wl.mac_divergence3d(u)).max() <= 1e-12
