"""Synthetic scene generators: sizes of the five workloads, watertightness,
determinism."""
import numpy as np

from rtgpu import scenes


def test_torus_size_and_determinism():
    a = scenes.torus()
    assert a.shape == (65536, 9) and a.dtype == np.float32
    assert np.array_equal(a, scenes.torus())


def test_geodesic_counts_and_watertight():
    for f in (1, 2, 5, 9):
        P, F = scenes.geodesic_sphere(f)
        assert len(F) == 20 * f * f
        assert len(P) == 10 * f * f + 2
        assert np.all(np.bincount(F.ravel(), minlength=len(P)) > 0)
        # every edge is shared by exactly two faces (closed manifold)
        e = np.sort(np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]]), axis=1)
        _, cnt = np.unique(e, axis=0, return_counts=True)
        assert np.all(cnt == 2)
    assert 20 * 324 * 324 == 2099520


def test_icosphere_frames_small():
    s = scenes.icosphere(freq=8)
    f0, f1 = s.frame(0), s.frame(1)
    assert f0.shape == (20 * 64, 9)
    assert not np.array_equal(f0, f1)
    assert np.array_equal(f0, s.frame(0))
    r = np.linalg.norm(s.verts, axis=1)
    assert r.min() > 0.8 and r.max() < 1.2


def test_gi_box():
    g = scenes.gi_box(n_soup=1000)
    assert g.tris.shape == (1014, 9)
    assert np.all(g.emission[12:14] == 10.0) and np.all(g.emission[14:] == 0) and np.all(g.emission[:12] == 0)
    assert g.albedo[14:].min() >= 0.2 and g.albedo[14:].max() <= 0.8
    assert scenes.gi_box().tris.shape[0] == 262158


def test_batch_sizes():
    s = scenes.batch_sizes()
    assert len(s) == 256 and s.min() >= 1000 and s.max() <= 200000
