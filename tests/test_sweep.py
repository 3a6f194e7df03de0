"""The batched-sweep scene generator (host only)."""
import numpy as np
import pytest

pytest.importorskip("scipy")
from ear_gb300 import scenes  # noqa: E402


def _volume(v):
    t = v.reshape(-1, 3, 3).astype(np.float64)
    return np.einsum("ij,ij->i", t[:, 0], np.cross(t[:, 1], t[:, 2])).sum() / 6.0


def test_sweep_rooms_shape():
    rooms, render = scenes.sweep_rooms(num_rooms=4, pairs_per_room=3, keyframes=5,
                                       min_tris=500, max_tris=20000, seed=11)
    assert render["num_bins"] == 2 * 44100 and render["num_rays"] == 1_000_000
    for r in rooms:
        assert 400 <= r.num_triangles <= 24000
        assert 4 <= len(r.materials) <= 8
        assert r.material_ids.min() >= 0 and r.material_ids.max() < len(r.materials)
        assert _volume(r.vertices) > 0  # outward winding
        assert len(r.sources) == len(r.listeners) == 3
        for s, l in zip(r.sources, r.listeners):
            loc = s.location
            assert loc.shape == (5, 3)
            assert np.linalg.norm(loc[-1] - loc[0]) == pytest.approx(5.0, rel=1e-5)
            for p in list(loc) + [l.location]:
                assert np.all(r.halfspaces[:, :3] @ p + r.halfspaces[:, 3] <= -0.5 + 1e-4)


def test_subdivision_keeps_area_and_winding():
    rng = np.random.default_rng(0)
    t = rng.standard_normal((5, 9))
    s = scenes._subdivide(t, 2)
    assert s.shape == (80, 9)

    def area_normal(x):
        x = x.reshape(-1, 3, 3)
        return np.cross(x[:, 1] - x[:, 0], x[:, 2] - x[:, 0]) * 0.5

    np.testing.assert_allclose(area_normal(s).reshape(5, 16, 3).sum(1), area_normal(t), atol=1e-9)
