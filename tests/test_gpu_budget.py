"""Device-side loop limits.  Every BVH traversal runs under a budget of node
visits (ear_render_params.traverse_budget, automatic by default); one that
needs more stops, the launch still ends, and the call returns
EAR_ERR_DEVICE_BUDGET.  The limit is made to run out here with a budget of
one visit -- no GPU fault, trap or unbounded wait -- and the context stays
usable: the next render equals a render on a fresh scene."""
import numpy as np
import pytest

from ear_gb300 import Tracer, scenes
from ear_gb300 import _native as N

pytestmark = pytest.mark.gpu


def _render(tr, w, **kw):
    return tr.render(w.source, w.recorders, exact=True, **dict(w.render, num_rays=400, **kw))


@pytest.mark.parametrize("name", ["small_test_room", "relief_hall"])  # binary and 4-wide trees
def test_traversal_budget_ends_the_render_with_a_status(name):
    w = getattr(scenes, name)()
    with Tracer(w.vertices, w.material_ids, w.materials, device=0) as tr:
        assert tr.info()["width"] == (4 if w.vertices.shape[0] >= 4096 else 2)
        with pytest.raises(N.EarError) as e:
            _render(tr, w, traverse_budget=1)
        assert e.value.status == N.EAR_ERR_DEVICE_BUDGET
        after = _render(tr, w)
    with Tracer(w.vertices, w.material_ids, w.materials, device=0) as fresh:
        ref = _render(fresh, w)
    for key in ("rays", "segments", "shadow_queries", "contributions"):
        assert after.stats[key] == ref.stats[key] > 0
    np.testing.assert_array_equal(after.first_sample, ref.first_sample)
    np.testing.assert_array_equal(after.last_sample, ref.last_sample)


def test_a_sufficient_budget_changes_nothing():
    w = scenes.small_test_room()
    with Tracer(w.vertices, w.material_ids, w.materials, device=0) as tr:
        auto = _render(tr, w)
        wide = _render(tr, w, traverse_budget=1 << 20)
    assert auto.stats["segments"] == wide.stats["segments"]
    np.testing.assert_array_equal(auto.first_sample, wide.first_sample)
    with pytest.raises(N.EarError) as e:
        with Tracer(w.vertices, w.material_ids, w.materials, device=0) as tr:
            _render(tr, w, traverse_budget=-1)
    assert e.value.status == N.EAR_ERR_INVALID_ARG
