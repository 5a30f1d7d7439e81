"""Host side of the schedule search: features of an analysed matrix (CPU)."""
import numpy as np

from sylver_gb300 import scheduler as sc


def test_tree_features_are_finite_and_deterministic(sylver):
    p = sc.kkt_instance(100)
    a1 = sc.analyse(p)
    a2 = sc.analyse(p)
    f1 = sc.tree_features(a1, False, 0, 37)
    f2 = sc.tree_features(a2, False, 0, 37)
    assert f1.dtype == np.float32 and np.all(np.isfinite(f1))
    assert np.array_equal(f1, f2)
    # front-count fractions are monotone in the threshold
    fr = f1[5:12]
    assert np.all(np.diff(fr) >= 0) and fr[-1] <= 1.0
    x = np.concatenate([f1, sc.schedule_features(64)])
    assert x.size == f1.size + 2


def test_kkt_instances_vary_in_size():
    ns = {sc.kkt_instance(s).a.n for s in range(100, 106)}
    assert len(ns) >= 3
