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


def test_chol_level_features_and_candidates(sylver):
    """Per-level features of the Cholesky schedule learner: one finite row per
    level of the assembly tree, deterministic; the default schedule is one of
    the candidates and every candidate is a valid schedule."""
    from sylver_gb300 import scheduler as sc
    p = sc.spd_instance(500)
    an = sc.spd_analyse(p)
    lf = sc.level_features(an)
    sy = an.symbolic()
    par = sy["sparent"] - 1
    nn = sy["nnodes"]
    h = np.zeros(nn, int)
    for i in range(nn):
        if 0 <= par[i] < nn:
            h[par[i]] = max(h[par[i]], h[i] + 1)
    assert lf.shape == (h.max() + 1, sc.CHOL_LEVEL_FEATURES)
    assert np.all(np.isfinite(lf))
    np.testing.assert_array_equal(lf, sc.level_features(an))
    assert sc.CHOL_DEFAULT in sc.CHOL_CANDIDATES
    for c in sc.CHOL_CANDIDATES:
        assert c["fs_panel_cols"] % 64 == 0 and c["fs_panel_cols"] * c["fs_panel_group"] <= 512
        f = sc.chol_schedule_features(c)
        assert f.shape == (4,) and np.all(np.isfinite(f))
