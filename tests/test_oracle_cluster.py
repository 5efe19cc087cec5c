"""The C oracle of the clustering step (sort_ normalisation, postCluster_ /
assignCluster_knn_) against a second, literal restatement in Python.

MATLAB is not available here and the reference holds no fixtures for these
functions, so two independent restatements of the same MATLAB text checking
each other is the strongest check available on the CPU."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.cluster_cases import (assign_cluster_knn_literal, geometric_case, random_case,
                                 sort_rho_literal)


def _same(a, b):
    for k in ("nClu", "nClu_pre", "nClu_post"):
        assert a[k] == b[k], k
    for k in ("viClu", "icl", "vnSpk_clu"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


@pytest.mark.parametrize("seed", range(4))
def test_sort_rho_matches_literal(seed):
    rng = np.random.default_rng(seed)
    rho = rng.gamma(2.0, 1.0, 500).astype(np.float32)
    rho[::37] = rho[5]                      # ties
    if seed % 2:
        rho[rng.random(500) < 0.03] = np.nan
    r1, o1 = O.sort_rho(rho)
    r2, o2 = sort_rho_literal(rho)
    np.testing.assert_array_equal(r1.view(np.uint32), r2.view(np.uint32))
    np.testing.assert_array_equal(o1, o2)


CASES = [
    dict(seed=1),
    dict(seed=2, vocab=150),                  # dense overlap: large merged groups
    dict(seed=3, vocab=2000, knn=3),          # sparse overlap: many singletons
    dict(seed=4, levels=4),                   # rho ties
    dict(seed=5, p_quirk=0.3),                # nneigh to later spikes / itself: extra passes
    dict(seed=6, p_nan=0.03),                 # NaN rho and delta
    dict(seed=7, delta_scale=0.05),           # very few peaks
    dict(seed=8, n=60, knn=2, vocab=400),
    dict(seed=9, levels=4, vocab=3000, knn=4),   # ties with several clusters
    dict(seed=10, p_quirk=0.3, vocab=4000, knn=3),
    dict(seed=11, p_nan=0.03, vocab=4000, knn=3),
    dict(seed=12, p_quirk=0.6, vocab=20000, knn=2),  # self loops: spikes left at 0 after ten passes
]


@pytest.mark.parametrize("case", CASES, ids=[str(c["seed"]) for c in CASES])
@pytest.mark.parametrize("min_count", [0, 5])
def test_assign_matches_literal(case, min_count):
    rho, delta, ordrho, nneigh, mk = random_case(**case)
    a = O.assign_cluster_knn(rho, delta, ordrho, nneigh, mk, 1.0, min_count)
    b = assign_cluster_knn_literal(rho, delta, ordrho, nneigh, mk, 1.0, min_count)
    _same(a, b)


@pytest.mark.parametrize("cut", [1.0, 1e30, 0.0])
def test_assign_edge_peak_counts(cut):
    """No peak, every spike a peak, and the usual cut."""
    rho, delta, ordrho, nneigh, mk = random_case(11, n=200)
    a = O.assign_cluster_knn(rho, delta, ordrho, nneigh, mk, cut, 3)
    b = assign_cluster_knn_literal(rho, delta, ordrho, nneigh, mk, cut, 3)
    _same(a, b)
    if cut == 1e30:
        assert a["nClu_pre"] == 0 and a["nClu_post"] == 1 and a["icl"][0] == ordrho[0]


def test_assign_geometric():
    rho, delta, ordrho, nneigh, mk = geometric_case(3, n=1500)
    a = O.assign_cluster_knn(rho, delta, ordrho, nneigh, mk, 1.0, 10)
    b = assign_cluster_knn_literal(rho, delta, ordrho, nneigh, mk, 1.0, 10)
    _same(a, b)
    assert a["nClu"] >= 2


def test_assign_bad_index_raises():
    rho, delta, ordrho, nneigh, mk = random_case(12, n=100, knn=2, vocab=5000)
    assert O.assign_cluster_knn(rho, delta, ordrho, nneigh, mk, 1.0, 0)["nClu_post"] > 1
    nneigh = nneigh.copy()
    unlabeled = np.nonzero(delta < 1.0)[0]
    nneigh[unlabeled[0]] = 0
    with pytest.raises(ValueError):
        O.assign_cluster_knn(rho, delta, ordrho, nneigh, mk, 1.0, 0)
