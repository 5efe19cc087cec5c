"""The C oracle of calc_dc2_drift_ (matlab/irc.m:24582-24608) against a
plain NumPy FP64 restatement: same subsampling, cut index and medians, so the
two agree to single-precision rounding; planted changes of the percentile and
of the subsample size are seen."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.dc2_cases import dc2_fp64, subsample_vr, window


def test_subsample_vr_matches_the_matlab_rule():
    assert subsample_vr(range(5), 10) == list(range(5))
    assert subsample_vr(range(10), 5) == [0, 2, 4, 6, 8]          # nSkip = 2
    v = subsample_vr(range(11), 5)                                 # nSkip 2 -> 6 entries, then one removed (the last)
    assert v == [0, 2, 4, 6, 8]
    v = subsample_vr(range(13), 4)                                 # nSkip 3 -> 5, remove round(linspace(1,5,1)) = 5
    assert v == [0, 3, 6, 9]


@pytest.mark.parametrize("n12,n1,nC,n_sites,sub,pct,seed", [(3000, 600, 12, 4, 100, 2.0, 1),
                                                            (5000, 900, 24, 7, 150, 5.0, 2),
                                                            (1200, 1200, 33, 3, 1000, 2.0, 3)])
def test_oracle_equals_fp64_restatement(n12, n1, nC, n_sites, sub, pct, seed):
    F1, F2, s1, s2 = window(n12, n1, nC, n_sites, seed)
    d, site = O.calc_dc2_drift(n1, s1, s2, F1, F2, n_sites, sub, pct)
    r, rsite = dc2_fp64(n1, s1, s2, F1, F2, n_sites, sub, pct)
    ok = np.isfinite(rsite)
    assert np.array_equal(np.isfinite(site), ok)
    assert np.allclose(site[ok], rsite[ok], rtol=1e-4, atol=1e-3)
    assert abs(d - r) <= 1e-4 * abs(r) + 1e-3
    # a different percentile or subsample size changes the answer
    assert O.calc_dc2_drift(n1, s1, s2, F1, F2, n_sites, sub, 2 * pct)[0] > d
    small = max(10, n1 // n_sites // 8)                             # thins every site's lists
    assert O.calc_dc2_drift(n1, s1, s2, F1, F2, n_sites, small, pct)[0] != d


def test_site_without_queries_is_nan_and_skipped():
    F1, F2, s1, s2 = window(2000, 400, 8, 3, 4)
    s1[:400][s1[:400] == 3] = 1                                    # no own spike on site 3
    d, site = O.calc_dc2_drift(400, s1, s2, F1, F2, 3, 100, 2.0)
    assert np.isnan(site[2]) and np.isfinite(site[:2]).all()
    assert d == np.float32(site[0] + (site[1] - site[0]) / np.float32(2)) or d == np.float32((site[0] + site[1]) / 2)
