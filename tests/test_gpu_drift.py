"""Device drift linkage (irc_calc_drift) against the numpy restatement of
calc_drift_ (oracle/drift_oracle.py): chunk limits and linkage identical."""
import numpy as np
import pytest

from ironclust_gb300 import irc
from oracle import drift_oracle as DO

pytestmark = pytest.mark.gpu


def _spikes(n, seed, grid=None, n_sites=16):
    """Amplitudes and positions with a slow drift; rounded to a grid when
    asked, so that ties (equal values, equal edges) occur."""
    rng = np.random.default_rng(seed)
    t = np.linspace(0, 1, n)
    amp = (rng.gamma(3.0, 20.0, n) * (1 + 0.2 * t)).astype(np.float32)
    pos = (rng.integers(0, n_sites, n) * 25.0 + rng.normal(0, 5, n) + 30 * t).astype(np.float32)
    if grid:
        amp = (np.round(amp / grid) * grid).astype(np.float32)
        pos = (np.round(pos / grid) * grid).astype(np.float32)
    return amp, pos


CASES = [
    dict(n=20000, seed=1, nTime_drift=40, nTime_batch=15),                 # all pairs
    dict(n=20000, seed=2, nTime_drift=40, nTime_batch=15, grid=5.0),       # ties
    dict(n=60000, seed=3, nTime_drift=300, nTime_batch=15),                # band (300 > 256)
    dict(n=350001, seed=4, nTime_drift=500, nTime_batch=12, grid=2.0),     # subsample with removal
    dict(n=30, seed=5, nTime_drift=40, nTime_batch=15),                    # empty chunks
    dict(n=5000, seed=6, nTime_drift=10, nTime_batch=15),                  # single-chunk branch
    dict(n=8000, seed=7, nTime_drift=64, nTime_batch=15, nTime_max_drift=32, n_sites=8),
]


@pytest.mark.parametrize("case", CASES, ids=[str(c["seed"]) for c in CASES])
def test_calc_drift_matches_oracle(gpu, case):
    c = dict(case)
    n_sites = c.pop("n_sites", 16)
    amp, pos = _spikes(c.pop("n"), c.pop("seed"), c.pop("grid", None), n_sites)
    kw = dict(nTime_drift=c["nTime_drift"], nTime_batch=c["nTime_batch"],
              nTime_max_drift=c.get("nTime_max_drift", 256))
    lim_o, ml_o = DO.calc_drift(amp, pos, n_sites, **kw)
    lim_d, ml_d, mem = irc.calc_drift(amp, pos, n_sites, members=True, **kw)
    np.testing.assert_array_equal(lim_d, lim_o)
    np.testing.assert_array_equal(ml_d, ml_o)
    if ml_d.shape[0] > 1:
        assert (ml_d.sum(0) == kw["nTime_batch"]).all()


def test_calc_drift_member_order(gpu):
    """Member lists come back in distance order: the chunk itself first
    (distance 0) unless an earlier chunk has an identical histogram."""
    amp, pos = _spikes(40000, 11)
    _, _, mem = irc.calc_drift(amp, pos, 16, 50, 15, members=True)
    assert (mem[0] == np.arange(50)).mean() > 0.9


def test_calc_drift_rejects_bad_band(gpu):
    from ironclust_gb300 import _lib
    amp, pos = _spikes(1000, 12)
    with pytest.raises(_lib.IrcError):
        irc.calc_drift(amp, pos, 16, 300, 15, nTime_max_drift=258)
