"""The tensor-core work layouts give identical results; the autotuner picks
one of them by timing and caches its choice."""
import numpy as np
import pytest
import torch

from ironclust_gb300 import autotune, irc
from ironclust_gb300.batch import SiteBatch
from ironclust_gb300.synth import make_site

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small_batch(gpu):
    """Sites with chunks of every size class: > 64 queries, 33-64, <= 32."""
    sites = [make_site(n, d, 8, nch, seed=100 + k)
             for k, (n, d, nch) in enumerate([(9000, 33, 40), (2600, 24, 60), (900, 18, 40), (5000, 33, 200)])]
    b = SiteBatch(sites)
    return b, torch.from_numpy(b.F).to(gpu)


@pytest.mark.parametrize("mode", ["bf16", "fp8"])
def test_layouts_give_identical_results(small_batch, mode):
    b, F = small_batch
    P = irc.Plan(b.plan)
    ref = None
    for lay in autotune.CANDIDATES:
        autotune.apply(P, lay)
        k = irc.site_knn(P, F, 30, mode)
        got = (k["miKnn"].cpu().numpy(), k["d2Knn"].cpu().numpy().view(np.int32), k["rho"].cpu().numpy().view(np.int32))
        if ref is None:
            ref = got
        else:
            for a, r in zip(got, ref):
                assert np.array_equal(a, r), lay
    P.close()


def test_tune_picks_and_caches(small_batch, tmp_path, monkeypatch):
    monkeypatch.setenv("IRC_TUNE_CACHE", str(tmp_path / "tune.json"))
    b, F = small_batch
    P = irc.Plan(b.plan)
    r1 = autotune.tune(P, F, 30, "bf16")
    assert not r1["cached"] and tuple(r1["layout"]) in autotune.CANDIDATES
    assert set(r1["ms"]) == set(autotune.CANDIDATES) and all(v > 0 for v in r1["ms"].values())
    r2 = autotune.tune(P, F, 30, "bf16")
    assert r2["cached"] and tuple(r2["layout"]) == tuple(r1["layout"])
    P.close()
