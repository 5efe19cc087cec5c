"""A batch of sites (different feature dimensions, chunk sizes down to a
single query) through one plan equals each site run on its own: bit for bit
in the REF and EXACT forms (zero-padded features add exactly 0), and for the
BF16 form wherever its filter kept the true neighbours (>= 99.9% of rows;
the position of the norm terms in K moves with the padding, so the
approximate distances may round differently)."""
import numpy as np
import pytest
import torch

from ironclust_gb300 import batch, irc, synth

pytestmark = pytest.mark.gpu

SPECS = [dict(n_spk=3000, n_dim=18, n_clusters=5, n_chunks=40, seed=1),
         dict(n_spk=700, n_dim=33, n_clusters=4, n_chunks=40, seed=2),
         dict(n_spk=9000, n_dim=24, n_clusters=8, n_chunks=40, seed=3),
         dict(n_spk=90, n_dim=24, n_clusters=3, n_chunks=40, seed=4),      # ~2 queries per chunk
         dict(n_spk=5200, n_dim=33, n_clusters=6, n_chunks=12, seed=5)]    # 433 per chunk: 128-row items


@pytest.fixture(scope="module")
def sites():
    return [synth.make_site(**s) for s in SPECS]


def _site_result(site, mode, gpu):
    plan = synth.site_plan(site)
    P = irc.Plan(plan)
    F = torch.from_numpy(site["F"]).to(gpu)
    out = irc.knn_rho_delta_site(P, F, knn=30, mode=mode)
    return {k: (v.cpu().numpy() if v is not None else None) for k, v in out.items()}


@pytest.mark.parametrize("mode", ["ref", "exact", "bf16"])
def test_batch_equals_sites(gpu, sites, mode):
    b = batch.SiteBatch(sites)
    P = irc.Plan(b.plan)
    F = torch.from_numpy(b.F).to(gpu)
    out = irc.knn_rho_delta_site(P, F, knn=30, mode=mode)
    got = {k: (v.cpu().numpy() if v is not None else None) for k, v in out.items()}
    for i, site in enumerate(sites):
        want = _site_result(site, mode, gpu)
        sl = b.site_slice(i)
        mi = b.split_knn(got["miKnn"], i)
        if mode == "bf16":
            same = np.all(mi == want["miKnn"], axis=1).mean()
            assert same >= 0.999, (i, same)
        else:
            assert np.array_equal(mi, want["miKnn"]), i
            assert np.array_equal(got["vrKnn"][sl].view(np.int32), want["vrKnn"].view(np.int32)), i
            assert np.array_equal(got["delta"][sl].view(np.int32), want["delta"].view(np.int32)), i
            assert np.array_equal(got["nneigh"][sl] - int(b.bases[i]), want["nneigh"]), i


def test_batch_plan_packs_small_chunks(sites):
    b = batch.SiteBatch(sites)
    nq = b.plan["nq"]
    assert (nq <= 32).sum() > 40 and (nq > 128).sum() >= 12
    assert b.F.shape == (sum(s["F"].shape[0] for s in sites), 33)
    # padding columns are zero
    assert not b.F[b.site_slice(0), 18:].any()
