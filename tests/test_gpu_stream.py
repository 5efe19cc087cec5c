"""The streaming pipeline (FP16 host features, overlapped copies, group
plans) gives the results of the same plans run directly, and the BF16 form
keeps its recall against the FP64 oracle."""
import numpy as np
import pytest
import torch

from ironclust_gb300 import irc, stream
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def streamed(gpu):
    wl = stream.make_workload(n_sites=24, total=1_500_000, n_chunks=1000)
    st = stream.Streamer(wl, knn=30, mode="bf16", group_target=200_000)
    st.run()                                      # first pass allocates the plans' operand buffers
    ms = st.run()
    yield wl, st, ms
    st.close()


def test_stream_matches_direct_plans(streamed):
    wl, st, ms = streamed
    assert len(st.groups) > 3 and ms > 0
    for g, (a, z) in enumerate(st.bounds):
        F = torch.from_numpy(wl["F16"][a:z].numpy().astype(np.float32)).cuda()
        r = irc.knn_rho_delta_site(st.plans[g], F, knn=30, mode="bf16")
        assert np.array_equal(st.out["miKnn"][a:z].numpy(), r["miKnn"].cpu().numpy()), g
        assert np.array_equal(st.out["rho"][a:z].numpy().view(np.int32), r["rho"].cpu().numpy().view(np.int32))
        assert np.array_equal(st.out["delta"][a:z].numpy().view(np.int32), r["delta"].cpu().numpy().view(np.int32))
        assert np.array_equal(st.out["nneigh"][a:z].numpy(), r["nneigh"].cpu().numpy())


def test_stream_recall_vs_fp64(streamed):
    wl, st, _ = streamed
    s = 1                                          # one site of the first group
    b0 = int(wl["bases"][st.groups[0][0]])
    a, z = int(wl["bases"][s]) - b0, int(wl["bases"][s + 1]) - b0
    plan = stream.site_plan_from_members(wl["lims"][s], wl["members"], 0)
    plan.update(q_base=0, n_out=z - a, n_f=z - a)
    F = wl["F16"][b0 + a:b0 + z].numpy().astype(np.float32)
    i64, d64 = O.exact_knn_f64(F, plan, 30)
    got = st.out["miKnn"][b0 + a:b0 + z].numpy() - a
    rec = np.mean([len(set(x) & set(y)) / 30.0 for x, y in zip(got, i64)])
    assert rec >= 0.999, rec
    ok = np.isfinite(d64[:, 29])
    rho64 = 1.0 / np.sqrt(d64[ok, 29])
    rel = np.abs(st.out["rho"][b0 + a:b0 + z].numpy()[ok] - rho64) / rho64
    assert rel.max() <= 1e-4, rel.max()
