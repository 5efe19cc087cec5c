"""The page-streaming pipeline (FP16 host features, a five-block device ring,
overlapped copies, kNN one block ahead of delta) gives the results of the
same block plans run directly, and the BF16 form keeps its recall, rho and
delta accuracy against the FP64 oracle."""
import numpy as np
import pytest
import torch

from ironclust_gb300 import irc, stream
from oracle import accuracy as A

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def streamed(gpu):
    wl = stream.make_workload(n_sites=24, total=1_500_000, n_chunks=1000)
    st = stream.Streamer(wl, knn=30, mode="bf16")
    st.run()                                      # first pass: caches, lazily made plan buffers
    ms = st.run()
    yield wl, st, ms
    st.close()


def _ring_for(st, k):
    """Ring holding blocks k-2 .. k+2 in their slots: enough for the plans of
    blocks k-1 .. k+1."""
    F = np.zeros((st.N_SLOTS * st.slot_rows, st.wl["n_dim"]), np.float32)
    for j in range(k - 2, k + 3):
        if 0 <= j < st.wl["n_blocks"]:
            a, z = st.block_rows(j)
            F[st._slot(j):st._slot(j) + (z - a)] = st.wl["F16"][a:z].numpy()
    return torch.from_numpy(F).cuda()


@pytest.mark.parametrize("k", [0, 3, -1])
def test_stream_matches_direct_plans(streamed, k):
    wl, st, ms = streamed
    nb = wl["n_blocks"]
    k = k % nb
    assert nb >= 6 and ms > 0
    F = _ring_for(st, k)
    R = torch.zeros(F.shape[0], dtype=torch.float32, device="cuda")
    res = {}
    for j in (k - 1, k, k + 1):
        if 0 <= j < nb:
            r = irc.site_knn(st.plans[j], F, 30, "bf16")
            n = st.plans[j].n_out
            R[st._slot(j):st._slot(j) + n] = r["rho"]
            res[j] = r
    delta, nneigh = irc.site_delta(st.plans[k], F, R, "bf16", knn=30, miKnn=res[k]["miKnn"], d2Knn=res[k]["d2Knn"])
    a, z = st.block_rows(k)
    assert np.array_equal(st.out["miKnn"][a:z].numpy(), res[k]["miKnn"].cpu().numpy())
    assert np.array_equal(st.out["rho"][a:z].numpy().view(np.int32), res[k]["rho"].cpu().numpy().view(np.int32))
    assert np.array_equal(st.out["delta"][a:z].numpy().view(np.int32), delta.cpu().numpy().view(np.int32))
    assert np.array_equal(st.out["nneigh"][a:z].numpy(), nneigh.cpu().numpy())


@pytest.mark.parametrize("where", ["first", "middle", "last"])
def test_stream_accuracy_vs_fp64(streamed, where):
    """kNN recall, rho and delta (nearest higher-rho neighbour included) of a
    streamed block against FP64 (oracle.accuracy.stream_block_check: FP64
    kNN on the block and its two neighbours, FP64 delta on the block)."""
    wl, st, _ = streamed
    k = {"first": 0, "middle": wl["n_blocks"] // 2, "last": wl["n_blocks"] - 1}[where]
    acc = A.stream_block_check(st, k, 30)
    assert acc["checked"] == acc["block_spikes"] > 0
    assert acc["recall_vs_fp64"] >= 0.999, acc
    assert acc["rho_max_rel_err"] <= 1e-5, acc
    assert acc["delta_checked"] > 0.9 * acc["checked"], acc
    assert acc["delta_max_rel_err"] <= 1e-5, acc
    assert acc["nneigh_errors"] == 0, acc


def test_stream_global_rows(streamed):
    """to_global maps ring rows back to recording rows: every neighbour of a
    block lies in the block or its two neighbours, and the mapping inverts
    the block layout."""
    wl, st, _ = streamed
    k = 2
    a, z = st.block_rows(k)
    g = st.to_global(k, st.out["miKnn"][a:z].numpy())
    lo, hi = st.block_rows(k - 1)[0], st.block_rows(k + 1)[1]
    assert ((g == 0) | ((g > lo) & (g <= hi))).all()
    F16 = wl["F16"].numpy()
    ring = st.ring_rows(k)
    mi = st.out["miKnn"][a:z].numpy()
    sel = mi[:, 0] > 0
    assert np.array_equal(ring[mi[sel, 0] - 1], F16[g[sel, 0] - 1].astype(np.float32))
