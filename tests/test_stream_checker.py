"""The streamed-block FP64 check (oracle.accuracy.stream_block_check) on
CPU: block results computed with the exact FP32 oracle in the streaming
layout (ring coordinates, blocks k-1 .. k+1 around block k) pass on the first,
a middle and the last block, and a planted wrong neighbour is caught."""
import numpy as np
import pytest
import torch

from ironclust_gb300 import stream
from oracle import accuracy as A
from oracle import oracle as O

KNN = 10


class Recording:
    """The parts of a stream.Streamer the checker reads, with every block's
    kNN, rho and delta from the exact FP32 oracle on its ring."""

    N_SLOTS = 5

    def __init__(self, wl):
        self.wl = wl
        base, nb = wl["block_base"], wl["n_blocks"]
        self.slot_rows = int(np.max(np.diff(base)))
        self.slot_rows += (-self.slot_rows) % 4
        self.plans = [type("P", (), {"d": stream.block_plan(wl, k, self.slot_rows, self.N_SLOTS)})()
                      for k in range(nb)]
        N = int(base[-1])
        rho = np.zeros(N, np.float32)
        knn = {}
        for k in range(nb):
            idx, d2 = O.exact_knn_f32(self.ring(k), self.plans[k].d, KNN)
            a, z = int(base[k]), int(base[k + 1])
            rho[a:z] = np.float32(1) / np.sqrt(d2[:, KNN - 1])
            knn[k] = idx
        out = dict(rho=rho, miKnn=np.zeros((N, KNN), np.int32), delta=np.zeros(N, np.float32),
                   nneigh=np.zeros(N, np.int32))
        for k in range(nb):
            R = np.zeros(self.N_SLOTS * self.slot_rows, np.float32)
            for j in (k - 1, k, k + 1):
                if 0 <= j < nb:
                    a, z = int(base[j]), int(base[j + 1])
                    R[self._slot(j):self._slot(j) + z - a] = rho[a:z]
            nn, dd = O.exact_delta_f32(self.ring(k), R, self.plans[k].d)
            a, z = int(base[k]), int(base[k + 1])
            out["miKnn"][a:z] = knn[k]
            out["nneigh"][a:z] = nn
            out["delta"][a:z] = np.sqrt(dd) * rho[a:z]
        self.out = {key: torch.from_numpy(v) for key, v in out.items()}

    def _slot(self, j):
        return (j % self.N_SLOTS) * self.slot_rows

    def ring(self, k):
        base = self.wl["block_base"]
        F = np.zeros((self.N_SLOTS * self.slot_rows, self.wl["n_dim"]), np.float32)
        for j in (k - 1, k, k + 1):
            if 0 <= j < self.wl["n_blocks"]:
                a, z = int(base[j]), int(base[j + 1])
                F[self._slot(j):self._slot(j) + z - a] = self.wl["F16"][a:z].numpy()
        return F


@pytest.fixture(scope="module")
def rec():
    wl = stream.make_workload(n_sites=4, total=120_000, n_chunks=400, n_dim=12, pin=False)
    assert wl["n_blocks"] == 4
    return Recording(wl)


@pytest.mark.parametrize("k", [0, 2, 3])
def test_exact_fp32_blocks_pass(rec, k):
    acc = A.stream_block_check(rec, k, KNN)
    base = rec.wl["block_base"]
    assert acc["checked"] == acc["block_spikes"] == int(base[k + 1] - base[k])
    assert acc["recall_vs_fp64"] == 1.0
    assert acc["nneigh_errors"] == 0
    assert acc["rho_max_rel_err"] < 1e-6 and acc["delta_max_rel_err"] < 1e-6
    assert acc["delta_checked"] > 0.9 * acc["checked"]


def test_planted_wrong_neighbour_is_caught(rec):
    k = 1
    a = int(rec.wl["block_base"][k])
    nn = rec.out["nneigh"]
    old = nn.clone()
    try:
        q = a + int(np.flatnonzero(nn[a:a + 1000].numpy() != rec._slot(k) + np.arange(1, 1001))[0])
        nn[q] = nn[q] + 1 if nn[q] + 1 != rec._slot(k) + (q - a) + 1 else nn[q] + 2
        acc = A.stream_block_check(rec, k, KNN)
        assert acc["nneigh_errors"] == 1
    finally:
        rec.out["nneigh"] = old
