"""Host-side logic (no GPU): drift linkage, paging, launch plans, MATLAB
post-processing semantics, site sharding."""
import math

import numpy as np
import pytest
import torch

from ironclust_gb300 import drift, irc, shard, synth
from oracle import drift_oracle as DO
from oracle import oracle as O
from tests.cases import small_site


def test_chunk_limits_equal_counts():
    lim = drift.chunk_limits(1003, 7)
    assert lim[0] == 0 and lim[-1] == 1003
    assert list(lim[1:]) == [math.ceil(i / 7 * 1003) for i in range(1, 8)]


def test_mi2ml_and_dist_mask_keep_self_and_count():
    rng = np.random.default_rng(0)
    mrF = rng.normal(size=(5, 40))
    ml = DO.dist_mask_ml(mrF, np.ones((40, 40), bool), 7)
    assert ml.sum(0).tolist() == [7] * 40
    assert np.all(np.diag(ml))                     # distance 0 to itself sorts first
    mi = np.argsort(rng.random((40, 40)), 0)[:5]
    ml2 = drift.mi2ml_drift(mi)
    for j in range(40):
        assert set(np.flatnonzero(ml2[:, j])) == set(mi[:, j])


def test_drift_mask_band_and_edges():
    m = drift.drift_mask(300, 64)
    assert m[0, 0] and m[10, 74] and not m[0, 200]
    assert m[:129, :64].all() and m[-129:, -64:].all()


def test_calc_drift_linkage_shape():
    rng = np.random.default_rng(1)
    n = 20000
    amp = rng.gamma(2.0, 50.0, n).astype(np.float32)
    pos = rng.uniform(0, 600, n).astype(np.float32)
    lim, ml = DO.calc_drift(amp, pos, n_sites=16, nTime_drift=40, nTime_batch=15)
    assert lim[0] == 0 and lim[-1] == n and len(lim) == 41
    assert ml.shape == (40, 40) and np.all(np.diag(ml)) and np.all(ml.sum(0) == 15)
    lim1, ml1 = DO.calc_drift(amp, pos, 16, nTime_drift=10, nTime_batch=15)
    assert ml1.shape == (1, 1) and list(lim1) == [0, n]
    lim2, ml2 = DO.calc_drift(amp, pos, 16, nTime_drift=300, nTime_batch=15, nTime_max_drift=256)
    assert np.all(ml2.sum(0) == 15)
    i, j = np.nonzero(ml2)
    assert np.all(np.abs(i - j) <= 64 + 64)        # band of +/-64 plus the edge blocks


def test_quantile_and_subsample_follow_matlab_rounding():
    vr = np.arange(1, 11, dtype=np.float32)
    q = DO.quantile_vr(vr, [0, 0.25, 0.5, 1.0])
    # idx = max(min(round(n*q), n), 1): 1, round(2.5)=3, 5, 10
    assert q.tolist() == [1, 3, 5, 10]
    assert DO.subsample_vr(np.arange(10), 20).tolist() == list(range(10))
    assert DO.subsample_vr(np.arange(100), 10).tolist() == list(range(0, 100, 10))


@pytest.mark.parametrize("n", [100, 128, 200, 256, 300, 1000])
def test_plan_sort_page_covers_every_chunk_once(n):
    lim = drift.chunk_limits(n * 10, n)
    pages = drift.plan_sort_page(n, lim)
    covered = []
    for p in pages:
        a, b = p["drift_in"]
        A, B = p["drift_out"]
        assert A <= a <= b <= B and B - A + 1 <= 256
        covered.extend(range(a, b + 1))
    assert covered == list(range(n))


def test_build_plan_matches_the_matlab_run_selection():
    F, plan, vd = small_site(n=2500, d=8, n_chunks=4, seed=8, secondary=True, n_dup=0)
    vl = np.zeros(vd.size, bool)
    vl[:2500] = True
    ml = synth.make_site(2500, 8, 6, 4, 8)["mlDrift"]
    # restate the MATLAB loop directly
    change = [0] + [i for i in range(1, vd.size) if vd[i] != vd[i - 1]] + [vd.size]
    runs = [(change[k], change[k + 1] - change[k], vd[change[k]]) for k in range(len(change) - 1)]
    for i, a in enumerate(sorted(set(vd[:2500].tolist()))):
        want = [(s, n) for (s, n, c) in runs if ml[c, a]]
        r0, r1 = plan["roff"][i], plan["roff"][i + 1]
        got = list(zip(plan["rs"][r0:r1].tolist(), plan["rn"][r0:r1].tolist()))
        assert got == want
        q = np.flatnonzero(vd[:2500] == a)
        assert plan["q0"][i] == q[0] and plan["nq"][i] == q.size
    assert plan["n_out"] == 2500 and plan["q_base"] == 0 and plan["n_f"] == vd.size


def test_build_plan_rejects_non_contiguous_queries():
    vd = np.array([0, 0, 1, 1, 0])
    with pytest.raises(ValueError):
        drift.build_plan(vd, np.array([1, 0, 1, 1, 1], bool), np.ones((2, 2), bool))


def test_plan_pairs_counts_linked_candidates():
    F, plan, _ = small_site(n=1000, d=8, n_chunks=1, seed=3)
    assert drift.plan_pairs(plan) == 1000 * 1000


def test_matlab_sort_and_min_semantics_match_the_oracle():
    rng = np.random.default_rng(5)
    D = rng.integers(0, 6, (40, 64)).astype(np.float32)      # many ties
    D[3, 5] = np.nan
    D[7, :] = np.nan
    I = rng.integers(1, 1000, (40, 64)).astype(np.int32)
    v, m = irc.matlab_sort_knn(torch.from_numpy(D), torch.from_numpy(I), 10)
    vo, mo = O.post_sort_knn(D, I, 10)
    assert np.array_equal(np.nan_to_num(v.numpy(), nan=-1), np.nan_to_num(vo, nan=-1))
    assert np.array_equal(m.numpy(), mo)
    v, m = irc.matlab_min(torch.from_numpy(D), torch.from_numpy(I))
    vo, mo = O.post_min(D, I)
    assert np.array_equal(np.nan_to_num(v.numpy(), nan=-1), np.nan_to_num(vo, nan=-1))
    assert np.array_equal(m.numpy(), mo)


def test_rho_and_delta_post_processing_quirks():
    rho, mi = irc.rho_post(np.array([2.0, 4.0], np.float32), np.array([[1, 2], [2, 2]]),
                           np.array([10, 20, 30]), knn=3)
    assert rho.tolist() == [0.5, 0.25]
    assert mi.tolist() == [[10, 20, 20], [20, 20, 20]]       # padded by repeating the last row
    d, nn = irc.delta_post(np.array([1.0, np.inf, np.nan], np.float32), np.array([2, 3, 1]),
                           np.array([10, 20, 30]))
    assert nn.tolist() == [20, 2, 3]                          # NaN/Inf -> the spike's own local position
    assert d[1] == d[2] == irc.SQRT_SINGLE_INF_F


def test_synthetic_sites_are_seeded():
    a = synth.make_site(500, 6, 3, 5, seed=11)
    b = synth.make_site(500, 6, 3, 5, seed=11)
    assert np.array_equal(a["F"], b["F"]) and np.array_equal(a["mlDrift"], b["mlDrift"])
    assert a["F"].dtype == np.float32 and a["F"].shape == (500, 6)
    specs = synth.probe_site_specs(n_sites=384)
    assert len(specs) == 384 and all(500 <= s["n_spk"] for s in specs)


def test_lpt_site_assignment():
    costs = [50, 40, 30, 30, 20, 10, 5, 5]
    a = shard.assign_sites(costs, 3)
    assert sorted(sum(a, [])) == list(range(8))
    assert shard.imbalance(costs, a) < 1.15
    assert shard.assign_sites(costs, 3) == a                 # deterministic
    assert shard.assign_sites(costs, 1) == [list(range(8))]


def test_fet_selection_matches_reference_reader(tmp_path):
    """The host side of load_fet_site_ (which record of which load) picks the
    records the reference reader returns."""
    from ironclust_gb300 import files
    from oracle import io_oracle as IO
    rng = np.random.default_rng(2)
    tr = [rng.normal(size=(n, 4, 3)).astype(np.float32) for n in (300, 0, 500)]
    site = [rng.integers(0, 4, len(x)) for x in tr]
    fs, cc = IO.write_fet_files(str(tmp_path / "r"), tr, site, 4)
    recs = []
    for path, load in zip(fs, cc):
        raw = np.fromfile(path, np.float32).reshape(-1, 12)
        recs.append(raw)
    for s in range(4):
        everyone = np.concatenate([load[s] for load in cc])
        vi = np.sort(rng.choice(everyone, len(everyone) // 2, replace=False))
        before, counts, sel, spikes = files.fet_selection(cc, s, vi)
        site_recs = np.concatenate([r[b:b + c] for r, b, c in zip(recs, before, counts)])
        assert np.array_equal(site_recs[sel], IO.load_fet_site(fs, cc, s, vi, 3, 4))
        assert np.array_equal(spikes, vi)


def test_stream_block_plans_address_the_linked_chunks():
    """Every block plan of the page-streaming pipeline, with its ring rows
    mapped back to the block-major recording, queries exactly the block's
    (site, chunk) pieces and lists the non-empty linked chunks of the same
    site, in ascending chunk order."""
    from ironclust_gb300 import stream
    wl = stream.make_workload(n_sites=5, total=20000, n_chunks=300, pin=False)
    S, Bc, nb = 5, wl["block_chunks"], wl["n_blocks"]
    lims, seg, base = wl["lims"], wl["seg"], wl["block_base"]
    owner = np.full((int(base[-1]), 2), -1, np.int64)              # (site, chunk) of every recording row
    for kb in range(nb):
        for s in range(S):
            for c in range(kb * Bc, min((kb + 1) * Bc, wl["n_chunks"])):
                r0 = seg[kb, s] + lims[s, c] - lims[s, kb * Bc]
                owner[r0:r0 + lims[s, c + 1] - lims[s, c]] = (s, c)
    assert (owner >= 0).all()
    n_slots, slot_rows = 5, int(np.max(np.diff(base)))
    for k in range(nb):
        p = stream.block_plan(wl, k, slot_rows, n_slots)
        assert p["q_base"] == (k % n_slots) * slot_rows and p["n_out"] == base[k + 1] - base[k]

        def glob(r):                                                # ring row -> recording row
            j = [j for j in (k - 1, k, k + 1) if 0 <= j < nb and (j % n_slots) * slot_rows <= r
                 < (j % n_slots) * slot_rows + base[j + 1] - base[j]]
            assert len(j) == 1
            return int(base[j[0]] + r - (j[0] % n_slots) * slot_rows)

        seen = 0
        for i in range(len(p["q0"])):
            g = glob(int(p["q0"][i]))
            s, c = owner[g]
            assert p["nq"][i] == lims[s, c + 1] - lims[s, c]
            assert (owner[g:g + p["nq"][i]] == (s, c)).all()
            want = [m for m in wl["members"][:, c] if lims[s, m + 1] > lims[s, m]]
            runs = range(p["roff"][i], p["roff"][i + 1])
            got = [tuple(owner[glob(int(p["rs"][r]))]) for r in runs]
            assert got == [(s, m) for m in want]
            assert [int(p["rn"][r]) for r in runs] == [lims[s, m + 1] - lims[s, m] for m in want]
            seen += int(p["nq"][i])
        assert seen == p["n_out"]


def test_min_time_roofline_reports_both_terms():
    """bench.min_time_roofline: the minimum time is the larger of the tensor
    and the HBM term, and frac = minimum / measured."""
    import bench
    peaks = dict(hbm=1000.0, bf16=2000.0, bf16_sus=1000.0, src="test")
    r = bench.min_time_roofline(2e12, 5e9, 10.0, peaks)       # 2 ms of tensor work, 5 ms of bytes
    assert r["bound"] == "hbm" and abs(r["t_tensor_ms"] - 2.0) < 1e-9 and abs(r["t_hbm_ms"] - 5.0) < 1e-9
    assert abs(r["min_ms"] - 5.0) < 1e-9 and abs(r["frac"] - 0.5) < 1e-9
    r = bench.min_time_roofline(8e12, 1e9, 16.0, peaks)
    assert r["bound"] == "tensor" and abs(r["frac"] - 0.5) < 1e-9
