"""The FP8 recall-ceiling analysis (oracle/fp8_ceiling.py) on CPU: its e4m3
rounding equals PyTorch's float8_e4m3fn cast, and on a small drift site the
ceiling grows with the list length and is the same under per-chunk-pair
scaling as under one scale (scaling does not change e4m3's precision)."""
import numpy as np
import torch

from ironclust_gb300 import synth
from oracle import fp8_ceiling as C


def test_e4m3_rounding_matches_torch():
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.normal(0, s, 20000) for s in (0.001, 0.05, 1.0, 30.0, 200.0)])
    x = np.concatenate([x, [0.0, 448.0, -448.0, 2.0 ** -9, 2.0 ** -6, 3 * 2.0 ** -10, 0.6875, 17.0, 19.0]])
    x = np.clip(x, -448, 448)                                 # the cast is undefined past the largest value
    want = torch.from_numpy(x.astype(np.float32)).to(torch.float8_e4m3fn).to(torch.float64).numpy()
    got = C.e4m3(x)
    assert np.array_equal(got, want)


def test_ceiling_grows_with_list_length_and_ignores_scaling():
    site = synth.make_workload("drift400k", scale=0.05)
    res, n = C.ceiling(site["F"], synth.site_plan(site), Ms=(30, 60, 192), queries_per_chunk=32)
    assert n > 0
    for mode, r in res.items():
        assert r[30] <= r[60] <= r[192] <= 1.0, (mode, r)
    assert abs(res["global"][60] - res["per_pair"][60]) < 0.02
    assert res["global"][192] > res["global"][30]
