"""The FP64 accuracy checker (oracle/accuracy.py) on CPU: an exact FP32
result passes, a planted wrong neighbour is an error, and a neighbour whose
rho order differs between FP32 and FP64 is counted as a rho-order flip."""
import numpy as np

from ironclust_gb300 import synth
from oracle import accuracy as A
from oracle import oracle as O


def exact_fp32(site, plan):
    idx, d2 = O.exact_knn_f32(site["F"], plan, 30)
    rho = (np.float32(1) / np.sqrt(d2[:, 29])).astype(np.float32)
    nn, dd = O.exact_delta_f32(site["F"], rho, plan)
    return dict(miKnn=idx, rho=rho, delta=(np.sqrt(dd) * rho).astype(np.float32), nneigh=nn)


def test_checker_passes_exact_and_catches_planted_mistakes():
    site = synth.make_site(3000, 12, 5, 3, seed=5)
    plan = synth.site_plan(site)
    ref = A.fp64_reference(site["F"], plan, 30)
    out = exact_fp32(site, plan)
    acc = A.compare(out, ref)
    assert acc["recall_vs_fp64"] == 1.0 and acc["nneigh_errors"] == 0
    assert acc["rho_max_rel_err"] < 1e-6 and acc["delta_max_rel_err"] < 1e-6
    # a wrong nearest higher-rho neighbour: an error, and a large delta error
    q = int(np.flatnonzero(out["nneigh"] != np.arange(1, 3001))[0])
    bad = dict(out, nneigh=out["nneigh"].copy(), delta=out["delta"].copy())
    bad["nneigh"][q] = q + 2 if q + 2 != out["nneigh"][q] else q + 3
    bad["delta"][q] *= 2
    acc = A.compare(bad, ref)
    assert acc["nneigh_errors"] == 1 and acc["delta_max_rel_err"] > 0.5
    # a wrong kNN entry lowers the recall
    knn_bad = dict(out, miKnn=out["miKnn"].copy())
    knn_bad["miKnn"][:10, 0] = knn_bad["miKnn"][:10, 29]
    assert A.compare(knn_bad, ref)["recall_vs_fp64"] < 1.0


def test_rho_order_flip_only_below_fp32_resolution():
    """Spike 0's FP64 nearest higher-rho neighbour is spike 1, whose rho64 is
    5e-7 above spike 0's; the result's FP32 rho ranks spike 1 below spike 0
    and picks spike 2: a rho-order flip.  The same choice with rho64 values
    far apart is an error."""
    def case(r1):
        ref = dict(idx=np.array([[2], [3], [2]]), d2=np.array([[1.0], [1.0], [1.0]]),
                   rho=np.array([1.0, r1, 2.0]), nneigh=np.array([2, 3, 0]), delta=np.array([1.0, r1, np.inf]))
        out = dict(miKnn=np.array([[2], [3], [2]]), rho=np.array([1.0, 0.9999999, 2.0], np.float32),
                   delta=np.array([2.0, r1, 1e19], np.float32), nneigh=np.array([3, 3, 3]))
        return A.compare(out, ref)
    acc = case(1.0 + 5e-7)
    assert acc["nneigh_rho_order_flips"] == 1 and acc["nneigh_errors"] == 0
    acc = case(1.5)
    assert acc["nneigh_rho_order_flips"] == 0 and acc["nneigh_errors"] == 1
