"""Generate golden vectors from the reference's own CUDA kernels.

Runs on a machine with a GPU: the reference kernels (PTX built from
the reference sources by oracle/build_oracle.py) are launched with the
MATLAB launch configuration through oracle/ref_harness.cu on seeded inputs
with the edge cases the kernels meet (exact duplicates, ragged chunks,
secondary-site runs, rho ties, runs that do not divide the bin count).  The
inputs and outputs are written to tests/golden/ref_kernels.npz; the large
[nThreads x nA] outputs are stored as SHA-256 digests plus their MATLAB
post-processed form (sort / min), so the fixture stays small.

    python tests/golden/make_golden.py [out.npz]
"""
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import torch  # noqa: E402

from oracle import oracle as O  # noqa: E402
from tests.cases import rho_with_ties, small_site  # noqa: E402


def digest(t):
    return hashlib.sha256(t.detach().cpu().numpy().tobytes()).hexdigest()


def main(out):
    dev = torch.device("cuda:0")
    rk = O.RefKernels()
    g = {}
    # --- search_min_drift / search_delta_drift on two sites --------------------------
    for name, case in (("s1", dict(n=1500, d=24, n_chunks=3, seed=21)),
                       ("s2", dict(n=1203, d=33, n_chunks=3, seed=22, sizes=[1, 601, 601], secondary=True))):
        F, plan, _ = small_site(**case)
        R = rho_with_ties(F.shape[0], 31)
        g[name + "_F"], g[name + "_R"] = F, R
        Fd, Rd = torch.from_numpy(F).to(dev), torch.from_numpy(R).to(dev)
        for i in range(len(plan["q0"])):
            r0, r1 = plan["roff"][i], plan["roff"][i + 1]
            IBB, NBB = plan["rs"][r0:r1], plan["rn"][r0:r1]
            vn = np.array([F.shape[1], F.shape[0], r1 - r0, plan["q0"][i], plan["nq"][i]], np.int32)
            key = "%s_c%d" % (name, i)
            g[key + "_IBB"], g[key + "_NBB"], g[key + "_vn"] = IBB, NBB, vn
            tI, tN = torch.from_numpy(IBB).to(dev), torch.from_numpy(NBB).to(dev)
            D, I = rk.search_min_drift(Fd, tI, tN, vn, nT=1024)
            g[key + "_min_sha"] = np.array([digest(D), digest(I)])
            v, m = O.post_sort_knn(D.cpu().numpy(), I.cpu().numpy(), 30)
            g[key + "_min_vrKnn"], g[key + "_min_miKnn"] = v, m
            D, I = rk.search_delta_drift(Fd, Rd, tI, tN, vn, nT=512)
            g[key + "_delta_sha"] = np.array([digest(D), digest(I)])
            v, m = O.post_min(D.cpu().numpy(), I.cpu().numpy())
            g[key + "_delta_min"], g[key + "_delta_idx"] = v, m
    # --- cuda_knn_index ---------------------------------------------------------------
    rng = np.random.default_rng(23)
    B = rng.normal(0, 3, (700, 33)).astype(np.float32)
    B[11] = B[10]
    A = np.concatenate([B[:20], rng.normal(0, 3, (30, 33))]).astype(np.float32)
    K, I = rk.cuda_knn_index(torch.from_numpy(B).to(dev), torch.from_numpy(A).to(dev), 30)
    g.update(knn_B=B, knn_A=A, knn_K=K.cpu().numpy(), knn_I=I.cpu().numpy())
    # --- cuda_delta_knn ---------------------------------------------------------------
    RB, RA = rho_with_ties(700, 24), rho_with_ties(50, 25)
    RA[0] = RB.max() + 1
    t = lambda x: torch.from_numpy(np.ascontiguousarray(x)).to(dev)
    D, N = rk.cuda_delta_knn(t(B), t(A), t(RB), t(RA))
    g.update(dknn_RB=RB, dknn_RA=RA, dknn_D=D.cpu().numpy(), dknn_N=N.cpu().numpy())
    # --- jrc3_cuda_rho_drift ----------------------------------------------------------
    f1 = rng.normal(0, 2, (800, 18)).astype(np.float32)
    f2 = (f1 + rng.normal(0, 0.5, (800, 18))).astype(np.float32)
    s1 = rng.integers(1, 4, 800).astype(np.int32)
    s2 = rng.integers(1, 4, 800).astype(np.int32)
    dc2 = np.float32(20.0)
    rho = rk.rho_drift(t(np.concatenate([s1, s2])), t(f1), t(f2), 200, float(dc2))
    g.update(rho_f1=f1, rho_f2=f2, rho_s1=s1, rho_s2=s2, rho_dc2=dc2, rho_out=rho.cpu().numpy())
    # --- jrc3_cuda_delta_drift (rho of all 800 spikes of the window) ------------------
    r12 = rho_with_ties(800, 26)
    de, nn = rk.delta_drift(t(np.concatenate([s1, s2])), t(f1), t(f2), t(r12), 200, float(dc2))
    g.update(ddrift_rho=r12, ddrift_delta=de.cpu().numpy(), ddrift_nn=nn.cpu().numpy())
    # --- cuda_knn / cuda_knn_full / cuda_knn_ib -----------------------------------------
    Bd, Ad = t(B), t(A)
    g.update(cknn_K=rk.cuda_knn(Bd, Ad, 30).cpu().numpy())
    K, I = rk.cuda_knn_full(Bd, Ad, 30)
    g.update(cknnf_K=K.cpu().numpy(), cknnf_I=I.cpu().numpy())
    IB = rng.integers(1, 701, 400).astype(np.int32)
    IB[:5] = IB[5]
    K, I = rk.cuda_knn_ib(Bd, Ad, t(IB), 30)
    g.update(cknnib_IB=IB, cknnib_K=K.cpu().numpy(), cknnib_I=I.cpu().numpy())
    # --- jrc3_cuda_rho / jrc3_cuda_delta (time window) ----------------------------------
    F12 = rng.normal(0, 2, (900, 24)).astype(np.float32)
    F12[3] = F12[2]
    ordr = np.sort(rng.integers(0, 450, 900)).astype(np.int32)[rng.permutation(900)]
    rr = (np.argsort(np.argsort(-rho_with_ties(900, 27), kind="stable"), kind="stable") + 1).astype(np.int32)
    g.update(st_F=F12, st_ord=ordr, st_rr=rr)
    for fdc, dcs in ((0, np.float32(4.0)), (1, np.float32(0.05))):
        rho = rk.cuda_rho(t(F12), t(ordr), 300, 60, float(dcs), fdc)
        de, nn = rk.cuda_delta(t(F12), t(ordr), t(rr), 300, 60, float(dcs), fdc)
        g["st%d_dc2" % fdc] = dcs
        g["st%d_rho" % fdc], g["st%d_delta" % fdc], g["st%d_nn" % fdc] = (
            rho.cpu().numpy(), de.cpu().numpy(), nn.cpu().numpy())
    torch.cuda.synchronize()
    np.savez_compressed(out, **g)
    print("wrote", out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                                            "ref_kernels.npz"))
