"""Plans at the size limit of irc_site_knn_exact_noalloc's fixed array.

The array holds 2^21 int32 words; a plan takes
    4 + 2*n_out + 4*nChunks + 2 + 2*nRuns
of them (queue counters, two query queues, q0, nq, roff, rs, rn and the
16-query tile table).  With C one-query chunks of one 32-candidate run each
and n_out = C + extra, a plan takes 8 + 8*C + 2*(extra - 1) words, so
C = 262143, extra = 1 fills the array exactly and extra = 2 is two words over
(every term is even, so no plan is exactly one word over).
"""
import numpy as np

LIMIT_WORDS = 1 << 21
N_CHUNKS = 262143


def plan_words(plan):
    n_chunks = len(plan["q0"])
    return 4 + 2 * int(plan["n_out"]) + 4 * n_chunks + 2 + 2 * int(plan["roff"][-1])


def boundary_plan(extra=1, run=32):
    c = N_CHUNKS
    n_out = c + extra
    q0 = np.arange(c, dtype=np.int32)
    rs = np.clip(q0 - run // 2, 0, n_out - run).astype(np.int32)
    return dict(q0=q0, nq=np.ones(c, np.int32), roff=np.arange(c + 1, dtype=np.int32), rs=rs,
                rn=np.full(c, run, np.int32), q_base=0, n_out=n_out, n_f=n_out)
