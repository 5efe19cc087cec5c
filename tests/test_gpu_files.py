"""The on-disk formats through the library (irc_fet_load_site,
irc_knn_save_site, irc_sort_save / irc_sort_load) against the numpy
restatement in oracle/io_oracle.py: identical values and bytes."""
import numpy as np
import pytest
import torch

from ironclust_gb300 import _lib, files
from oracle import io_oracle as IO

pytestmark = pytest.mark.gpu


def _fixture(tmp_path, n_loads=3, n_sites=5, n_pc=3, n_sites_spk=4, per_load=(700, 0, 1300), seed=0, tag="_fet_"):
    rng = np.random.default_rng(seed)
    tr, site = [], []
    for l in range(n_loads):
        n = per_load[l % len(per_load)]
        tr.append(rng.normal(0, 5, (n, n_sites_spk, n_pc)).astype(np.float32))
        site.append(rng.integers(0, n_sites, n))
    fs, cc = IO.write_fet_files(str(tmp_path / "rec"), tr, site, n_sites, tag)
    return fs, cc


TAPER = np.array([[1, 1, 1, 0], [1, 1, 0, 0], [1, 0, 0, 0]], bool)      # [nPc x nSites_spk]


@pytest.mark.parametrize("mask", [None, TAPER], ids=["all", "taper"])
@pytest.mark.parametrize("subset", [False, True])
def test_fet_load_site_matches_reference_reader(gpu, tmp_path, mask, subset):
    fs, cc = _fixture(tmp_path)
    rng = np.random.default_rng(1)
    for s in range(5):
        everyone = np.concatenate([load[s] for load in cc])
        vi = np.sort(rng.choice(everyone, size=max(1, len(everyone) // 3), replace=False)) if subset else None
        before, counts, sel, spikes = files.fet_selection(cc, s, vi)
        F = files.fet_load_site(fs, before, counts, 3, 4, mask, sel)
        ref = IO.load_fet_site(fs, cc, s, vi, 3, 4, mask)
        assert F.shape == ref.shape
        assert np.array_equal(F.cpu().numpy().view(np.int32), ref.view(np.int32))
        if vi is not None:
            assert np.array_equal(spikes, vi)


def test_fet_load_site_streams_large_blocks(gpu, tmp_path):
    """~46 MB of one site's records: more than one pinned staging buffer."""
    fs, cc = _fixture(tmp_path, n_loads=1, n_sites=2, n_pc=3, n_sites_spk=14, per_load=(500000,), seed=3)
    for s in range(2):
        before, counts, sel, _ = files.fet_selection(cc, s)
        F = files.fet_load_site(fs, before, counts, 3, 14)
        ref = IO.load_fet_site(fs, cc, s, None, 3, 14)
        assert np.array_equal(F.cpu().numpy(), ref)


def test_fet_load_site_errors(gpu, tmp_path):
    fs, cc = _fixture(tmp_path)
    before, counts, _, _ = files.fet_selection(cc, 1)
    with pytest.raises(_lib.IrcError):
        files.fet_load_site(fs, before, counts, 3, 4, None, np.array([0, int(counts.sum())]))
    with pytest.raises(_lib.IrcError):
        files.fet_load_site([str(tmp_path / "missing.irc")] * 3, before, counts, 3, 4)


def test_knn_save_site_write_and_append(gpu, tmp_path):
    rng = np.random.default_rng(4)
    nF, knn = 5000, 30
    viSpk = np.sort(rng.choice(10 ** 7, nF, replace=False)).astype(np.int64) + 1
    path = tmp_path / "rec_knn_3.irc"
    pages = []
    for page in range(3):
        n = 700 + 100 * page
        mi = rng.integers(1, nF + 1, (n, 20)).astype(np.int32)                 # 20 < knn: padded
        files.knn_save_site(path, torch.from_numpy(mi).cuda(), torch.from_numpy(viSpk).cuda(), knn, append=page > 0)
        pages.append(IO.knn_rows(mi, viSpk, knn))
    got = np.fromfile(path, np.int64)
    assert np.array_equal(got, np.concatenate(pages).reshape(-1))


def test_sort_save_load_roundtrip(gpu, tmp_path):
    rng = np.random.default_rng(5)
    n = 123457
    rho = rng.random(n).astype(np.float32)
    delta = rng.exponential(1, n).astype(np.float32)
    nneigh = rng.integers(1, n + 1, n).astype(np.int64)
    ordrho = rng.permutation(n).astype(np.int64) + 1
    t = lambda x: torch.from_numpy(x).cuda()
    path = tmp_path / "sort.irc"
    files.sort_save(path, t(rho), t(delta), t(nneigh), t(ordrho))
    assert path.read_bytes() == IO.sort_bytes(rho, delta, nneigh, ordrho)
    r, d, nn, od = files.sort_load(path, n)
    assert np.array_equal(r.cpu().numpy(), rho) and np.array_equal(d.cpu().numpy(), delta)
    assert np.array_equal(nn.cpu().numpy(), nneigh) and np.array_equal(od.cpu().numpy(), ordrho)
