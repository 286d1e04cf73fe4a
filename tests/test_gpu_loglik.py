"""The standalone likelihood call against a float64 restatement of
UpdateQNoAdmix's likelihood sum (sum over loci and copies of ln p)."""
import ctypes as C

import numpy as np
import pytest

from vcfpop_gb300 import _lib as B
from vcfpop_gb300 import structure as S
from vcfpop_gb300 import synth

pytestmark = pytest.mark.gpu


def loglik_ref(G, freq):
    """float64: LL[i,k] = sum_l c0*ln p0 + c1*ln p1 (missing calls add nothing)."""
    L, N, _ = G.shape
    K = freq.shape[0]
    typed = G[:, :, 0] >= 0
    c1 = np.where(typed, G[:, :, 0].astype(np.int64) + G[:, :, 1], 0).astype(np.float64)  # [L, N]
    c0 = np.where(typed, 2 - c1, 0.0)
    lp = np.log(freq.astype(np.float64).reshape(K, L, 2))
    return c0.T @ lp[:, :, 0].T + c1.T @ lp[:, :, 1].T  # [N, K]


@pytest.mark.parametrize("N,L,K", [(300, 1000, 3), (1000, 4000, 7), (2048, 2500, 12)])
def test_loglik_packed2_matches_float64(N, L, K):
    import torch
    d = synth.fmodel(N + L + K, N, L, 4, 0.1, 0.03)
    packed = S.pack2(d["G"])
    rng = np.random.default_rng(K)
    p = rng.dirichlet([1.0, 1.0], size=(K, L)).astype(np.float32)  # [K, L, 2]
    freq = p.reshape(K, 2 * L)
    g = torch.from_numpy(packed.view(np.int32)).cuda()
    f = torch.from_numpy(freq).cuda()
    out = torch.zeros((N, K), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    B.check(B.lib().vp_loglik_packed2(g.data_ptr(), N, L, f.data_ptr(), K, out.data_ptr(), None))
    torch.cuda.synchronize()
    ref = loglik_ref(d["G"], freq)
    rel = np.abs(out.cpu().numpy() - ref) / np.abs(ref)
    assert rel.max() < 1e-5, rel.max()


def _loglik_device(G, freq, N, L, K):
    import torch
    packed = S.pack2(G)
    g = torch.from_numpy(packed.view(np.int32)).cuda()
    f = torch.from_numpy(freq).cuda()
    out = torch.full((N, K), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    B.check(B.lib().vp_loglik_packed2(g.data_ptr(), N, L, f.data_ptr(), K, out.data_ptr(), None))
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("N", [5, 701, 5003])
def test_loglik_packed2_every_cluster_count(N):
    """Every K from 1 to 17 against float64: the FMA form (K = 1, 2, 5, 6, 13,
    14: 1, 2, 6 or 14 columns, 16, 4 or 2 individuals per thread) and the
    table form (the other K, 4 to 16 columns, two groups at K = 17);
    N below one genotype word, N with a partial last word, and N spanning
    several CTA columns of every instantiation."""
    L = 900 if N > 1000 else 1500
    d = synth.fmodel(N + 17, N, L, 3, 0.1, 0.05)
    rng = np.random.default_rng(N)
    for K in range(1, 18):
        p = rng.dirichlet([0.7, 0.7], size=(K, L)).astype(np.float32)
        p = np.maximum(p, 1e-6)
        p /= p.sum(axis=2, keepdims=True)
        freq = np.ascontiguousarray(p.reshape(K, 2 * L))
        got = _loglik_device(d["G"], freq, N, L, K)
        ref = loglik_ref(d["G"], freq)
        assert np.isfinite(got).all(), K
        rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1.0)
        assert rel.max() < 1e-5, (K, rel.max())
