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
