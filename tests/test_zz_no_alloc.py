"""The allocation-free likelihood call, for callers that may not allocate
device memory (a host framework owning the whole device budget, or a plugin
whose host forbids allocation on its hot path).

It must give what the allocating call gives, on two calls in a row (the second
call reuses the fixed scratch array the first one filled), and refuse sizes
whose scratch would not fit in that array. This file is collected last so that
a run stopping at the first failure has already run every other test.
"""
import numpy as np
import pytest

from vcfpop_gb300 import _lib as B
from vcfpop_gb300 import structure as S
from vcfpop_gb300 import synth

pytestmark = pytest.mark.gpu

REL = 1e-5  # the likelihood tolerance used by the parity tests


def _inputs(seed, N, L, K):
    import torch
    d = synth.fmodel(seed, N, L, 4, 0.1, 0.03)
    packed = S.pack2(d["G"])
    p = np.random.default_rng(seed).dirichlet([1.0, 1.0], size=(K, L)).astype(np.float32)
    g = torch.from_numpy(packed.view(np.int32)).cuda()
    f = torch.from_numpy(p.reshape(K, 2 * L)).cuda()
    return g, f


def _call(fn, g, f, N, L, K):
    import torch
    out = torch.full((N, K), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    B.check(fn(g.data_ptr(), N, L, f.data_ptr(), K, out.data_ptr(), None))
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_noalloc_matches_allocating_call_twice():
    lib = B.lib()
    for seed, (N, L, K) in [(1, (700, 3000, 5)), (2, (1500, 2200, 11))]:
        g, f = _inputs(seed, N, L, K)
        want = _call(lib.vp_loglik_packed2, g, f, N, L, K)
        got = _call(lib.vp_loglik_packed2_noalloc, g, f, N, L, K)
        assert np.isfinite(got).all()
        rel = np.abs(got - want) / np.abs(want)
        assert rel.max() < REL, rel.max()


def test_noalloc_replays_from_a_captured_graph():
    """After one uncaptured call, the call captured into a CUDA graph and
    replayed twice gives what the uncaptured call gives, bit for bit: its
    chain descriptor travels as a kernel parameter, so a replay reads nothing
    of the capturing call's host frame."""
    import ctypes as C
    import torch
    lib = B.lib()
    N, L, K = 700, 3000, 5
    g, f = _inputs(3, N, L, K)
    want = _call(lib.vp_loglik_packed2_noalloc, g, f, N, L, K)
    out = torch.full((N, K), float("nan"), dtype=torch.float64, device="cuda")
    graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.graph(graph, stream=side):
        B.check(lib.vp_loglik_packed2_noalloc(g.data_ptr(), N, L, f.data_ptr(), K, out.data_ptr(),
                                              C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    for _ in range(2):
        out.fill_(float("nan"))
        graph.replay()
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), want)


def test_noalloc_rejects_oversized_problems():
    import torch
    N, L, K = 20000, 400000, 12  # table + partial sums far beyond the fixed array
    dummy = torch.zeros(16, dtype=torch.int32, device="cuda")
    with pytest.raises(B.VpError, match="fixed array"):
        B.check(B.lib().vp_loglik_packed2_noalloc(dummy.data_ptr(), N, L, dummy.data_ptr(), K, dummy.data_ptr(), None))


def test_noalloc_at_the_size_limit():
    """The largest locus count whose scratch still fits the fixed array gives
    what the allocating call gives; one locus more is refused with VP_E_ARG.
    The limit is found by bisection on the call's own answer (a refused call
    does no device work), so the test follows the plan's alignment slack."""
    import torch
    lib = B.lib()
    N, K, L_hi = 64, 4, 600_000      # 600,000 loci need about 38 MB of scratch
    rng = np.random.default_rng(11)
    words = rng.integers(0, 2**32, size=(L_hi, (N + 15) // 16), dtype=np.uint64).astype(np.uint32)
    g = torch.from_numpy(words.view(np.int32)).cuda()
    p = rng.dirichlet([1.0, 1.0], size=(K, L_hi)).astype(np.float32)   # [K][L][2]
    out = torch.empty((N, K), dtype=torch.float64, device="cuda")

    def fits(L):
        f = torch.from_numpy(np.ascontiguousarray(p[:, :L].reshape(K, 2 * L))).cuda()
        torch.cuda.synchronize()
        rc = lib.vp_loglik_packed2_noalloc(g.data_ptr(), N, L, f.data_ptr(), K, out.data_ptr(), None)
        torch.cuda.synchronize()
        assert rc in (0, B.VP_E_ARG), rc
        return rc == 0, f

    lo, hi = 1, L_hi
    assert fits(lo)[0] and not fits(hi)[0]
    while hi - lo > 1:
        mid = (lo + hi) // 2
        if fits(mid)[0]:
            lo = mid
        else:
            hi = mid
    assert 400_000 < lo < L_hi
    _, f = fits(lo)
    want = _call(lib.vp_loglik_packed2, g, f, N, lo, K)
    for _ in range(2):
        got = _call(lib.vp_loglik_packed2_noalloc, g, f, N, lo, K)
        assert np.isfinite(got).all()
        assert (np.abs(got - want) / np.abs(want)).max() < REL
    _, f1 = fits(lo + 1)
    assert lib.vp_loglik_packed2_noalloc(g.data_ptr(), N, lo + 1, f1.data_ptr(), K, out.data_ptr(), None) == B.VP_E_ARG
    assert b"fixed array" in lib.vp_last_error()
