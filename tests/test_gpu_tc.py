"""The tensor-core contraction (tcgen05, TMA, TMEM) against a float64 reference,
and the batched split-BF16 K-sweep against the FP32 plain form."""
import ctypes as C

import numpy as np
import pytest

from vcfpop_gb300 import _lib as B
from vcfpop_gb300 import structure as S
from vcfpop_gb300 import synth

pytestmark = pytest.mark.gpu


def bf16_bits(x):
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return r.astype(np.uint16)


def bf16_val(b):
    return (b.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def gemm(A, B0, B1, BN, piece, splits=1, stages=2, mt=1, bk=64):
    M, K = A.shape
    N = B0.shape[0]
    D = np.zeros((splits, M, N), np.float32)
    B.check(B.lib().vp_debug_gemm_bf16(A.ctypes.data, B0.ctypes.data, None if B1 is None else B1.ctypes.data,
                                       M, N, K, BN, piece, splits, stages, mt, bk, D.ctypes.data))
    return D.astype(np.float64).sum(0)


# every tile shape compiled into the library, ragged M, split K, a K shorter
# than the pipeline
@pytest.mark.parametrize("M,N,K,BN,piece,nb,splits,stages,mt,bk", [
    (300, 384, 768, 192, 192, 2, 2, 2, 2, 64),
    (200, 576, 1024, 192, 192, 2, 3, 2, 2, 64),
    (640, 192, 1024, 192, 192, 1, 1, 3, 2, 64),
    (100, 192, 64, 192, 192, 1, 1, 3, 2, 64),
    (256, 576, 512, 288, 144, 2, 1, 2, 1, 64),
    (200, 576, 1024, 288, 144, 2, 3, 2, 1, 64),
    (128, 256, 64, 256, 256, 1, 1, 2, 1, 64),
    (384, 512, 640, 256, 256, 1, 1, 4, 1, 64),
    (300, 384, 800, 192, 192, 2, 3, 5, 2, 32),
])
def test_gemm_matches_float64(M, N, K, BN, piece, nb, splits, stages, mt, bk):
    rng = np.random.default_rng(M + N + K + bk)
    A = bf16_bits(rng.integers(0, 3, (M, K)).astype(np.float32))       # allele counts 0..2
    B0 = bf16_bits(rng.normal(0, 1, (N, K)).astype(np.float32))
    B1 = bf16_bits(rng.normal(0, 1e-3, (N, K)).astype(np.float32)) if nb == 2 else None
    D = gemm(A, B0, B1, BN, piece, splits, stages, mt, bk)
    Bsum = bf16_val(B0) + (bf16_val(B1) if B1 is not None else 0)
    ref = bf16_val(A) @ Bsum.T
    err = np.abs(D - ref).max() / max(1.0, np.abs(ref).max())
    assert err < 1e-5, err


E4M3 = {0: 0x00, 1: 0x38, 2: 0x40, 3: 0x44, 4: 0x48}   # small integers, exact in e4m3


@pytest.mark.parametrize("M,N,K,stages", [(300, 384, 1024, 4), (130, 192, 128, 2), (640, 576, 2048, 3)])
def test_gemm_e4m3_counts_exact(M, N, K, stages):
    """The count contraction's kind::f8f6f4 form: allele counts 0..2 times
    one-hot labels, summed exactly in FP32."""
    rng = np.random.default_rng(M * 7 + K)
    A = rng.integers(0, 3, (M, K))
    lab = rng.integers(0, N, K)
    Bm = np.zeros((N, K), np.int64)
    Bm[lab, np.arange(K)] = 1
    enc = np.vectorize(E4M3.get)
    A8 = np.ascontiguousarray(enc(A).astype(np.uint8))
    B8 = np.ascontiguousarray(enc(Bm).astype(np.uint8))
    D = np.zeros((M, N), np.float32)
    B.check(B.lib().vp_debug_gemm_e4m3(A8.ctypes.data, B8.ctypes.data, M, N, K, 192, 192, stages, 2, D.ctypes.data))
    assert np.array_equal(D.astype(np.int64), A @ Bm.T)


def test_batched_tc_sweep_matches_plain():
    """Same Ni, same Philox draws: the tensor-core sweep and the plain FP32 sweep
    give the same frequencies, near-identical likelihoods, and the same labels
    except at category boundaries."""
    d = synth.fmodel(51, 1000, 3000, 4, 0.05, 0.01)
    ds = S.Dataset.from_synth(d)
    ctx = S.Context(ds)
    Ks = [2, 3, 5]
    kw = dict(admix=0, nadmburnin=0, nburnin=50, nreps=50)
    plain = [S.Chain(ctx, S.params(K, 300 + K, **kw)) for K in Ks]
    tc = [S.Chain(ctx, S.params(K, 300 + K, form=B.VP_FORM_TC, **kw)) for K in Ks]
    S.run_chains(plain, 1)
    S.run_chains(tc, 1)
    assert B.lib().vp_tc_status(ctx.h) == 0
    for p, t in zip(plain, tc):
        assert np.array_equal(p.get("FREQ"), t.get("FREQ"))
        llp, llt = p.get("LL"), t.get("LL")
        rel = np.abs(llp - llt) / np.abs(llp)
        assert rel.max() < 1e-5, rel.max()
        zp, zt = p.get("Z"), t.get("Z")
        assert (zp != zt).mean() < 0.01
        if (zp == zt).all():
            assert np.array_equal(p.get("NI"), t.get("NI"))
            lp, lt = p.get("LNL")[0], t.get("LNL")[0]
            assert abs(lp - lt) <= 1e-6 * abs(lp)


def test_deferred_initial_counts_equal_plain():
    """A tensor-core chain leaves its initial counts to its batch; read before
    any batch exists they are computed on demand, and equal the plain chain's."""
    d = synth.fmodel(52, 600, 1200, 3, 0.05, 0.02)
    ds = S.Dataset.from_synth(d)
    ctx = S.Context(ds)
    kw = dict(admix=0, nadmburnin=0, nburnin=5, nreps=5)
    for K in (2, 4):
        p = S.Chain(ctx, S.params(K, 700 + K, **kw))
        t = S.Chain(ctx, S.params(K, 700 + K, form=B.VP_FORM_TC, **kw))
        assert np.array_equal(p.get("Z"), t.get("Z"))
        assert np.array_equal(p.get("NI"), t.get("NI"))
