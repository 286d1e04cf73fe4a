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
    (300, 432, 1024, 144, 144, 2, 2, 3, 2, 64),
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


def _lnp_fp64(ch):
    """lnP(D) of a no-admixture chain's current state in FP64: Record's sum
    (structure.cpp:1902-1938) is the sum of Ni x ln p over clusters, loci and
    alleles (pinned on the oracle by test_oracle_golden)."""
    ni, p = ch.get("NI").astype(np.float64), ch.get("FREQ").astype(np.float64)
    return float(np.sum(ni[ni > 0] * np.log(p[ni > 0])))


def test_lnp_relative_error_against_fp64_at_most_1e6():
    """Tolerance 1e-6 relative: the recorded lnP(D) of the batched split-bf16
    form and of the plain FP32 form against the FP64 evaluation of the same
    state, on every one of several recorded sweeps (thinning 1), for chains of
    K = 1..8 in one batch. The data follow the K-sweep benchmark's F-model (8
    populations, F = 0.03). The batch runs one split of all alleles (the
    longest FP32 accumulation of the likelihood contraction), so the recorded
    value must not come from that accumulation."""
    d = synth.fmodel(53, 3000, 20000, 8, 0.03, 0.01)
    ds = S.Dataset.from_synth(d)
    ctx = S.Context(ds)
    kw = dict(admix=0, nadmburnin=0, nburnin=0, nreps=50, nthinning=1, writelnl=1)
    Ks = list(range(1, 9))
    tc = [S.Chain(ctx, S.params(K, 400 + K, form=B.VP_FORM_TC, **kw)) for K in Ks]
    plain = [S.Chain(ctx, S.params(K, 500 + K, **kw)) for K in Ks]
    S.tc_configure(tc, splits=1)
    worst = 0.0
    for _ in range(4):
        S.run_chains(tc, 1)
        S.run_chains(plain, 1)
        for ch in tc + plain:
            want, got = _lnp_fp64(ch), ch.get("LNL")[0]
            worst = max(worst, abs(got - want) / abs(want))
            assert abs(got - want) <= 1e-6 * abs(want), (got, want, abs(got - want) / abs(want))
    assert worst < 1e-6
    assert B.lib().vp_tc_status(ctx.h) == 0


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


def test_plain_steps_on_a_batch_chain_equal_plain_chain():
    """A chain made for a tensor-core batch carves the plain form's likelihood
    table and partials only on its first plain-form step; stepped in the plain
    form it then follows a plain chain of the same seed bit for bit, also when
    its frequencies were set before that first step."""
    d = synth.fmodel(53, 500, 900, 3, 0.05, 0.02)
    ds = S.Dataset.from_synth(d)
    ctx = S.Context(ds)
    kw = dict(admix=0, nadmburnin=0, nburnin=5, nreps=5)
    for K in (3, 6):
        p = S.Chain(ctx, S.params(K, 900 + K, **kw))
        t = S.Chain(ctx, S.params(K, 900 + K, form=B.VP_FORM_TC, **kw))
        p.step("UPDATEP")
        t.set("FREQ", p.get("FREQ"))
        for name in ("LOGLIK", "UPDATEQ", "UPDATEZ", "UPDATEP", "LOGLIK"):
            p.step(name)
            t.step(name)
        for f in ("FREQ", "LL", "Z", "NI"):
            assert np.array_equal(p.get(f), t.get(f)), f
        t.close()
        p.close()
    ctx.close()


TILES = [(64, 2, 192, 192), (64, 2, 144, 144), (64, 1, 288, 144), (32, 2, 192, 192)]


def _tc_set(ctx, Ks, seed0):
    return [S.Chain(ctx, S.params(K, seed0 + j, form=B.VP_FORM_TC, admix=0, nadmburnin=0, nburnin=20, nreps=20))
            for j, K in enumerate(Ks)]


def _state(chains):
    return [{f: c.get(f) for f in ("Z", "NI", "FREQ", "LL", "LNL")} for c in chains]


def test_every_tc_configuration_gives_the_same_sweep():
    """Every compiled tile, pipeline depth and CTA order of both contractions,
    at one split count: with 64-allele stages the sweep is bit-identical to
    the default configuration's (the same FP32 accumulation order per
    output); with 32-allele stages the likelihoods agree to 1e-5 relative
    and the first sweep's frequencies exactly."""
    d = synth.fmodel(54, 700, 2000, 4, 0.05, 0.01)
    ds = S.Dataset.from_synth(d)
    ctx = S.Context(ds)
    Ks = [10] * 40          # 400 cluster rows, padded to 576: whole groups of 192 and of 288
    ref, ran = None, 0
    for bk, mt, cols, piece in TILES:
        for stages in range(2, 7):
            for gm in (0, 1):
                chains = _tc_set(ctx, Ks, 600)
                try:
                    S.tc_configure(chains, bk=bk, row_tiles=mt, cols=cols, piece=piece, stages=stages, splits=3,
                                   group_major=gm, count_stages=2 + (stages + gm) % 3, count_group_major=1 - gm)
                except B.VpError:
                    for c in chains:
                        c.close()
                    continue        # does not fit in shared memory
                cfg = S.tc_config(chains)
                assert (cfg["bk"], cfg["cols"], cfg["stages"], cfg["splits"], cfg["group_major"]) == \
                    (bk, cols, stages, 3, gm)
                S.run_chains(chains, 1)
                one = _state(chains)
                S.run_chains(chains, 1)
                two = _state(chains)
                assert B.lib().vp_tc_status(ctx.h) == 0
                for c in chains:
                    c.close()
                ran += 1
                if ref is None:
                    ref = (one, two)
                    continue
                for a, b in zip(ref[0], one):
                    assert np.array_equal(a["FREQ"], b["FREQ"])
                    if bk == 64:
                        for f in a:
                            assert np.array_equal(a[f], b[f]), (bk, cols, stages, gm, f)
                    else:
                        assert np.abs(a["LL"] - b["LL"]).max() <= 1e-5 * np.abs(a["LL"]).max()
                        assert (a["Z"] != b["Z"]).mean() < 1e-3
                if bk == 64:
                    for a, b in zip(ref[1], two):
                        for f in a:
                            assert np.array_equal(a[f], b[f]), (bk, cols, stages, gm, f)
    assert ran >= 12


@pytest.mark.parametrize("bk,splits,share", [(64, 2, 2), (64, 3, 1), (64, 7, 8), (32, 5, 2), (64, 1, 2)])
def test_sweep_by_allele_ranges_equals_one_pass(bk, splits, share):
    """The sweep by allele ranges (UpdateP of one range beside the likelihood
    contraction of the range before it) against UpdateP of every locus, then
    the whole contraction: the same state bit for bit after every sweep,
    including a last range shorter than the rest, an odd number of 32-allele
    k-blocks per range (ranges that do not start on a 64-allele boundary), and
    one split (no ranges), and caps of 1, 2 and 8 UpdateP blocks beside a
    contraction CTA. Both profiling modes time one span per sweep."""
    d = synth.fmodel(56, 300, 3103, 3, 0.05, 0.02)
    ds = S.Dataset.from_synth(d)
    if bk == 32:
        # a split count (near the one asked) with an odd number of k-blocks per split
        kblocks = (2 * ds.L + 63) // 64 * 2
        splits = next(s for s in (splits, splits - 2, splits + 2, splits + 4, splits + 6)
                      if (-(-kblocks // s)) % 2 == 1 and -(-kblocks // -(-kblocks // s)) == s)
    states = []
    for pipe in (share, 0):
        ctx = S.Context(ds)
        ctx.tc_pipeline(pipe)
        chains = _tc_set(ctx, [2, 3, 5, 10], 700)
        mt, cols, piece = next((m, c, p) for b, m, c, p in TILES if b == bk)
        S.tc_configure(chains, bk=bk, row_tiles=mt, cols=cols, piece=piece, stages=2, splits=splits)
        assert S.tc_config(chains)["splits"] == splits
        seq = []
        for mode in (1, 2, 0):
            B.check(B.lib().vp_prof_enable(ctx.h, mode))
            S.run_chains(chains, 1)
            if mode:
                ms, nl = C.c_double(), C.c_int32()
                B.check(B.lib().vp_prof_read(ctx.h, C.byref(ms), C.byref(nl)))
                assert nl.value == 1 and ms.value > 0
            seq.append(_state(chains))
        assert B.lib().vp_tc_status(ctx.h) == 0
        states.append(seq)
        for c in chains:
            c.close()
        ctx.close()
    for a_sweep, b_sweep in zip(*states):
        for a, b in zip(a_sweep, b_sweep):
            for f in a:
                assert np.array_equal(a[f], b[f]), (bk, splits, f)


def test_label_draw_does_not_depend_on_the_batch_around_a_chain():
    """The label draw runs by tiles of 32 individuals and groups of
    consecutive chains (at most 160 cluster rows per group). 40 chains of
    K = 10 alone (groups of 16 chains from the first) and behind 13 chains of
    K = 3 (39 rows first: every group boundary moves), at the same split
    count, reach the same labels, counts, frequencies and likelihoods bit for
    bit, and the same per-sweep likelihood sums to 1e-12."""
    d = synth.fmodel(57, 333, 1500, 4, 0.05, 0.02)
    ds = S.Dataset.from_synth(d)
    got = []
    for extra in (0, 13):
        ctx = S.Context(ds)
        front = [S.Chain(ctx, S.params(3, 2000 + j, form=B.VP_FORM_TC, admix=0, nadmburnin=0, nburnin=20, nreps=20))
                 for j in range(extra)]
        chains = front + _tc_set(ctx, [10] * 40, 1300)
        S.tc_configure(chains, splits=3)
        S.run_chains(chains, 3)
        assert B.lib().vp_tc_status(ctx.h) == 0
        got.append((_state(chains[extra:]), [c.get("LNL")[0] for c in chains[extra:]]))
        for c in chains:
            c.close()
        ctx.close()
    (a, la), (b, lb) = got
    for x, y in zip(a, b):
        for f in ("Z", "NI", "FREQ", "LL"):
            assert np.array_equal(x[f], y[f]), f
    assert np.allclose(la, lb, rtol=1e-12, atol=0)


def test_tune_keeps_chain_state_and_serves_later_batches(tmp_path, monkeypatch):
    """vp_tune times candidates on the batch without changing any chain's
    state, keeps the fastest for the batch, hands it to the next batch of the
    same shape, and appends it to the VP_TUNE_CACHE file."""
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("VP_TUNE_CACHE", str(cache))
    d = synth.fmodel(55, 900, 2500, 4, 0.05, 0.01)
    ds = S.Dataset.from_synth(d)
    ctx = S.Context(ds)
    Ks = [2, 3, 4, 5, 6, 7, 8] * 8
    chains = _tc_set(ctx, Ks, 800)
    S.run_chains(chains, 2)
    before = _state(chains)
    info = S.tune(chains, effort=2)
    after = _state(chains)
    for a, b in zip(before, after):
        for f in a:
            assert np.array_equal(a[f], b[f]), f
    assert info["candidates"] > 8
    for k in ("ms_likelihood", "ms_counts", "ms_likelihood_default", "ms_counts_default"):
        assert 0 < info[k] < 1e3, (k, info)
    assert info["ms_counts"] <= info["ms_counts_default"]
    cfg = S.tc_config(chains)
    for k in ("bk", "row_tiles", "cols", "piece", "stages", "splits", "group_major", "count_stages",
              "count_group_major"):
        assert cfg[k] == info[k], k
    S.run_chains(chains, 2)
    assert B.lib().vp_tc_status(ctx.h) == 0
    lines = cache.read_text().split("\n")
    assert len([ln for ln in lines if len(ln.split()) == 13]) >= 1
    ctx2 = S.Context(ds)
    other = _tc_set(ctx2, Ks, 900)
    cfg2 = S.tc_config(other)
    for k in ("bk", "cols", "stages", "splits", "group_major", "count_stages", "count_group_major"):
        assert cfg2[k] == cfg[k], k


def test_pipeline_wait_runs_out_with_an_error_status_and_the_device_stays_usable():
    """Failure detection without a fault: a contraction whose stage barriers
    never complete (they expect 16 bytes more than their copies bring) ends
    with a non-zero error status after its bounded waits, and the same
    contraction launched right after on the same device is exact."""
    st, after, err = C.c_int32(0), C.c_int32(-1), C.c_double(-1.0)
    B.check(B.lib().vp_debug_gemm_wait_timeout(C.byref(st), C.byref(after), C.byref(err)))
    assert st.value in (1, 2, 3), st.value
    assert after.value == 0
    assert err.value == 0.0


def test_tc_chain_runs_its_admixture_burn_in_in_the_plain_form():
    """The reference's default no-admixture run starts with nadmburnin
    sweeps drawn per allele copy (src/structure.cpp:460-462). A tensor-core
    chain runs those sweeps in the plain form, then joins the batch: through
    the burn-in its trace equals the plain chain's bit for bit (same kernels,
    same Philox draws), and at the first single-label sweep, whose state is
    the same, its likelihood agrees within 1e-5."""
    d = synth.fmodel(57, 800, 2500, 3, 0.05, 0.02)
    ds = S.Dataset.from_synth(d)
    ctx = S.Context(ds)
    kw = dict(admix=0, nadmburnin=12, nburnin=4, nreps=6, nthinning=1, writelnl=1)
    Ks = [1, 2, 4]
    plain = [S.Chain(ctx, S.params(K, 700 + K, **kw)) for K in Ks]
    tc = [S.Chain(ctx, S.params(K, 700 + K, form=B.VP_FORM_TC, **kw)) for K in Ks]
    S.finish(plain)
    S.finish(tc)
    assert B.lib().vp_tc_status(ctx.h) == 0
    for p, t in zip(plain, tc):
        rp, rt = p.result(final=True), t.result(final=True)
        assert len(rp["lnl"]) == len(rt["lnl"]) == 12 + 4 + 6
        assert np.array_equal(rp["lnl"][:12], rt["lnl"][:12])
        assert abs(rp["lnl"][12] - rt["lnl"][12]) <= 1e-5 * abs(rp["lnl"][12])
        assert np.isfinite(rt["lnl"]).all() and np.isfinite(rt["rout"][:4]).all()
        assert rt["nr"] == 6


def test_tc_chains_in_burn_in_refuse_the_tuner():
    """The batch only holds chains past their admixture burn-in."""
    d = synth.fmodel(58, 300, 800, 2, 0.05, 0.02)
    ctx = S.Context(S.Dataset.from_synth(d))
    tc = [S.Chain(ctx, S.params(K, 70 + K, form=B.VP_FORM_TC, admix=0, nadmburnin=3, nburnin=2, nreps=2))
          for K in (2, 3)]
    with pytest.raises(B.VpError, match="admixture burn-in"):
        S.tune(tc, 0)
    S.run_chains(tc, 3)
    S.tune(tc, 0)
    S.finish(tc)
    assert all(np.isfinite(c.result(final=True)["rout"][3]) for c in tc)
