"""Edge cases of the CUDA path against the oracle, reference random streams:
tiny and ragged shapes (one individual, a handful of loci, counts that are not
multiples of a warp or a block), an individual without a single typed call, a
locus typed in one individual only, and the largest cluster counts (padded
kernel templates, several cluster groups).

Traces are compared as in the whole-chain tests: the recorded likelihoods agree
to 1e-5 relative until a last-bit difference of a device log flips a label;
counts are bit-exact.
"""
import numpy as np
import pytest

from vcfpop_gb300 import _lib as B
from vcfpop_gb300 import structure as S
from vcfpop_gb300 import synth

from . import orc

pytestmark = pytest.mark.gpu

REL = 1e-5


def _trace_pair(d, K, seed, packed=None, **kw):
    od = orc.Data(d)
    oc = orc.Chain(od, orc.params(K, seed, **kw))
    orc.lib().orc_run(oc.h)
    o = dict(lnl=oc.get("LNL"), rout=oc.get("ROUT"))
    ds = S.Dataset.from_synth(d, packed=packed)
    ctx = S.Context(ds)
    c = S.Chain(ctx, S.params(K, seed, rng=B.VP_RNG_REFERENCE, **kw))
    S.finish([c])
    g = c.result(final=True)
    c.close()
    ctx.close()
    return o, g, ds


def _check_trace(o, g, n_first):
    assert len(g["lnl"]) == len(o["lnl"])
    assert np.isfinite(g["lnl"]).all()
    rel = np.abs(g["lnl"] - o["lnl"]) / np.abs(o["lnl"])
    assert rel[:n_first].max() < REL, rel


# (individuals, loci drawn, packed 2-bit store, admixture): one individual,
# two, a warp plus one, a block plus one, and widths that leave ragged words
SHAPES = [(1, 60, True, 0), (2, 9, False, 0), (33, 3, True, 0), (33, 3, False, 1), (257, 5, True, 1),
          (31, 130, False, 1), (129, 17, True, 0)]


@pytest.mark.parametrize("n,l,packed,admix", SHAPES)
def test_tiny_and_ragged_shapes_follow_oracle_trace(n, l, packed, admix):
    d = synth.fmodel(40 + n + l, n, l, 2, 0.1, 0.05, admix_alpha=0.5 if admix else None)
    kw = dict(admix=admix, nadmburnin=0 if not admix else 2, nburnin=3, nreps=3, nthinning=1, writelnl=1)
    o, g, ds = _trace_pair(d, 2, 7 + n, packed=packed, **kw)
    assert ds.N == n
    _check_trace(o, g, 3)


def _with_untyped(d, ind, loc):
    """Every call of individual `ind` missing; locus `loc` typed in one
    individual only (a heterozygote, so that it stays polymorphic)."""
    G = d["G"].copy()
    G[:, ind, :] = -1
    G[loc, :, :] = -1
    keep = (ind + 1) % G.shape[1]
    G[loc, keep, :] = -1
    G[loc, keep, 0], G[loc, keep, 1] = 0, 1
    return dict(d, G=G)


@pytest.mark.parametrize("admix", [0, 1])
def test_individual_without_typed_calls(admix):
    d = _with_untyped(synth.fmodel(51, 90, 300, 3, 0.08, 0.03, admix_alpha=0.5 if admix else None), 17, 5)
    kw = dict(admix=admix, nadmburnin=0 if not admix else 2, nburnin=3, nreps=3, nthinning=1, writelnl=1)
    o, g, ds = _trace_pair(d, 3, 2024, packed=False, **kw)
    _check_trace(o, g, 3)
    q = g["ancestry"].reshape(ds.N, 3)
    assert np.isfinite(q).all()
    assert np.allclose(q.sum(axis=1), 1.0, atol=1e-6)


def _pair_steps(d, K, seed=99, **kw):
    od = orc.Data(d)
    oc = orc.Chain(od, orc.params(K, seed, **kw))
    oc.init()
    ds = S.Dataset.from_synth(d)
    ctx = S.Context(ds)
    gc = S.Chain(ctx, S.params(K, seed, rng=B.VP_RNG_REFERENCE, **kw))
    return oc, ds, ctx, gc


def _sync(oc, gc, names):
    for n in names:
        v = oc.get(n)
        gc.set(n, v.astype(np.int32) if n == "MI" else v)


@pytest.mark.parametrize("K", [33, 64])
def test_largest_k_admixture_counts_exact(K):
    """The padded 64-cluster template of the per-copy label kernel (reference
    streams): Ni and Mi bit-exact, initialisation included."""
    d = synth.fmodel(52, 64, 160, 4, 0.05, 0.02, admix_alpha=0.5)
    oc, ds, ctx, gc = _pair_steps(d, K, admix=1)
    assert np.array_equal(gc.get("NI"), oc.get("NI"))
    assert np.array_equal(gc.get("MI"), oc.get("MI").astype(np.int32))
    for m in (0, 1):
        oc.m = m
        gc.set("M", np.array([m], np.int32))
        oc.step("update_p")
        oc.step("update_q_admix")
        _sync(oc, gc, ("FREQ", "Q", "Z", "NI", "MI", "ALPHA"))
        oc.step("update_z_admix")
        gc.step("UPDATEZ")
        assert np.array_equal(gc.get("NI"), oc.get("NI")), f"Ni differs at m={m}"
        assert np.array_equal(gc.get("MI"), oc.get("MI").astype(np.int32)), f"Mi differs at m={m}"


@pytest.mark.parametrize("packed", [True, False])
def test_largest_k_noadmix_likelihood_and_counts(packed):
    """K = 64: four cluster groups of 16 in the likelihood and count kernels."""
    K = 64
    d = synth.fmodel(53, 200, 400, 3, 0.1, 0.05)
    od = orc.Data(d)
    oc = orc.Chain(od, orc.params(K, 5, admix=0, nadmburnin=0))
    oc.init()
    ds = S.Dataset.from_synth(d, packed=packed)
    ctx = S.Context(ds)
    gc = S.Chain(ctx, S.params(K, 5, rng=B.VP_RNG_REFERENCE, admix=0, nadmburnin=0))
    assert np.array_equal(gc.get("NI"), oc.get("NI"))
    oc.step("update_p")
    _sync(oc, gc, ("FREQ", "Q", "Z", "NI", "MI", "ALPHA"))
    ll_o = oc.loglik().reshape(-1, K)
    gc.step("LOGLIK")
    ll_g = gc.get("LL").reshape(-1, K)
    rel = np.abs(ll_g - ll_o) / np.maximum(np.abs(ll_o), 1e-300)
    assert rel.max() < REL, rel.max()
    z = np.random.default_rng(1).integers(0, K, ds.N).astype(np.uint16)
    oc.set("Z", z)
    gc.set("Z", z)
    oc.step("update_z_noadmix")
    gc.set("M", np.array([0], np.int32))
    gc.step("UPDATEZ")
    assert np.array_equal(gc.get("NI"), oc.get("NI"))


def test_k_out_of_range_rejected():
    d = synth.fmodel(54, 40, 50, 2, 0.1, 0.0)
    ds = S.Dataset.from_synth(d)
    ctx = S.Context(ds)
    for K in (0, 65):
        with pytest.raises(B.VpError, match="K must be"):
            S.Chain(ctx, S.params(K, 1))
    ctx.close()


def test_no_step_past_the_end_of_the_run():
    """A caller driving its own loop is stopped at the end of the run: the
    trace is sized for nburnin + nreps sweeps, so a further Record or sweep
    index would write beyond it. The sweep index may not be set outside the
    run either."""
    d = synth.fmodel(71, 40, 30, 2, 0.1, 0.05)
    ds = S.Dataset.from_synth(d)
    ctx = S.Context(ds)
    c = S.Chain(ctx, S.params(2, 5, admix=0, nadmburnin=0, nburnin=2, nreps=2, nthinning=1, writelnl=1))
    S.finish([c])
    assert int(c.get("M")[0]) == 4
    for step in ("RECORD", "NEXT", "UPDATEP"):
        with pytest.raises(B.VpError, match="is over"):
            c.step(step)
    with pytest.raises(B.VpError, match="outside the run"):
        c.set("M", np.array([5], np.int32))
    with pytest.raises(B.VpError, match="outside the run"):
        c.set("M", np.array([-1], np.int32))
    r = c.result(final=True)
    assert len(r["lnl"]) == 4 and np.isfinite(r["lnl"]).all()
    # rewinding inside the run is allowed; repeated Records at one sweep
    # index stop at the trace's capacity (ceil(2/1) + ceil(2/1) + 2 records)
    c.set("M", np.array([3], np.int32))
    for _ in range(4):
        c.step("RECORD")
    assert len(c.result(final=True)["lnl"]) == 6
    c.step("NEXT")
    with pytest.raises(B.VpError, match="is over"):
        c.step("NEXT")
