"""Parity at the shapes of the benchmark configurations themselves.

The step tests in test_gpu_parity.py run reduced shapes; these run the CUDA
path against the oracle on the data of each configuration at its own size:

  c1  N=200 diploids x L=2,000 SNPs, K=3 without admixture: one whole sweep
      step by step with the reference streams, and 10 whole runs of 1,000 +
      2,000 sweeps with the production counter streams (plain and
      tensor-core forms) against 10 oracle runs, within Monte-Carlo tolerance
  c2  N=2,000 x L=50,000, K=5 with admixture: one per-copy UpdateZ (Ni and Mi
      bit-exact), one Metropolis Q step and one alpha step
  c4  N=5,000 polyploids (2/4/6) x L=20,000 loci of 2-8 alleles at 20
      locations, K=8: one step of every kernel of the admixture + location
      prior model, and UpdateLocPriori's r/eta/gamma steps of the
      no-admixture location model

The bars are those of the reduced-shape tests: integer counts bit-exact,
likelihoods within 1e-5 relative, Dirichlet draws within 4 float ulps,
labels equal except at category boundaries (counted), double-precision
Metropolis-Hastings states within 1e-9 relative.
"""
import ctypes as C
import os

import numpy as np
import pytest

from vcfpop_gb300 import _lib as B
from vcfpop_gb300 import structure as S
from vcfpop_gb300 import workloads as W

from . import orc
from .test_gpu_chain import _membership, _perm_distance
from .test_gpu_parity import _admix_lnl, _flags, _sync_state, _ulps

pytestmark = pytest.mark.gpu

REL = 1e-5


@pytest.fixture(scope="module")
def c1():
    return W.c1(1)[0]


@pytest.fixture(scope="module")
def c2():
    return W.c2(2)[0]


@pytest.fixture(scope="module")
def c4():
    return W.c4(4)[0]


def _pair(d, K, seed=4242, **kw):
    od = orc.Data(d)
    oc = orc.Chain(od, orc.params(K, seed, **kw))
    oc.init()
    ds = S.Dataset.from_synth(d)
    ctx = S.Context(ds)
    gc = S.Chain(ctx, S.params(K, seed, rng=B.VP_RNG_REFERENCE, **_flags(kw)))
    return od, oc, ds, ctx, gc


LOCP_PARTS = ("ETA", "GAMMA", "ALPHALOCAL", "SUMALPHA")


def _locp_sizes(gc):
    K, S_ = gc.p.K, gc.ctx.ds.S
    return [1, K, S_ * K, S_ * K, S_]


def _locp_from_oracle(oc, gc):
    """The library's location-prior block (r, Eta, Gamma, AlphaLocal,
    SumAlpha) from the oracle's state; parts the oracle's model has no use
    for (it leaves them unallocated) keep the library's values."""
    cur = gc.get("LOCP")
    parts, o = [np.array([oc.r])], 1
    for name, n in zip(LOCP_PARTS, _locp_sizes(gc)[1:]):
        v = oc.get(name)
        parts.append(v if v.size == n else cur[o:o + n])
        o += n
    return np.concatenate(parts)


def _locp_close(oc, gc):
    got, o = gc.get("LOCP"), 1
    assert np.allclose(got[0], oc.r, rtol=1e-9, atol=1e-12), (got[0], oc.r)
    for name, n in zip(LOCP_PARTS, _locp_sizes(gc)[1:]):
        v = oc.get(name)
        if v.size == n:
            assert np.allclose(got[o:o + n], v, rtol=1e-9, atol=1e-12), (name, np.abs(got[o:o + n] - v).max())
        o += n


def _set_m(oc, gc, m):
    oc.m = m
    gc.set("M", np.array([m], np.int32))


def _freq_close(g, o):
    u = _ulps(g, o)
    assert u.max() <= 4, f"max ulps {u.max()}"
    assert (u == 0).mean() > 0.99


# ---------------------------------------------------------------- c1


def test_c1_one_sweep_step_by_step(c1):
    """Init, UpdateP, the likelihood and label draw, the counts and Record's
    likelihood of c1 at its full shape, reference streams, over two sweeps."""
    od, oc, ds, ctx, gc = _pair(c1, 3, admix=0, nadmburnin=0, nburnin=1000, nreps=2000)
    assert ds.N == 200
    assert np.array_equal(gc.get("Z"), oc.get("Z"))
    assert np.array_equal(gc.get("MI"), oc.get("MI").astype(np.int32))
    assert np.array_equal(gc.get("NI"), oc.get("NI"))
    for m in (0, 1):
        _set_m(oc, gc, m)
        _sync_state(oc, gc, ("NI",))
        oc.step("update_p")
        gc.step("UPDATEP")
        _freq_close(gc.get("FREQ"), oc.get("FREQ"))
        _sync_state(oc, gc, ("FREQ",))
        ll_o = oc.loglik().reshape(-1, 3)
        gc.step("LOGLIK")
        ll_g = gc.get("LL").reshape(-1, 3)
        assert (np.abs(ll_g - ll_o) / np.abs(ll_o)).max() < REL
        _set_m(oc, gc, m)
        oc.step("update_q_noadmix")
        gc.step("UPDATEQ")
        zo, zg = oc.get("Z"), gc.get("Z")
        assert int((zo != zg).sum()) <= 1, "label flips"
        gc.set("Z", zo)
        oc.step("update_z_noadmix")
        gc.step("UPDATEZ")
        assert np.array_equal(gc.get("NI"), oc.get("NI")), f"Ni differs at m={m}"
        lnl_o = orc.lib().orc_record_lnl(oc.h)
        if (zo == zg).all():
            assert abs(gc.get("LNL")[0] - lnl_o) <= REL * abs(lnl_o)


def _oracle_runs(d, K, seeds, **kw):
    """Whole oracle runs (init, every sweep, Arrange), one host thread per run."""
    od = orc.Data(d)
    cs = [orc.Chain(od, orc.params(K, s, **kw)) for s in seeds]
    arr = (C.c_void_p * len(cs))(*[c.h for c in cs])
    p = cs[0].p
    assert p.admix or p.locpriori or p.nadmburnin == 0, "whole runs here have no admixture burn-in"
    orc.lib().orc_sweep_many(arr, len(cs), p.nburnin + p.nreps, min(len(cs), os.cpu_count() or 1), 1)
    out = []
    for c in cs:
        orc.lib().orc_arrange(c.h)
        out.append(dict(rout=c.get("ROUT"), anc=c.field("MISUM").view(np.float64).copy()))
    return out


@pytest.fixture(scope="module")
def c1_oracle_runs(c1):
    return _oracle_runs(c1, 3, [1000 + s for s in range(10)], admix=0, nadmburnin=0, nburnin=1000, nreps=2000)


@pytest.mark.parametrize("form", ["plain", "tc"])
def test_c1_ten_whole_runs_match_oracle_statistically(c1, c1_oracle_runs, form):
    """c1 as specified (K=3, 1,000 burn-in + 2,000 sweeps), 10 seeds each:
    lnP(D) and the posterior membership of the best run agree with the
    oracle's within Monte-Carlo tolerance, for the plain form and for the
    tensor-core batch."""
    ds = S.Dataset.from_synth(c1)
    ctx = S.Context(ds)
    f = B.VP_FORM_TC if form == "tc" else B.VP_FORM_PLAIN
    cs = [S.Chain(ctx, S.params(3, 2000 + s, form=f, admix=0, nadmburnin=0, nburnin=1000, nreps=2000))
          for s in range(10)]
    S.finish(cs)
    if form == "tc":
        assert B.lib().vp_tc_status(ctx.h) == 0
    g = [c.result(final=True) for c in cs]
    lo = np.array([r["rout"][3] for r in c1_oracle_runs])
    lg = np.array([r["rout"][3] for r in g])
    spread = max(np.std(lo), np.std(lg), 1.0)
    assert abs(lo.max() - lg.max()) < 3 * spread + 1e-4 * abs(lo.max()), (lo, lg)
    assert abs(np.median(lo) - np.median(lg)) < 4 * spread + 1e-4 * abs(np.median(lo)), (lo, lg)
    pop = c1["pop"]
    bo = _membership(c1_oracle_runs[int(np.argmax(lo))]["anc"], pop, 3, 3)
    bg = _membership(g[int(np.argmax(lg))]["ancestry"], pop, 3, 3)
    assert _perm_distance(bo, bg) < 0.1


# ---------------------------------------------------------------- c2


def test_c2_admixture_steps(c2):
    """c2 at its full shape, reference streams: one per-copy UpdateZ (Ni and
    Mi bit-exact, Record's admixture likelihood within 1e-5), one Metropolis
    Q step and one alpha step."""
    od, oc, ds, ctx, gc = _pair(c2, 5, admix=1, inferalpha=1, nburnin=5000, nreps=10000)
    assert ds.N == 2000 and c2["G"].shape[0] == 50000   # L before the monomorphic filter
    assert np.array_equal(gc.get("MI"), oc.get("MI").astype(np.int32))
    assert np.array_equal(gc.get("NI"), oc.get("NI"))
    # UpdateZ at a Gibbs sweep, after the oracle's UpdateP and UpdateQ
    _set_m(oc, gc, 1)
    oc.step("update_p")
    oc.step("update_q_admix")
    _sync_state(oc, gc)
    oc.step("update_z_admix")
    gc.step("UPDATEZ")
    assert np.array_equal(gc.get("NI"), oc.get("NI"))
    assert np.array_equal(gc.get("MI"), oc.get("MI").astype(np.int32))
    lnl_o = orc.lib().orc_record_lnl(oc.h)
    assert abs(_admix_lnl(gc) - lnl_o) <= REL * abs(lnl_o)
    # Metropolis Q step (m = 10, a multiple of metrofreq)
    _set_m(oc, gc, 10)
    oc.step("update_p")
    _sync_state(oc, gc)
    oc.step("update_q_metro")
    gc.step("UPDATEQ")
    d_o, d_g = oc.get("METRO"), gc.get("METRO")
    assert (np.abs(d_g - d_o) / np.maximum(1.0, np.abs(d_o))).max() < 1e-4
    u = _ulps(gc.get("Q"), oc.get("Q"))
    assert (u > 4).sum() <= 2 * 5, "proposals accepted on one side only"
    # alpha
    _set_m(oc, gc, 11)
    _sync_state(oc, gc)
    oc.step("update_alpha")
    gc.step("ALPHA")
    assert np.allclose(gc.get("ALPHA"), oc.get("ALPHA"), rtol=1e-9, atol=0)


# ---------------------------------------------------------------- c4


def test_c4_every_step_of_the_location_prior_admixture_model(c4):
    """c4 at its full shape (mixed ploidy, multiallelic, 20 locations, K=8),
    reference streams: init, UpdateP, UpdateQ (Gibbs and Metropolis),
    UpdateLocPriori's r step, UpdateZ and the local alpha steps."""
    od, oc, ds, ctx, gc = _pair(c4, 8, admix=1, locpriori=1, nburnin=10000, nreps=10000)
    assert (ds.N, ds.S) == (5000, 20)
    assert np.array_equal(gc.get("MI"), oc.get("MI").astype(np.int32))
    assert np.array_equal(gc.get("NI"), oc.get("NI"))
    sync_locp = lambda: gc.set("LOCP", _locp_from_oracle(oc, gc))        # noqa: E731
    locp_close = lambda: _locp_close(oc, gc)                              # noqa: E731

    for m in (1, 10):
        _set_m(oc, gc, m)
        _sync_state(oc, gc, ("NI",))
        oc.step("update_p")
        gc.step("UPDATEP")
        _freq_close(gc.get("FREQ"), oc.get("FREQ"))
        _sync_state(oc, gc, ("FREQ", "Q", "MI", "ALPHA"))
        sync_locp()
        oc.step("update_q")
        gc.step("UPDATEQ")
        u = _ulps(gc.get("Q"), oc.get("Q"))
        if m % 10:
            assert u.max() <= 4 and (u == 0).mean() > 0.99
        else:
            d_o, d_g = oc.get("METRO"), gc.get("METRO")
            assert (np.abs(d_g - d_o) / np.maximum(1.0, np.abs(d_o))).max() < 1e-4
            assert (u > 4).sum() <= 2 * 8
        _sync_state(oc, gc, ("Q",))
        oc.step("update_locpriori")
        gc.step("LOCPRIORI")
        locp_close()
        oc.step("update_z_admix")
        gc.step("UPDATEZ")
        assert np.array_equal(gc.get("NI"), oc.get("NI")), f"Ni differs at m={m}"
        assert np.array_equal(gc.get("MI"), oc.get("MI").astype(np.int32)), f"Mi differs at m={m}"
        sync_locp()
        _sync_state(oc, gc, ("ALPHA",))
        oc.step("update_alpha")
        gc.step("ALPHA")
        assert np.allclose(gc.get("ALPHA"), oc.get("ALPHA"), rtol=1e-9, atol=0)
        locp_close()


@pytest.mark.parametrize("m", [3, 10])
def test_c4_update_locpriori_without_admixture(c4, m):
    """UpdateLocPriori (src/structure.cpp:1168-1255) of the no-admixture
    location model on c4's data: the Metropolis steps of r, eta and every
    location's gamma from the same state and the same reference stream, and
    at m = 10 the renormalisation of eta and gamma. The state is taken from
    the oracle after a few sweeps, so eta, gamma and the location counts Di
    are not at their initial values."""
    od = orc.Data(c4)
    oc = orc.Chain(od, orc.params(8, 77, admix=0, locpriori=1, nburnin=10000, nreps=10000))
    oc.init()
    for _ in range(3):
        orc.lib().orc_sweep(oc.h)
    ds = S.Dataset.from_synth(c4)
    ctx = S.Context(ds)
    gc = S.Chain(ctx, S.params(8, 77, rng=B.VP_RNG_REFERENCE, admix=0, locpriori=1, nburnin=10000, nreps=10000))
    before = _locp_from_oracle(oc, gc)
    gc.set("LOCP", before)
    gc.set("DI", oc.get("DI"))
    _set_m(oc, gc, m)
    oc.step("update_locpriori")
    gc.step("LOCPRIORI")
    _locp_close(oc, gc)
    assert not np.array_equal(_locp_from_oracle(oc, gc), before), "no step was accepted; nothing was compared"
