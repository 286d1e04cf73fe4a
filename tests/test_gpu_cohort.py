"""Cohorts: runs of different datasets (their own N, L, K and model) swept
together with one launch per kernel of the sweep.

Every member's blocks do the work of the chain's own launch, so a run gives
the same results bit for bit alone and in a cohort, whatever else shares its
launches, however long the other runs are, and whenever members join or
leave. Counter streams (the production path) and the reference streams are
both covered."""
import numpy as np
import pytest

from vcfpop_gb300 import _lib as B
from vcfpop_gb300 import structure as S
from vcfpop_gb300 import synth

pytestmark = pytest.mark.gpu


def _poly(seed, n=100, l=260, loc=False):
    rng = np.random.default_rng(seed)
    kw = dict(loc_ids=np.repeat(np.arange(4), n // 4), loc_alpha=1.0) if loc else {}
    return synth.fmodel(seed, n, l, 3, 0.08, 0.03, ploidy=np.array([2, 2, 4, 6] * (n // 4)),
                        n_alleles=rng.integers(2, 9, l), anc_alpha=1.0, **kw)


# (data, K, run parameters): packed and general layouts, small and large K
# (K = 20: two cluster groups of the likelihood and count kernels), the
# bit-plane count path (N >= 512), admixture with alpha, the location prior,
# the F model, the no-admixture burn-in, and runs of different lengths
RUNS = [
    (lambda: synth.fmodel(61, 300, 700, 3, 0.1, 0.05), 3, dict(admix=0, nadmburnin=0, nburnin=8, nreps=12)),
    (lambda: synth.fmodel(62, 600, 500, 4, 0.05, 0.02), 20, dict(admix=0, nadmburnin=0, nburnin=5, nreps=9)),
    (lambda: synth.fmodel(63, 150, 400, 3, 0.05, 0.02, admix_alpha=0.5), 4,
     dict(admix=1, nburnin=10, nreps=14, metrofreq=3)),
    (lambda: _poly(64, loc=True), 3, dict(admix=1, locpriori=1, nburnin=6, nreps=6)),
    (lambda: _poly(65), 2, dict(admix=0, fmodel=1, fsame=1, nadmburnin=4, nburnin=5, nreps=7)),
    (lambda: synth.fmodel(66, 40, 90, 2, 0.1, 0.05), 5, dict(admix=0, nadmburnin=3, nburnin=3, nreps=4,
                                                              nthinning=2)),
]


def _params(K, seed, rng, kw):
    kw = {dict(fmodel="f", fsame="singlef").get(k, k): v for k, v in kw.items()}
    return S.params(K, seed, rng=rng, writelnl=1, **kw)


def _results(ch):
    r = ch.result(final=True)
    return dict(rout=r["rout"], lnl=r["lnl"], Q=r["Q"], anc=r["ancestry"], freqm=r["freqm"], ni=ch.get("NI"),
                z=ch.get("Z"), mi=ch.get("MI"))


def _alone(data, rng, launches=None):
    out = []
    for (make, K, kw), d in zip(RUNS, data):
        ctx = S.Context(S.Dataset.from_synth(d))
        ch = S.Chain(ctx, _params(K, 900 + K, rng, kw))
        ch.run(1)                # one sweep alone: its launches (the graph's nodes)
        n0 = ctx.launches()
        ch.run(1)
        if launches is not None:
            launches.append(ctx.launches() - n0)
        S.finish([ch])
        out.append(_results(ch))
        ch.close()
        ctx.close()
    return out


def _same(a, b):
    for k in a:
        assert np.array_equal(a[k], b[k]), k


@pytest.fixture(scope="module")
def data():
    return [make() for make, _, _ in RUNS]


@pytest.mark.parametrize("rng", [B.VP_RNG_COUNTER, B.VP_RNG_REFERENCE])
def test_cohort_results_equal_runs_alone(data, rng):
    alone_launches = []
    want = _alone(data, rng, alone_launches)
    ctxs = [S.Context(S.Dataset.from_synth(d)) for d in data]
    chains = [S.Chain(x, _params(K, 900 + K, rng, kw)) for x, (_, K, kw) in zip(ctxs, RUNS)]
    co = S.Cohort()
    co.set(chains)
    longest = max(c.result()["nburnin"] + c.result()["nreps"] for c in chains)
    co.run(longest + 3)          # the short runs idle at their end
    for c in chains:
        S.finish([c])            # Arrange only: every sweep is done
    for c, w in zip(chains, want):
        _same(_results(c), w)
    # one launch per kernel variant in use, fewer than the runs launch alone
    # (these runs differ in model and cluster count, the least favourable mix)
    nq, per = co.launches()
    assert per < sum(alone_launches), (per, alone_launches)
    co.close()


def test_cohort_of_alike_runs_launches_each_kernel_once(data):
    """Runs of one model and cluster count on different datasets: one sweep
    of the whole cohort is as many launches as one run's sweep alone."""
    rng = B.VP_RNG_COUNTER
    sets = [synth.fmodel(70 + j, 100 + 37 * j, 300 + 91 * j, 3, 0.1, 0.05) for j in range(8)]
    ctxs = [S.Context(S.Dataset.from_synth(d)) for d in sets]
    kw = dict(admix=0, nadmburnin=0, nburnin=5, nreps=5)
    one = S.Chain(S.Context(S.Dataset.from_synth(sets[0])), _params(3, 5, rng, kw))
    one.run(1)
    n0 = one.ctx.launches()
    one.run(1)
    alone = one.ctx.launches() - n0
    chains = [S.Chain(x, _params(3, 100 + j, rng, kw)) for j, x in enumerate(ctxs)]
    co = S.Cohort()
    co.set(chains)
    co.run(10)
    assert co.launches()[1] == alone
    co.set([])
    co.close()


def test_cohort_members_join_and_leave(data):
    """Members change between sweeps: two runs start, two join after 3
    sweeps, one leaves (and finishes alone) after 6, the rest run to the end.
    Every run ends as it ends alone."""
    rng = B.VP_RNG_COUNTER
    want = _alone(data, rng)
    ctxs = [S.Context(S.Dataset.from_synth(d)) for d in data]
    chains = [S.Chain(x, _params(K, 900 + K, rng, kw)) for x, (_, K, kw) in zip(ctxs, RUNS)]
    co = S.Cohort()
    co.set(chains[:2])
    co.run(3)
    co.set(chains[:4])
    co.run(3)
    co.set(chains[1:4] + chains[4:])
    S.finish([chains[0]])        # runs its remaining sweeps on its own
    co.run(40)
    co.set([])
    for c in chains[1:]:
        S.finish([c])
    for c, w in zip(chains, want):
        _same(_results(c), w)
    co.close()


def test_cohort_guards(data):
    ctx = S.Context(S.Dataset.from_synth(data[0]))
    a = S.Chain(ctx, _params(3, 1, B.VP_RNG_COUNTER, dict(admix=0, nadmburnin=0, nburnin=4, nreps=4)))
    t = S.Chain(ctx, S.params(3, 2, form=B.VP_FORM_TC, admix=0, nadmburnin=0, nburnin=4, nreps=4))
    co = S.Cohort()
    with pytest.raises(B.VpError, match="plain-form"):
        co.set([t])
    co.set([a])
    with pytest.raises(B.VpError, match="cohort"):
        a.run(1)
    assert B.lib().vp_chain_destroy(a.h) == B.VP_E_STATE
    assert B.lib().vp_close(ctx.h) == B.VP_E_STATE
    co2 = S.Cohort()
    with pytest.raises(B.VpError, match="another cohort"):
        co2.set([a])
    co.run(8)
    co.set([])
    S.finish([a])
    assert np.isfinite(a.result(final=True)["rout"][3])
    co.close()
    co2.close()
