"""The serving loop (vp_server_*): a run's results do not depend on what else
runs beside it, admission honours the device-memory budget in arrival order,
and misuse fails with a status instead of hanging."""
import numpy as np
import pytest

from vcfpop_gb300 import _lib as B
from vcfpop_gb300 import structure as S
from vcfpop_gb300 import synth

pytestmark = pytest.mark.gpu


def _runs():
    """Datasets of different shapes and runs of every model family."""
    rng = np.random.default_rng(5)
    d_bi = synth.fmodel(61, 300, 1500, 3, 0.08, 0.02)
    d_adm = synth.fmodel(62, 240, 900, 4, 0.06, 0.02, admix_alpha=0.5)
    d_poly = synth.fmodel(63, 120, 300, 3, 0.08, 0.03, ploidy=np.array([2, 4, 6] * 40),
                          n_alleles=rng.integers(2, 7, 300), anc_alpha=1.0, loc_ids=np.repeat(np.arange(4), 30),
                          loc_alpha=1.0)
    ds_bi, ds_adm = S.Dataset.from_synth(d_bi), S.Dataset.from_synth(d_adm)
    ds_poly = S.Dataset.from_synth(d_poly, packed=False)
    runs = [
        (ds_bi, S.params(3, S.run_seed(1, 1), nburnin=30, nreps=60, nadmburnin=20)),
        (ds_bi, S.params(4, S.run_seed(1, 2), rng=B.VP_RNG_REFERENCE, nburnin=20, nreps=40, nadmburnin=0)),
        (ds_adm, S.params(4, S.run_seed(2, 1), admix=1, inferalpha=1, nburnin=30, nreps=50)),
        (ds_poly, S.params(3, S.run_seed(3, 1), admix=1, locpriori=1, nburnin=20, nreps=40)),
        (ds_poly, S.params(2, S.run_seed(3, 2), f=1, nburnin=20, nreps=40, nadmburnin=10)),
    ]
    return runs


def _collect(srv, rid):
    info = srv.wait(rid, 120.0)
    assert info["state"] == "done", info
    r = srv.result(rid)
    srv.release(rid)
    return r, info


def _same(a, b):
    for k in ("rout", "lnl", "Q", "ancestry", "freqm"):
        assert np.array_equal(a[k], b[k]), k


def test_results_alone_equal_results_in_mix():
    runs = _runs()
    alone = []
    srv = S.Server(max_active=1, chunk=7)
    for ds, p in runs:
        alone.append(_collect(srv, srv.submit(ds, p))[0])
    srv.close()
    srv = S.Server(max_active=8, chunk=5)
    ids = [srv.submit(ds, p) for ds, p in runs]
    for rid, ref in zip(ids, alone):
        _same(_collect(srv, rid)[0], ref)
    srv.close()


def test_server_run_equals_direct_chain():
    ds, p = _runs()[2]
    ctx = S.Context(ds)
    ch = S.Chain(ctx, p)
    S.finish([ch])
    direct = ch.result(final=True)
    ch.close()
    ctx.close()
    srv = S.Server()
    got = _collect(srv, srv.submit(ds, p))[0]
    srv.close()
    _same(got, direct)


def test_budget_admits_in_arrival_order_one_at_a_time():
    runs = _runs()[:3]
    probe = S.Server()
    sizes = []
    for ds, p in runs:
        rid = probe.submit(ds, p)
        sizes.append(probe.poll(rid)["device_bytes"])
        probe.wait(rid)
        probe.release(rid)
    probe.close()
    # room for the largest run only: runs must not overlap
    srv = S.Server(mem_budget=max(sizes) + 1, max_active=8, chunk=4)
    ids = [srv.submit(ds, p) for ds, p in runs]
    infos = []
    for rid in ids:
        infos.append(srv.wait(rid, 120.0))
        assert infos[-1]["state"] == "done"
        srv.release(rid)          # frees the budget for the next run
    for a, b in zip(infos, infos[1:]):
        assert b["t_start"] >= a["t_done"] - 1e-3, (a, b)
    srv.close()


def test_oversized_run_rejected_and_misuse_reports_state():
    ds, p = _runs()[0]
    srv = S.Server(mem_budget=1 << 16)
    with pytest.raises(B.VpError, match="budget"):
        srv.submit(ds, p)
    srv.close()
    srv = S.Server(max_active=1)
    long_p = S.params(3, S.run_seed(9, 1), nburnin=400, nreps=400, nadmburnin=0)
    a = srv.submit(ds, long_p)
    b = srv.submit(ds, p)
    assert srv.poll(b)["state"] in ("queued", "running", "done")
    with pytest.raises(B.VpError):
        srv.release(a) if srv.poll(a)["state"] != "done" else srv.release(10 ** 9)
    with pytest.raises(B.VpError, match="unknown"):
        srv.poll(10 ** 9)
    for rid in (a, b):
        assert srv.wait(rid, 120.0)["state"] == "done"
        srv.release(rid)
    srv.close()


def test_close_with_runs_in_flight():
    ds, p = _runs()[0]
    srv = S.Server(max_active=2)
    for j in range(4):
        srv.submit(ds, S.params(3, S.run_seed(4, j + 1), nburnin=200, nreps=200, nadmburnin=0))
    srv.close()                   # abandons the active runs, frees everything


def test_dataset_freed_before_its_run_ends():
    """A request holds its own reference to the dataset: the caller may free
    its handle right after vp_submit."""
    ds, p = _runs()[0]
    ctx = S.Context(ds)
    ch = S.Chain(ctx, p)
    S.finish([ch])
    direct = ch.result(final=True)
    ctx.close()
    d2 = S.Dataset.from_synth(synth.fmodel(61, 300, 1500, 3, 0.08, 0.02))
    srv = S.Server(max_active=1)
    rid = srv.submit(d2, p)
    B.lib().vp_dataset_free(d2.h)
    d2.h = None
    _same(_collect(srv, rid)[0], direct)
    srv.close()


def test_context_closed_before_its_chains():
    """vp_close destroys the chains still open on the context; a chain wrapper
    finalised after its context (as the collector may order a reference
    cycle) does not touch the freed context."""
    ds, p = _runs()[2]
    ctx = S.Context(ds)
    chains = [S.Chain(ctx, p) for _ in range(3)]
    chains[0].close()
    chains[1].run(5)
    ctx.close()
    for ch in chains:
        ch.close()
        assert ch.h is None
    ctx2 = S.Context(ds)          # the device is still usable
    ch = S.Chain(ctx2, p)
    ch.run(3)
    ch.close()
    ctx2.close()


def test_batched_cohorts_give_the_same_results_with_fewer_launches():
    """With batching (the default) the small runs of a mix sweep together in a
    cohort, one launch per kernel variant of the sweep for all of them: the
    results are those of every run on its own stream, bit for bit, with fewer
    kernel launches per run-sweep."""
    runs = _runs()
    # replicates with other seeds: runs of one sweep signature that merge
    runs += [(ds, S.params(p.K, p.seed + 17 * j, rng=p.rng, admix=p.admix, locpriori=p.locpriori, f=p.fmodel,
                           nburnin=p.nburnin, nreps=p.nreps, nadmburnin=p.nadmburnin))
             for j, (ds, p) in enumerate(runs[:1] * 3 + runs[2:3] * 3, start=1)]
    got = {}
    for batching in (False, True):
        srv = S.Server(max_active=8, chunk=6, batching=batching)
        ids = [srv.submit(ds, p) for ds, p in runs]
        got[batching] = [_collect(srv, rid)[0] for rid in ids]
        st = srv.stats()
        got[(batching, "lps")] = st["launches"] / st["run_sweeps"]
        srv.close()
    for a, b in zip(got[False], got[True]):
        _same(a, b)
    # runs of one model and cluster count (replicates) share a cohort and
    # merge every launch; the others sweep in cohorts of their own
    assert got[(True, "lps")] < 0.8 * got[(False, "lps")], (got[(True, "lps")], got[(False, "lps")])
