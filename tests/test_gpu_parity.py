"""Step parity of the CUDA path against the oracle, reference random streams.

Each test feeds the same state to the oracle (the CPU restatement pinned to the
reference program) and to the library, runs one step on both, and compares:
  * integer allele counts Ni, Mi and labels initialised from integer draws: bit-exact
  * likelihoods: within 1e-5 relative
  * sampled labels: equal except where the draw falls within tolerance of a
    category boundary (counted, must be rare)
  * Dirichlet frequencies: within 4 float ulps (the device's log/pow may differ
    from glibc's in the last bit of a double)
"""
import numpy as np
import pytest

from vcfpop_gb300 import _lib as B
from vcfpop_gb300 import structure as S
from vcfpop_gb300 import synth

from . import orc

pytestmark = pytest.mark.gpu

REL = 1e-5


def _pair(d, packed=None, **kw):
    K = kw.pop("K")
    seed = kw.pop("seed", 12345)
    od = orc.Data(d)
    oc = orc.Chain(od, orc.params(K, seed, **kw))
    oc.init()
    ds = S.Dataset.from_synth(d, packed=packed)
    ctx = S.Context(ds)
    gp = S.params(K, seed, rng=B.VP_RNG_REFERENCE, **{k: v for k, v in _flags(kw).items()})
    gc = S.Chain(ctx, gp)
    return od, oc, ds, ctx, gc


def _flags(kw):
    m = dict(fmodel="f", fsame="singlef", epsr="stdr")
    return {m.get(k, k): v for k, v in kw.items()}


def _sync_state(oc, gc, names=("FREQ", "Q", "Z", "NI", "MI", "ALPHA")):
    for n in names:
        v = oc.get(n)
        if n == "MI":
            v = v.astype(np.int32)
        gc.set(n, v)


def _ulps(a, b):
    a = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    return np.abs(a - b)


def _c1_small():
    return synth.fmodel(21, 160, 700, 3, 0.1, 0.05)


def _adm_small():
    return synth.fmodel(22, 120, 500, 4, 0.05, 0.02, admix_alpha=0.5)


def _poly_small():
    rng = np.random.default_rng(3)
    ids = np.repeat(np.arange(4), 25)
    return synth.fmodel(23, 100, 260, 3, 0.08, 0.03, ploidy=np.array([2, 2, 4, 6] * 25),
                        n_alleles=rng.integers(2, 9, 260), anc_alpha=1.0, loc_ids=ids, loc_alpha=1.0)


@pytest.mark.parametrize("packed", [True, False])
def test_init_noadmix_exact(packed):
    od, oc, ds, ctx, gc = _pair(_c1_small(), packed=packed, K=3, admix=0, nadmburnin=0)
    assert np.array_equal(gc.get("Z"), oc.get("Z"))
    assert np.array_equal(gc.get("MI"), oc.get("MI").astype(np.int32))
    assert np.array_equal(gc.get("NI"), oc.get("NI"))
    assert np.array_equal(gc.get("FREQ"), oc.get("FREQ"))


@pytest.mark.parametrize("data", ["adm", "poly"])
def test_init_admix_exact(data):
    d = _adm_small() if data == "adm" else _poly_small()
    od, oc, ds, ctx, gc = _pair(d, K=4, admix=1)
    assert np.array_equal(gc.get("MI"), oc.get("MI").astype(np.int32))
    assert np.array_equal(gc.get("NI"), oc.get("NI"))


@pytest.mark.parametrize("data", ["c1", "poly"])
def test_update_p(data):
    d = _c1_small() if data == "c1" else _poly_small()
    od, oc, ds, ctx, gc = _pair(d, K=3, admix=0, nadmburnin=0)
    for m in range(3):
        oc.m = m
        gc.set("M", np.array([m], np.int32))
        _sync_state(oc, gc, ("NI",))
        oc.step("update_p")
        gc.step("UPDATEP")
        u = _ulps(gc.get("FREQ"), oc.get("FREQ"))
        assert u.max() <= 4, f"max ulps {u.max()}"
        assert (u == 0).mean() > 0.99


# Packed data: K = 1, 2, 6 and 13 take the FMA form's 1-, 2-, 6- and
# 14-column kernels, K = 3 and 10 the table form's 4 and 12 columns, K = 20
# two table groups of 16; general data: the table form's 4 and 12 columns
@pytest.mark.parametrize("packed,K", [(True, 1), (True, 2), (True, 3), (False, 3), (True, 6), (True, 10), (False, 10),
                                      (True, 13), (True, 20)])
def test_loglik_and_labels_noadmix(packed, K):
    od, oc, ds, ctx, gc = _pair(_c1_small(), packed=packed, K=K, admix=0, nadmburnin=0)
    oc.step("update_p")
    _sync_state(oc, gc)
    ll_o = oc.loglik().reshape(-1, K)
    gc.step("LOGLIK")
    ll_g = gc.get("LL").reshape(-1, K)
    rel = np.abs(ll_g - ll_o) / np.maximum(np.abs(ll_o), 1e-300)
    assert rel.max() < REL, rel.max()
    # labels drawn by PolyLog from the same uniforms
    oc.step("update_q_noadmix")
    gc.step("UPDATEQ")
    zo, zg = oc.get("Z"), gc.get("Z")
    flips = int((zo != zg).sum())
    assert flips <= max(1, len(zo) // 200), f"{flips} label flips"
    if flips == 0:
        lnl_o = orc.lib().orc_record_lnl(oc.h)
        lnl_g = gc.get("LNL")[0]
        assert abs(lnl_g - lnl_o) <= REL * abs(lnl_o)
        assert np.array_equal(gc.get("Q"), oc.get("Q"))


@pytest.mark.parametrize("data", ["c1", "poly"])
def test_update_z_noadmix_counts_exact(data):
    d = _c1_small() if data == "c1" else _poly_small()
    od, oc, ds, ctx, gc = _pair(d, K=3, admix=0, nadmburnin=0)
    rng = np.random.default_rng(0)
    z = rng.integers(0, 3, ds.N).astype(np.uint16)
    oc.set("Z", z)
    gc.set("Z", z)
    oc.step("update_z_noadmix")
    gc.set("M", np.array([0], np.int32))
    gc.step("UPDATEZ")
    assert np.array_equal(gc.get("NI"), oc.get("NI"))


@pytest.mark.parametrize("data", ["adm", "poly"])
def test_update_z_admix_counts_exact(data):
    d = _adm_small() if data == "adm" else _poly_small()
    od, oc, ds, ctx, gc = _pair(d, K=4, admix=1)
    for m in (0, 1, 7):
        oc.m = m
        gc.set("M", np.array([m], np.int32))
        oc.step("update_p")
        oc.step("update_q_admix")
        _sync_state(oc, gc)
        oc.step("update_z_admix")
        gc.step("UPDATEZ")
        assert np.array_equal(gc.get("NI"), oc.get("NI")), f"Ni differs at m={m}"
        assert np.array_equal(gc.get("MI"), oc.get("MI").astype(np.int32)), f"Mi differs at m={m}"
        # the admixture likelihood is fused into the per-copy draws
        lnl_o = orc.lib().orc_record_lnl(oc.h)
        lnl_g = _admix_lnl(gc)
        assert abs(lnl_g - lnl_o) <= REL * abs(lnl_o), (lnl_g, lnl_o)


def _admix_lnl(gc):
    # Record's likelihood for admixture chains is the sum of the per-copy
    # normalisers accumulated by UPDATEZ; the library exposes it through a
    # recorded trace, so run a writelnl record on a copy of the state instead.
    return gc._admix_lnl() if hasattr(gc, "_admix_lnl") else _lnl_via_trace(gc)


def _lnl_via_trace(gc):
    ctx = gc.ctx
    p = gc.p
    q = S.params(p.K, p.seed, rng=B.VP_RNG_REFERENCE, admix=1, writelnl=1, nburnin=100, nthinning=1)
    c2 = S.Chain(ctx, q)
    for n in ("FREQ", "Q"):
        c2.set(n, gc.get(n))
    c2.set("M", np.array([1], np.int32))  # a Gibbs sweep, not Metropolis
    c2.step("UPDATEZ")
    c2.step("RECORD")
    c2.step("NEXT")
    r = c2.result()
    return r["lnl"][0]


def test_update_q_admix_gibbs():
    od, oc, ds, ctx, gc = _pair(_adm_small(), K=4, admix=1)
    for m in (1, 3):
        oc.m = m
        gc.set("M", np.array([m], np.int32))
        _sync_state(oc, gc)
        oc.step("update_q_admix")
        gc.step("UPDATEQ")
        u = _ulps(gc.get("Q"), oc.get("Q"))
        assert u.max() <= 4 and (u == 0).mean() > 0.99


def test_update_q_metropolis():
    od, oc, ds, ctx, gc = _pair(_adm_small(), K=4, admix=1)
    oc.step("update_p")
    oc.step("update_q_admix")
    oc.m = 10
    gc.set("M", np.array([10], np.int32))
    _sync_state(oc, gc)
    oc.step("update_q_metro")
    gc.step("UPDATEQ")
    d_o, d_g = oc.get("METRO"), gc.get("METRO")
    scale = np.maximum(1.0, np.abs(d_o))
    assert (np.abs(d_g - d_o) / scale).max() < 1e-4
    u = _ulps(gc.get("Q"), oc.get("Q"))
    # a proposal accepted on one side only would differ by far more than 4 ulps
    assert (u > 4).sum() <= 2 * 4


def test_update_alpha():
    od, oc, ds, ctx, gc = _pair(_adm_small(), K=4, admix=1)
    oc.step("update_p")
    oc.step("update_q_admix")
    for m in (1, 2, 5):
        oc.m = m
        gc.set("M", np.array([m], np.int32))
        _sync_state(oc, gc)
        oc.step("update_alpha")
        gc.step("ALPHA")
        assert np.allclose(gc.get("ALPHA"), oc.get("ALPHA"), rtol=1e-12, atol=0)


@pytest.mark.parametrize("model", ["admix_f", "noadmix_f_single"])
def test_fmodel_steps(model):
    kw = dict(K=3, f=1, admix=1) if model == "admix_f" else dict(K=3, f=1, admix=0, nadmburnin=0, singlef=1)
    od, oc, ds, ctx, gc = _pair(_poly_small(), **kw)
    assert np.allclose(gc.get("FREQA"), oc.get("FREQA")[: ds.KT], rtol=0, atol=0)
    for m in range(4):
        oc.m = m
        gc.set("M", np.array([m], np.int32))
        _sync_state(oc, gc, ("NI",))
        ff = np.concatenate([oc.get("f"), oc.get("F")])
        gc.set("FF", ff)
        gc.set("FREQA", oc.get("FREQA")[: ds.KT])
        oc.step("update_p")
        gc.step("UPDATEP")
        _sync_state(oc, gc, ("FREQ",))
        oc.step("update_a")
        gc.step("UPDATEA")
        fa_o, fa_g = oc.get("FREQA")[: ds.KT], gc.get("FREQA")
        assert (_ulps(fa_g, fa_o) > 4).mean() < 0.01
        gc.set("FREQA", fa_o)
        oc.step("update_f")
        gc.step("UPDATEF")
        ff_g = gc.get("FF")
        assert np.allclose(ff_g, np.concatenate([oc.get("f"), oc.get("F")]), rtol=1e-9)


def _allele_copies(d, ds):
    """Copies of every allele at every kept locus, in the library's sorted
    locus order and allele offsets; typed copies per individual."""
    order = ds.order()
    G = d["G"][order]                                  # [L, N, v]
    k = d["k"][order].astype(np.int64)
    off = np.concatenate([[0], np.cumsum(k)[:-1]])
    cnt = np.zeros(int(k.sum()), np.int64)
    for a in range(int(k.max())):
        c = (G == a).sum(axis=(1, 2))
        sel = a < k
        cnt[off[sel] + a] = c[sel]
    typed = (G >= 0).sum(axis=(0, 2))
    return cnt, typed


@pytest.mark.parametrize("data,K", [("adm", 5), ("adm", 13), ("adm", 16), ("adm", 20), ("poly", 4), ("poly", 6), ("poly", 14)])
def test_update_z_admix_counter_streams_count_every_copy(data, K):
    """The counter-stream per-copy kernel (warp-reduced histogram: packed
    redux.sync bins for K * max alleles <= 32, one per lane (K = 16 on
    biallelic data is the largest), a shared atomic per copy above;
    exact-K templates up to 12, padded ones above; mixed-ploidy warps): summed
    over clusters, Ni holds every allele copy of the data exactly once and Mi
    every typed copy of each individual."""
    d = _adm_small() if data == "adm" else _poly_small()
    ds = S.Dataset.from_synth(d)
    ctx = S.Context(ds)
    gc = S.Chain(ctx, S.params(K, 777, admix=1))
    cnt, typed = _allele_copies(d, ds)
    rng = np.random.default_rng(K)
    for m in (0, 3):
        gc.set("M", np.array([m], np.int32))
        gc.step("UPDATEP")
        gc.set("Q", rng.dirichlet(np.full(K, 0.7), ds.N).astype(np.float32))
        gc.step("UPDATEZ")
        ni = gc.get("NI").astype(np.int64).reshape(K, ds.KT)
        mi = gc.get("MI").astype(np.int64).reshape(ds.N, K)
        assert np.array_equal(ni.sum(axis=0), cnt), f"allele copies lost or doubled at m={m}"
        assert np.array_equal(mi.sum(axis=1), typed), f"typed copies lost or doubled at m={m}"
        assert (ni >= 0).all() and ni.sum() > 0
