"""Output reductions of WriteStructure on the device (vp_chain_divergence)
against the oracle's restatement of the reference loops (itself pinned to the
reference program's printed D block), on the same mean frequencies."""
import numpy as np
import pytest

from vcfpop_gb300 import structure as S
from vcfpop_gb300 import synth

from . import orc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("data,K", [("bi", 4), ("poly", 3), ("bi", 13)])
def test_device_divergence_matches_oracle(data, K):
    if data == "bi":
        d = synth.fmodel(71, 300, 2500, 4, 0.08, 0.02)
    else:
        rng = np.random.default_rng(7)
        d = synth.fmodel(72, 120, 400, 3, 0.08, 0.03, ploidy=np.array([2, 2, 4, 6] * 30),
                         n_alleles=rng.integers(2, 9, 400), anc_alpha=1.0, loc_ids=np.repeat(np.arange(3), 40),
                         loc_alpha=1.0)
    ds = S.Dataset.from_synth(d)
    ctx = S.Context(ds)
    ch = S.Chain(ctx, S.params(K, 4242, admix=1 if data == "poly" else 0, nadmburnin=0, nburnin=20, nreps=30))
    with pytest.raises(Exception, match="not finished"):
        ch.divergence()
    S.finish([ch])
    fm = ch.result(final=True)["freqm"]
    k_sorted = d["k"][ds.order()]
    want = orc.divergence(fm, k_sorted, K, per_locus=True)
    got = ch.divergence(per_locus=True)
    for key in ("H", "D", "Hl"):
        assert np.allclose(got[key], want[key], rtol=1e-12, atol=1e-14), key
    assert np.array_equal(np.diag(got["D"]), np.zeros(K))


NUMBER = __import__("re").compile(r"-?\d+\.\d+(?:e[-+]?\d+)?|nan")


def _poly_data(seed, locations=False):
    rng = np.random.default_rng(seed)
    kw = dict(loc_ids=np.repeat(np.arange(3), 30), loc_alpha=1.0) if locations else {}
    return synth.fmodel(seed, 90, 150, 3, 0.08, 0.03, ploidy=np.array([2, 2, 4, 6] * 22 + [2, 2]),
                        n_alleles=rng.integers(2, 9, 150), anc_alpha=1.0, **kw)


# every branch of WriteStructure's parameter block (alpha, per-cluster alpha,
# the location prior with and without admixture, F per cluster and single F)
# and the diversity table
WRITER_CASES = {
    "noadmix": (lambda: synth.fmodel(81, 150, 600, 3, 0.1, 0.05), 3, dict(admix=0, nadmburnin=0)),
    "admix_alpha": (lambda: synth.fmodel(82, 120, 500, 3, 0.05, 0.02, admix_alpha=0.5), 3, dict(admix=1)),
    "admix_diffalpha": (lambda: synth.fmodel(83, 120, 500, 3, 0.05, 0.02, admix_alpha=0.5), 3,
                        dict(admix=1, diffalpha=1)),
    "admix_locprior": (lambda: _poly_data(84, True), 3, dict(admix=1, locpriori=1)),
    "noadmix_locprior": (lambda: _poly_data(85, True), 2, dict(admix=0, locpriori=1)),
    "admix_f": (lambda: _poly_data(86), 3, dict(admix=1, fmodel=1)),
    "noadmix_singlef": (lambda: _poly_data(87), 2, dict(admix=0, fmodel=1, fsame=1, nadmburnin=4)),
}


@pytest.mark.parametrize("case", sorted(WRITER_CASES))
def test_result_files_equal_the_oracle_writer_on_the_same_state(case, tmp_path):
    """WriteStructure's numbers, not only its layout: one finished run's
    device state (parameter means, lnL trace, Q, ancestry, mean frequencies)
    is written by the library (vp_write_structure) and, loaded into an oracle
    chain, by the oracle's restatement of the reference writer
    (src/structure.cpp:86-377). The files are equal line for line and number
    for number; the divergence and diversity sums, formed on the device in
    another order, agree to 1e-12 relative."""
    make, K, kw = WRITER_CASES[case]
    d = make()
    ds = S.Dataset.from_synth(d)
    ctx = S.Context(ds)
    run = dict(kw, nburnin=12, nreps=21, nthinning=3, writelnl=1)
    gp = {dict(fmodel="f", fsame="singlef").get(k, k): v for k, v in run.items()}
    ch = S.Chain(ctx, S.params(K, 9191, **gp))
    S.finish([ch])
    r = ch.result(final=True)
    inds = [f"ind{i + 1}" for i in range(ds.N)]
    pops = [f"pop{s + 1}" for s in range(ds.S)]
    locs = [f"chr1_{l + 1}" for l in range(d["G"].shape[0])]
    ch.write(str(tmp_path / "gpu"), 1, 7, inds, pops, locs, decimal=15, diversity=True)

    od = orc.Data(d)
    oc = orc.Chain(od, orc.params(K, 9191, **run))
    oc.init()
    oc.set("ROUT", r["rout"])
    oc.set("Q", r["Q"])
    oc.set("FREQM", r["freqm"])
    oc.field("MISUM").view(np.float64)[:] = r["ancestry"]
    orc.lib().orc_nlnl(oc.h)[0] = len(r["lnl"])
    oc.set("LNL", r["lnl"])

    def arr(names):
        return (orc.C.c_char_p * len(names))(*[n.encode() for n in names])
    order = od.order(ds.L)
    keep = [arr(inds), arr(pops), arr([locs[o] for o in order])]
    assert orc.lib().orc_write_structure(oc.h, str(tmp_path / "orc").encode(), 1, 7, keep[0], keep[1], keep[2],
                                         15, 1) == 0
    files = [f"structure.k={K}_rep=1_id=7.txt", f"structure.k={K}_rep=1_id=7.lnl.txt"]
    for f in files:
        got = open(tmp_path / f"gpu.{f}", "rb").read().decode().split("\r\n")
        want = open(tmp_path / f"orc.{f}", "rb").read().decode().split("\r\n")
        assert len(got) == len(want), f
        for g, w in zip(got, want):
            assert NUMBER.sub("#", g) == NUMBER.sub("#", w), (f, g, w)
            for a, b in zip(NUMBER.findall(g), NUMBER.findall(w)):
                if a != b:
                    assert abs(float(a) - float(b)) <= 1e-12 * max(1.0, abs(float(b))), (f, g, w)
