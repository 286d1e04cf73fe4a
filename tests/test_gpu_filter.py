"""The -f_* locus filter on the device (vp_locus_filter_pack2) against the
oracle's restatement of CalcDiversity / MarkerDiversity, which is pinned to
the loci the reference program kept (test_oracle_locus_filter_matches_reference)."""
import numpy as np
import pytest

from vcfpop_gb300 import structure as S
from vcfpop_gb300 import synth

from . import orc

pytestmark = pytest.mark.gpu


def _orc_filter(f):
    o = orc.LocusFilter()
    for name, _ in orc.LocusFilter._fields_:
        setattr(o, name, getattr(f, name))
    return o


def _compare(packed, N, f):
    keep, stats = S.locus_filter(packed, N, f)
    okeep, ostats = orc.locus_filter_pack2(packed, N, _orc_filter(f))
    assert np.array_equal(keep, okeep)
    # every statistic bit for bit but Shannon's I, whose log may differ in the last place
    both = ~np.isnan(ostats)
    assert np.array_equal(np.isnan(stats), np.isnan(ostats))
    assert np.array_equal(stats[:, :8][both[:, :8]], ostats[:, :8][both[:, :8]])
    assert np.allclose(stats[:, 8][both[:, 8]], ostats[:, 8][both[:, 8]], rtol=1e-6)
    # the HWE p-value: logs of the G statistic and the device's erf may differ
    # in the last place
    assert np.allclose(stats[:, 9][both[:, 9]], ostats[:, 9][both[:, 9]], rtol=1e-5, atol=1e-12)
    return keep


def test_golden_filter_case_on_device():
    d = synth.fmodel(1, 200, 2000, 3, 0.1, 0.05)
    f = S.locus_filter_spec(bmaf=(0.15, 0.5), ptype=(0.96, 1.0), ho=(0.1, 0.6))
    keep = _compare(S.pack2(d["G"]), 200, f)
    assert 0 < keep.sum() < 2000


@pytest.mark.parametrize("single", [True, False])
def test_every_window_with_edge_loci(single):
    d = synth.fmodel(91, 333, 3000, 4, 0.05, 0.05)
    G = d["G"].copy()
    G[:20] = -1                     # no call typed
    G[20:40] = 0                    # monomorphic
    G[40:60, :, :] = np.where(G[40:60] >= 0, 1, -1)   # monomorphic in the other allele
    G[60:80, 5:] = -1               # almost nothing typed
    packed = S.pack2(G)
    windows = [dict(), dict(k=(2, 2)), dict(n=(300, 333)), dict(he=(0.1, 0.45)), dict(pic=(0.05, 0.3)),
               dict(ae=(1.2, 1.9)), dict(I=(0.2, 0.6)), dict(pval=(0.05, 1.0)),
               dict(bmaf=(0.05, 0.5), ptype=(0.9, 1.0), ho=(0.0, 0.5), pval=(1e-4, 1.0))]
    for w in windows:
        keep = _compare(packed, 333, S.locus_filter_spec(single=single, **w))
        assert not keep[:20].any()


def _compare_general(G, k, f, table=None):
    keep, stats = S.locus_filter_general(G, k, f, table=table)
    okeep, ostats = orc.locus_filter_general(G, k, _orc_filter(f), table=table)
    assert np.array_equal(keep, okeep)
    both = ~np.isnan(ostats)
    assert np.array_equal(np.isnan(stats), np.isnan(ostats))
    assert np.array_equal(stats[:, :8][both[:, :8]], ostats[:, :8][both[:, :8]])
    assert np.allclose(stats[:, 8][both[:, 8]], ostats[:, 8][both[:, 8]], rtol=1e-6)
    # the HWE p-value: its G statistic's logs and the tail function may differ
    # in the last places between the device and the host
    assert np.allclose(stats[:, 9][both[:, 9]], ostats[:, 9][both[:, 9]], rtol=1e-5, atol=1e-12)
    return keep, stats


@pytest.mark.parametrize("single", [1, 0])
def test_general_statistics_on_device_equal_the_oracle(single):
    """vp_locus_filter_general against the oracle, which is pinned to the
    loci the reference program kept (test_oracle_general_locus_filter_matches_
    reference): ploidy 2/4/6 with 2-8 alleles (mixed ploidy: no HWE test),
    diploid data with 2-6 alleles (the HWE test with allele collapsing and
    the chi-square tail of 1 to 15 degrees of freedom), tetraploid data, a
    table order taken from other calls, and every window at once."""
    rng = np.random.default_rng(20 + single)
    poly = synth.fmodel(8, 160, 400, 3, 0.08, 0.03, ploidy=np.array([2, 2, 4, 6] * 40),
                        n_alleles=rng.integers(2, 9, 400), anc_alpha=1.0)
    dip = synth.fmodel(9, 300, 400, 3, 0.05, 0.03, n_alleles=rng.integers(2, 7, 400), anc_alpha=1.0)
    tet = synth.fmodel(10, 200, 300, 2, 0.05, 0.02, ploidy=np.full(200, 4), n_alleles=rng.integers(2, 5, 300),
                       anc_alpha=1.0)
    for d in (poly, dip, tet):
        f = S.locus_filter_spec(single=bool(single))
        _, st = _compare_general(d["G"], d["k"], f)
    # the diploid set has defined p-values over several degrees of freedom
    _, st = _compare_general(dip["G"], dip["k"], S.locus_filter_spec(single=bool(single)))
    assert np.isfinite(st[:, 9]).sum() > 100
    # windows on every statistic
    f = S.locus_filter_spec(single=bool(single), k=(3, 7), he=(0.3, 0.8), ho=(0.2, 0.9), pic=(0.2, 0.8),
                            ae=(1.5, 5), I=(0.5, 2), ptype=(0.9, 1), n=(100, 300), bmaf=(0.05, 0.5), pval=(0.01, 1))
    keep, _ = _compare_general(dip["G"], dip["k"], f)
    assert 0 < keep.sum() < len(keep)
    # the genotype tables ordered by other calls (as the calls before a genotype filter)
    G2 = dip["G"].copy()
    G2[rng.random(G2.shape[:2]) < 0.2] = -1
    _compare_general(G2, dip["k"], S.locus_filter_spec(single=bool(single)), table=dip["G"])


@pytest.mark.parametrize("single", [1, 0])
def test_general_statistics_with_thousands_of_distinct_genotypes(single):
    """Loci whose genotype tables hold thousands of entries (tetraploid with
    30 alleles, diploid with 60): the tables and the HWE test's collapsed
    tables grow with the sample, in the order of first appearance."""
    tet = synth.fmodel(11, 3000, 12, 2, 0.01, 0.02, ploidy=np.full(3000, 4), n_alleles=np.full(12, 30),
                       anc_alpha=5.0)
    dip = synth.fmodel(12, 4000, 12, 2, 0.01, 0.02, n_alleles=np.full(12, 60), anc_alpha=5.0)
    for d, least in ((tet, 1500), (dip, 700)):
        G = d["G"]
        ndist = [len({tuple(sorted(c)) for c in G[l].tolist() if min(c) >= 0}) for l in range(G.shape[0])]
        assert min(ndist) > least
        _compare_general(G, d["k"], S.locus_filter_spec(single=bool(single)))
