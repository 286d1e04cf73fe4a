"""VCF genotype ingest on the device (vp_vcf_pack2) against the packing of
the genotypes the VCF was written from: bit-exact on the committed golden
VCFs and on synthetic files with phased/unphased calls, extra FORMAT keys,
CRLF line ends, a missing final line feed and half-missing calls; lines
outside the fast path fail with their line number."""
import gzip
import os

import numpy as np
import pytest

from vcfpop_gb300 import _lib as B
from vcfpop_gb300 import structure as S
from vcfpop_gb300 import synth

from . import orc

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _data_section(text: bytes):
    i = text.index(b"\n#CHROM")
    return text[text.index(b"\n", i + 1) + 1:]


def _vcf(G, phased=False, extra=False, crlf=False, tail=True):
    L, N, _ = G.shape
    sep = "|" if phased else "/"
    lines = []
    for l in range(L):
        calls = []
        for i in range(N):
            a, b = G[l, i]
            c = "./." if a < 0 else f"{a}{sep}{b}"
            calls.append(c + (":7" if extra else ""))
        fmt = "GT:DP" if extra else "GT"
        lines.append(f"1\t{l + 1}\t.\tA\tC\t.\tPASS\t.\t{fmt}\t" + "\t".join(calls))
    nl = "\r\n" if crlf else "\n"
    s = nl.join(lines) + (nl if tail else "")
    return s.encode()


@pytest.mark.parametrize("name,args", [("c1", (1, 200, 2000, 3, 0.1, 0.05)), ("adm", (2, 120, 400, 4, 0.05, 0.02))])
def test_golden_vcfs_pack_exactly(name, args):
    kw = dict(admix_alpha=0.5) if name == "adm" else {}
    d = synth.fmodel(*args, **kw)                      # the data make_golden.py wrote
    text = gzip.open(os.path.join(GOLD, f"{name}.vcf.gz"), "rb").read()
    packed, starts = S.vcf_pack2(_data_section(text), d["G"].shape[1])
    assert packed.shape[0] == d["G"].shape[0]
    assert np.array_equal(packed, S.pack2(d["G"]))


@pytest.mark.parametrize("phased,extra,crlf,tail", [(False, False, False, True), (True, True, False, True),
                                                    (False, True, True, False), (True, False, True, True)])
def test_synthetic_variants_pack_exactly(phased, extra, crlf, tail):
    d = synth.fmodel(81, 333, 257, 3, 0.1, 0.1)         # 333 samples: a ragged last word
    G = d["G"].copy()
    if phased:
        G = G[:, :, ::-1].copy()                       # 1|0 as well as 0|1
        G[G[:, :, 0] < 0] = -1
    text = _vcf(G, phased, extra, crlf, tail)
    packed, starts = S.vcf_pack2(text, 333)
    assert np.array_equal(packed, S.pack2(d["G"]))     # codes count allele 1: the copy order does not matter
    assert np.array_equal(packed, orc.vcf_pack2(text, 333, packed.shape[0]))
    assert starts[0] == 0 and starts[-1] == len(text)


def test_half_missing_call_is_missing():
    G = np.array([[[0, 1], [1, 1], [0, 0]]], np.int8)
    text = _vcf(G).replace(b"\t1/1", b"\t1/.")
    packed, _ = S.vcf_pack2(text, 3)
    assert packed[0, 0] & 0x3F == (1 | (3 << 2) | (0 << 4))


@pytest.mark.parametrize("bad,what", [(b"A\tC,G", "2 alleles"), (b"\t0\t", "diploid"), (b"GT\t", "GT is not")])
def test_unsupported_lines_name_the_line(bad, what):
    d = synth.fmodel(82, 20, 30, 2, 0.1, 0.0)
    text = _vcf(d["G"])
    lines = text.split(b"\n")
    if bad == b"A\tC,G":
        lines[4] = lines[4].replace(b"A\tC", b"A\tC,G", 1)
    elif bad == b"\t0\t":
        parts = lines[4].split(b"\t")
        parts[12] = b"0"
        lines[4] = b"\t".join(parts)
    else:
        lines[4] = lines[4].replace(b"\tGT\t", b"\tDP:GT\t", 1)
    with pytest.raises(B.VpError, match=f"data line 5: .*{what}"):
        S.vcf_pack2(b"\n".join(lines), 20)


def test_packed_vcf_runs_a_chain():
    d = synth.fmodel(83, 400, 1500, 3, 0.1, 0.02)
    packed, _ = S.vcf_pack2(_vcf(d["G"]), 400)
    ds = S.Dataset(np.full(400, 2, np.int32), np.full(1500, 2, np.int32), d["pop"], 3, packed2=packed)
    ref = S.Dataset.from_synth(d)
    assert np.array_equal(ds.order(), ref.order())
    ctx = S.Context(ds)
    ch = S.Chain(ctx, S.params(3, 5, admix=0, nadmburnin=0, nburnin=5, nreps=5))
    S.finish([ch])
    assert np.isfinite(ch.result()["rout"]).all()


def _general_vcf(d, phased_every=0, extra=False, crlf=False):
    """A VCF of any ploidy and allele count; calls in a shuffled copy order
    (and '|' every phased_every-th call), so the parser must sort them."""
    G, ploidy, k = d["G"], d["ploidy"], d["k"]
    L, N, _ = G.shape
    rng = np.random.default_rng(3)
    lines = []
    for l in range(L):
        calls = []
        for i in range(N):
            v = int(ploidy[i])
            g = G[l, i, :v]
            if g[0] < 0:
                c = "/".join(["."] * v)
            else:
                sep = "|" if phased_every and (l * N + i) % phased_every == 0 else "/"
                c = sep.join(str(int(x)) for x in rng.permutation(g))
            calls.append(c + (":12,3" if extra else ""))
        alt = ",".join(["G"] * (int(k[l]) - 1))
        lines.append(f"2\t{l + 1}\tv{l}\tA\t{alt}\t.\tPASS\t.\t{'GT:AD' if extra else 'GT'}\t" + "\t".join(calls))
    nl = "\r\n" if crlf else "\n"
    return (nl.join(lines) + nl).encode()


@pytest.mark.parametrize("case", ["poly", "poly_extra_crlf", "haploid_diploid"])
def test_general_parse_matches_the_source_genotypes(case):
    """vp_vcf_parse on polyploid multiallelic data (ploidy 2/4/6, 2-8
    alleles), with phased and unphased calls in any copy order, extra FORMAT
    keys and CRLF line ends: the allele copies the data were drawn with, in
    ascending order, -1 for missing calls, bit for bit; the alleles per locus
    and each sample's ploidy as the host reader sets them."""
    rng = np.random.default_rng(11)
    if case == "haploid_diploid":
        d = synth.fmodel(12, 50, 120, 2, 0.1, 0.05, ploidy=np.array([1, 2] * 25), n_alleles=rng.integers(2, 5, 120),
                         anc_alpha=1.0)
    else:
        d = synth.fmodel(13, 90, 300, 3, 0.08, 0.03, ploidy=np.array([2, 2, 4, 6] * 22 + [2, 2]),
                         n_alleles=rng.integers(2, 9, 300), anc_alpha=1.0)
    text = _general_vcf(d, phased_every=7, extra="extra" in case, crlf="crlf" in case)
    vmax = int(d["ploidy"].max())
    G, k, ploidy, starts = S.vcf_parse(text, d["G"].shape[1], vmax)
    assert np.array_equal(G, d["G"])
    assert np.array_equal(k, d["k"])
    assert np.array_equal(ploidy, d["ploidy"])
    assert starts[0] == 0 and starts[-1] == len(text)


def test_general_parse_of_the_golden_polyploid_vcf():
    raw = gzip.open(os.path.join(GOLD, "poly.vcf.gz")).read()
    header = raw[raw.index(b"\n#CHROM") + 1:].split(b"\n", 1)[0].decode().split("\t")
    N = len(header) - 9
    G, k, ploidy, _ = S.vcf_parse(_data_section(raw), N, 6)
    # the genotypes the golden file was written from (tests/golden/make_golden.py)
    d = synth.fmodel(3, 120, 300, 3, 0.08, 0.03, ploidy=np.array([2, 2, 4, 6] * 30),
                     n_alleles=np.random.default_rng(0).integers(2, 9, 300), anc_alpha=1.0,
                     loc_ids=np.repeat(np.arange(4), 30), loc_alpha=1.0)
    assert np.array_equal(G, d["G"]) and np.array_equal(k, d["k"]) and np.array_equal(ploidy, d["ploidy"])


def test_general_parse_rejects_what_it_cannot_store():
    d = synth.fmodel(14, 10, 5, 2, 0.1, 0.0)
    text = _general_vcf(d).replace(b"\t0/", b"\t200/", 1)
    with pytest.raises(B.VpError, match="line 1: an allele index above 127"):
        S.vcf_parse(text, 10, 2)
    bad = _general_vcf(d).replace(b"\tGT\t", b"\tDP:GT\t", 1)
    with pytest.raises(B.VpError, match="GT is not the first"):
        S.vcf_parse(bad, 10, 2)


# The genotype filter of the device parses against the oracle's parse, which
# restates the loader's line rewrite (GT, DP and GQ kept, case as written) and
# AddVCFGenotype literally and is pinned on the reference program by the
# fmt_dpgq and polyfmt_dpgq_ploidy golden cases. The golden fmt VCF has DP,
# GQ and AD keys in several orders, lowercase keys (which the loader drops),
# '.' and -1 values, and calls with fewer keys than FORMAT.
@pytest.mark.parametrize("windows", [dict(dp=(10, 60)), dict(gq=(25, 99)), dict(dp=(10, 60), gq=(25, 99)),
                                     dict(ploidy=(3, 4)), dict(dp=(0, 0x7FFFFFFF), gq=(0, 100))])
def test_genotype_filter_of_the_device_parses_matches_the_oracle(windows):
    raw = gzip.open(os.path.join(GOLD, "fmt.vcf.gz")).read()
    header = raw[raw.index(b"\n#CHROM") + 1:].split(b"\n", 1)[0].decode().split("\t")
    N = len(header) - 9
    text = _data_section(raw)
    L = text.count(b"\n")
    want = orc.vcf_pack2(text, N, L, calls=orc.call_filter(**windows))
    unfiltered = orc.vcf_pack2(text, N, L)
    got, _ = S.vcf_pack2(text, N, calls=S.call_filter(**windows))
    assert np.array_equal(got, want)
    codes = (want[:, np.arange(N) // 16] >> (2 * (np.arange(N) % 16))) & 3
    before = (unfiltered[:, np.arange(N) // 16] >> (2 * (np.arange(N) % 16))) & 3
    if windows.get("dp", (0, 0x7FFFFFFF)) != (0, 0x7FFFFFFF):
        assert (codes == 3).sum() > (before == 3).sum()      # the windows took calls away
    # the general parse of the same text gives the same calls
    G, k, ploidy, _ = S.vcf_parse(text, N, 2, calls=S.call_filter(**windows))
    typed = G[:, :, 0] >= 0
    assert np.array_equal(typed, codes != 3)
    assert np.array_equal(np.where(typed, G.sum(axis=2), 3), codes)
