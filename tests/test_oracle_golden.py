"""Pin the oracle: its output must equal the reference program's, byte for byte.

The fixtures under tests/golden/ were written by the reference vcfpop binary
(compiled from its own sources) via tests/golden/make_golden.py.
"""
import gzip
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
CASES = json.load(open(os.path.join(GOLD, "cases.json")))


def _summary_table(path):
    lines = open(path, "rb").read().decode().replace("\r", "").split("\n")
    i = next(j for j, ln in enumerate(lines) if ln.startswith("ID\tk\trep"))
    return [ln for ln in lines[i:] if ln.strip()]


# the oracle's driver takes the genotype filter (-f with -f_dp, -f_gq,
# -f_ploidy); cases with locus filters are checked by their own tests
CALL_FILTERS = ("-f_dp=", "-f_gq=", "-f_ploidy=")
WHOLE = sorted(c for c in CASES
               if all(not x.startswith("-f_") or x.startswith(CALL_FILTERS) for x in CASES[c]["flags"]))


@pytest.mark.parametrize("case", WHOLE)
def test_oracle_matches_reference(case, oracle_build, tmp_path):
    c = CASES[case]
    vcf = tmp_path / "data.vcf"
    with gzip.open(os.path.join(GOLD, c["data"]), "rb") as fi, open(vcf, "wb") as fo:
        shutil.copyfileobj(fi, fo)
    args = [os.path.join(oracle_build, "orc_cli"), f"-g_input={vcf}", f"-g_output={tmp_path}/out",
            f"-g_seed={c['seed']}", "-g_decimal=15", f"-g_indtext={c['indtext']}",
            "-structure_writelnl=yes"] + c["flags"]
    subprocess.run(args, check=True)
    for f in c["files"]:
        ref = os.path.join(GOLD, case, f)
        if f == "out.structure.txt":
            assert _summary_table(ref) == _summary_table(tmp_path / "out.oracle.structure.txt")
            continue
        got = open(tmp_path / f, "rb").read()
        want = open(ref, "rb").read()
        assert got == want, f"{case}/{f} differs from the reference output"


def _d_block(path, K):
    lines = open(path, "rb").read().decode().replace("\r", "").split("\n")
    i = next(j for j, ln in enumerate(lines) if ln.startswith("Allele-frequency divergence among pops"))
    return [[float(v) for v in lines[i + 3 + r].split("\t")[1:1 + K]] for r in range(K)]


def test_oracle_divergence_reproduces_reference_d_block(oracle_build):
    """orc_divergence (the heterozygosity / net nucleotide distance loops of
    WriteStructure) on the oracle's finished c1 chain gives the D block the
    reference program printed for the same run, to its 15 printed decimals."""
    import numpy as np
    from vcfpop_gb300 import synth
    from . import orc
    c = CASES["c1_noadmix"]
    d = synth.fmodel(1, 200, 2000, 3, 0.1, 0.05)          # the c1 data make_golden.py wrote
    od = orc.Data(d)
    K = 3
    seed = orc.lib().orc_hash_ulong_c(c["seed"] + 1)     # run id 1
    oc = orc.Chain(od, orc.params(K, seed, admix=0, nadmburnin=0, nburnin=100, nreps=200, writelnl=1))
    orc.lib().orc_run(oc.h)
    k = od.field(1, np.int32)
    out = orc.divergence(oc.get("FREQM"), k, K, per_locus=True)
    want = np.array(_d_block(os.path.join(GOLD, "c1_noadmix", "out.structure.k=3_rep=1_id=1.txt"), K))
    assert np.abs(out["D"] - want).max() < 1e-14, (out["D"], want)
    assert np.allclose(out["Hl"].mean(axis=1), out["H"])


@pytest.mark.parametrize("name,args,kw", [("c1", (1, 200, 2000, 3, 0.1, 0.05), {}),
                                         ("adm", (2, 120, 400, 4, 0.05, 0.02), {"admix_alpha": 0.5})])
def test_oracle_vcf_parse_matches_golden_data(name, args, kw, oracle_build):
    """The oracle's VCF genotype parse, on the committed golden VCFs, gives the
    2-bit packing of the genotypes those files were written from."""
    import numpy as np
    from vcfpop_gb300 import structure as S
    from vcfpop_gb300 import synth
    from . import orc
    d = synth.fmodel(*args, **kw)
    t = gzip.open(os.path.join(GOLD, f"{name}.vcf.gz"), "rb").read()
    i = t.index(b"\n#CHROM")
    data = t[t.index(b"\n", i + 1) + 1:]
    assert np.array_equal(orc.vcf_pack2(data, d["G"].shape[1], d["G"].shape[0]), S.pack2(d["G"]))


def _diversity_loci(path):
    """Locus names of the per-locus diversity table of a run file."""
    lines = open(path, "rb").read().decode().replace("\r", "").split("\n")
    i = next(j for j, ln in enumerate(lines) if ln.startswith("Estimated genetic diversity in each cluster"))
    names = []
    for ln in lines[i + 2:]:
        if not ln.strip():
            break
        head = ln.split("\t")[0]
        if head and head != "Average":
            names.append(head)
    return names


def test_oracle_locus_filter_matches_reference(oracle_build):
    """The oracle's locus filter (statistics of CalcDiversity, conditions of
    MarkerDiversity) keeps exactly the loci the reference program kept under
    -f -f_bmaf=[0.15,0.5] -f_ptype=[0.96,1] -f_ho=[0.1,0.6]: the loci listed
    in its diversity table (those passing, less the monomorphic ones that
    STRUCTURE drops). The statistics are in float, as the reference computes
    them under -g_float=single: 5 loci with ptype = 192/200 fall just below
    0.96 in float and are dropped, as the reference dropped them."""
    import numpy as np
    from vcfpop_gb300 import structure as S
    from vcfpop_gb300 import synth
    from . import orc
    d = synth.fmodel(1, 200, 2000, 3, 0.1, 0.05)          # the c1 data make_golden.py wrote
    packed = S.pack2(d["G"])
    f = orc.LocusFilter(bmaf_b=1, bmaf_min=0.15, bmaf_max=0.5, ptype_b=1, ptype_min=0.96, ptype_max=1.0,
                        ho_b=1, ho_min=0.1, ho_max=0.6, single=1)      # the golden runs use -g_float=single
    keep, stats = orc.locus_filter_pack2(packed, 200, f)
    kept = {f"1_snp{l + 1}" for l in range(len(keep)) if keep[l] and stats[l, 1] >= 2}
    want = set(_diversity_loci(os.path.join(GOLD, "c1_filter", "out.structure.k=2_rep=1_id=1.txt")))
    assert 0 < len(want) < 2000
    assert kept == want


def test_oracle_general_locus_filter_matches_reference(oracle_build):
    """The oracle's locus filter for the general genotype layout (ploidy
    2/4/6, 2-8 alleles: CalcDiversity over each locus' genotype table in order
    of first appearance) keeps exactly the loci the reference program kept
    under every diversity window at once (poly_filter), in float."""
    import numpy as np
    from . import orc
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLD, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    d = mg.datasets()["poly"][0]
    f = orc.LocusFilter(single=1, k_b=1, k_min=3, k_max=8, he_b=1, he_min=0.4, he_max=0.78, ho_b=1, ho_min=0.3,
                        ho_max=0.76, ae_b=1, ae_min=1.6, ae_max=4.6, ptype_b=1, ptype_min=0.96, ptype_max=1.0,
                        pic_b=1, pic_min=0.3, pic_max=0.75, I_b=1, I_min=0.6, I_max=1.68, n_b=1, n_min=110, n_max=120)
    keep, stats = orc.locus_filter_general(d["G"], d["k"], f)
    kept = {f"1_snp{l + 1}" for l in range(len(keep)) if keep[l] and stats[l, 1] >= 2}
    want = set(_diversity_loci(os.path.join(GOLD, "poly_filter", "out.structure.k=2_rep=1_id=1.txt")))
    assert 0 < len(want) < 300
    assert kept == want


def test_oracle_general_statistics_equal_the_biallelic_ones():
    """On biallelic diploid data the general statistics are the packed
    kernel's: n, k, ptype, bmaf, he, ho, pic, ae and I equal, in float and in
    double; the p-value to 1e-5 (the G statistic sums the genotypes in table
    order there, in a fixed order here)."""
    import numpy as np
    from vcfpop_gb300 import structure as S
    from vcfpop_gb300 import synth
    from . import orc
    d = synth.fmodel(3, 200, 500, 3, 0.1, 0.05)
    for single in (1, 0):
        f = orc.LocusFilter(single=single)
        kp, sp = orc.locus_filter_pack2(S.pack2(d["G"]), 200, f)
        kg, sg = orc.locus_filter_general(d["G"], d["k"], f)
        assert np.array_equal(kp, kg)
        assert np.array_equal(np.isnan(sp), np.isnan(sg))
        both = ~np.isnan(sp)
        assert np.array_equal(sp[:, :9][both[:, :9]], sg[:, :9][both[:, :9]])
        assert np.allclose(sp[:, 9][both[:, 9]], sg[:, 9][both[:, 9]], rtol=1e-5, atol=0)


def test_oracle_chi_square_tail_by_the_incomplete_gamma_function():
    """The HWE p-value of the general test: 1 - P(df/2, G/2) by the
    regularized incomplete gamma function, against scipy's chi-square
    survival function over the degrees of freedom the test meets."""
    import ctypes as C
    import numpy as np
    from scipy import stats
    from . import orc
    # a diploid triallelic locus of 400 individuals in HWE proportions: df = 3
    rng = np.random.default_rng(4)
    p = np.array([0.5, 0.3, 0.2])
    a = rng.choice(3, size=(1, 400, 2), p=p)
    G = np.sort(a, axis=2).astype(np.int8)
    f = orc.LocusFilter(single=0)
    _, st = orc.locus_filter_general(G, [3], f)
    pval = st[0, 9]
    # the G statistic from the same table: observed and expected counts
    n = 400
    cnt = np.bincount(G[0].ravel(), minlength=3) + 0.0
    fr = (cnt + 1e-10) / (cnt.sum() + 3e-10)
    obs = {}
    for g in map(tuple, G[0]):
        obs[g] = obs.get(g, 0) + 1
    Gs = 0.0
    for (x, y), o in obs.items():
        e = (fr[x] * fr[y] * (2 if x != y else 1)) * n
        Gs += 2 * o * np.log(o / e)
    assert abs(pval - stats.chi2.sf(Gs, 3)) <= 1e-9 * max(1.0, stats.chi2.sf(Gs, 3))


def test_oracle_record_lnl_is_counts_times_log_frequencies(oracle_build):
    """Without admixture, Record's lnP(D) (structure.cpp:1902-1938) is the sum
    over clusters, loci and alleles of Ni x ln p at the state it is recorded
    in: the identity the full-size lnP(D) error figure of the batched form is
    measured with."""
    import numpy as np
    from tests import orc
    from vcfpop_gb300 import synth
    d = synth.fmodel(71, 150, 400, 3, 0.1, 0.05)
    od = orc.Data(d)
    for K in (2, 4):
        oc = orc.Chain(od, orc.params(K, 900 + K, admix=0, nadmburnin=0, nburnin=5, nreps=5))
        oc.init()
        for _ in range(3):
            oc.step("sweep")
            got = orc.lib().orc_record_lnl(oc.h)
            ni, p = oc.get("NI").astype(np.float64), oc.get("FREQ").astype(np.float64)
            want = float(np.sum(ni[ni > 0] * np.log(p[ni > 0])))
            assert abs(got - want) <= 1e-12 * abs(want), (K, got, want)


SANITIZED = ["c1_k1", "tiny_noadmix", "tiny_admix", "poly_noadmix", "adm_admix"]


def test_oracle_driver_runs_clean_under_sanitizers(tmp_path):
    """The oracle's driver built with AddressSanitizer and UBSan, on the golden
    cases that stress its bookkeeping (loci dropped by the monomorphic filter,
    thinning that does not divide the run, K = 1, admixture): no memory or
    undefined-behaviour error, and the same files as the reference."""
    src = os.path.join(os.path.dirname(HERE), "oracle")
    exe = str(tmp_path / "orc_cli_san")
    r = subprocess.run(["gcc", "-O1", "-g", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math",
                        "-fsanitize=address,undefined", "-fno-sanitize-recover=all", "-w", "-o", exe,
                        os.path.join(src, "oracle_cli.c"), os.path.join(src, "structure_oracle.c"), "-lm", "-lpthread"],
                       capture_output=True)
    if r.returncode:
        pytest.skip("no sanitizer runtime for gcc here")
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0")
    for case in SANITIZED:
        c = CASES[case]
        w = tmp_path / case
        w.mkdir()
        with gzip.open(os.path.join(GOLD, c["data"]), "rb") as fi, open(w / "data.vcf", "wb") as fo:
            shutil.copyfileobj(fi, fo)
        r = subprocess.run([exe, f"-g_input={w / 'data.vcf'}", f"-g_output={w}/out", f"-g_seed={c['seed']}",
                            "-g_decimal=15", f"-g_indtext={c['indtext']}", "-structure_writelnl=yes"] + c["flags"],
                           capture_output=True, text=True, env=env, timeout=600)
        assert r.returncode == 0, f"{case}: {r.stderr[:2000]}"
        for f in c["files"]:
            if f != "out.structure.txt":
                assert open(w / f, "rb").read() == open(os.path.join(GOLD, case, f), "rb").read(), f"{case}/{f}"


def test_oracle_hwe_pvalue_is_the_g_test_upper_tail(oracle_build):
    """-f_pval's statistic (CalcDiversity's HWE test, src/diversity.cpp:
    337-492) for biallelic diploid loci: the G statistic of the observed
    genotype counts against HWE expectations from the sample's allele
    frequencies, and its chi-square upper tail with one degree of freedom;
    NaN when an expected count is below 5. The reference's own chi-square
    CDF comes from a library that is not in its tree, so the p-value is
    checked here against scipy's chi-square survival function of the same G
    (in double), over loci drawn with and without HWE deviations."""
    from . import orc
    scipy_stats = pytest.importorskip("scipy.stats")
    rng = np.random.default_rng(8)
    N, L = 300, 400
    p = rng.uniform(0.02, 0.98, L)
    F = rng.uniform(-0.2, 0.6, L)                     # inbreeding: departures from HWE
    probs = np.stack([p * p + F * p * (1 - p), 2 * p * (1 - p) * (1 - F), (1 - p) ** 2 + F * p * (1 - p)], 1)
    probs = np.clip(probs, 0, None)
    probs /= probs.sum(1, keepdims=True)
    codes = np.array([rng.choice(3, N, p=pr) for pr in probs])
    codes[rng.random((L, N)) < 0.05] = 3
    Nw = (N + 15) // 16
    pad = np.full((L, Nw * 16), 3, np.uint32)
    pad[:, :N] = codes
    packed = np.bitwise_or.reduce(pad.reshape(L, Nw, 16) << (np.arange(16, dtype=np.uint32) * 2), axis=2).astype(np.uint32)
    f = orc.LocusFilter(single=0)
    keep, stats = orc.locus_filter_pack2(packed, N, f)
    tested = 0
    for l in range(L):
        c = np.array([(codes[l] == g).sum() for g in range(3)], np.float64)
        n = c.sum()
        fr = np.array([2 * c[0] + c[1], c[1] + 2 * c[2]]) + 1e-10
        fr /= fr.sum()
        ex = np.array([fr[0] ** 2, 2 * fr[0] * fr[1], fr[1] ** 2]) * n
        if (ex[c > 0] < 5).any():
            assert np.isnan(stats[l, 9])
            continue
        G = float(np.sum(2 * c[c > 0] * np.log(c[c > 0] / ex[c > 0])))
        want = scipy_stats.chi2.sf(G, 1)
        assert abs(stats[l, 9] - want) <= 1e-12 + 1e-9 * want, (l, stats[l, 9], want)
        tested += 1
    assert tested > L // 2
    # the window drops the loci whose p-value falls outside it; NaN passes
    f2 = orc.LocusFilter(single=0, pval_b=1, pval_min=0.01, pval_max=1.0)
    keep2, _ = orc.locus_filter_pack2(packed, N, f2)
    pv = stats[:, 9]
    assert np.array_equal(keep2.astype(bool), keep.astype(bool) & ~(pv < 0.01))
    assert (pv < 0.01).sum() > 10
