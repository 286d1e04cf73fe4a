"""Regenerate the golden fixtures from the reference program itself.

Each case writes a seeded synthetic VCF (gzip) and runs the reference vcfpop
binary, compiled from its own sources by ``make -C oracle ref``, on it with one
thread and the scalar math path. The per-run output files it writes are stored
next to the VCF; ``tests/test_oracle_golden.py`` checks that the oracle
restatement reproduces them byte for byte.

Run from the repository root:  python tests/golden/make_golden.py [case ...]
With case names, only those cases are run (their VCF is written if missing)
and merged into cases.json; the other fixtures stay as they are.
"""
import gzip
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from vcfpop_gb300 import synth  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "vcfpop")

COMMON = ["-g_nthread=1", "-g_gpu=none", "-g_simd=none", "-g_float=single",
          "-g_fastsingle=yes", "-g_decimal=15", "-structure", "-structure_writelnl=yes",
          "-structure_nstream=1", "-structure_plot=no"]


def write_vcf_fmt(path, d, seed):
    """A VCF with GQ, DP and AD keys besides GT: FORMAT key orders (and case)
    that vary by line, values outside any window, '.' and negative values,
    calls that carry only some of the line's keys; three chromosomes (chr1,
    chr2, chr10) with increasing positions; one locus in ten an indel (REF T,
    ALT TA); FILTER PASS, pass, PASSED, q10 or '.'; QUAL a number or '.'.
    The last call of a line has a number in every key: the reference reads a
    '.' value on to the next number, past the end of its line if none
    follows."""
    rng = np.random.default_rng(seed)
    G, ploidy, k = d["G"], d["ploidy"], d["k"]
    L, N, _ = G.shape
    fmts = [["GT", "DP", "GQ"], ["GT", "GQ", "DP"], ["GT", "AD", "DP", "GQ"], ["GT"], ["GT", "dp", "Gq"]]
    chroms = np.where(np.arange(L) < L // 3, "chr1", np.where(np.arange(L) < 2 * L // 3, "chr2", "chr10"))
    pos = np.zeros(L, np.int64)
    for c in ("chr1", "chr2", "chr10"):
        idx = np.flatnonzero(chroms == c)
        pos[idx] = np.cumsum(rng.integers(200, 2500, len(idx)))
    filt = rng.choice(["PASS", "PASS", "PASS", "pass", "PASSED", "q10", "."], L)
    with open(path, "w") as f:
        f.write("##fileformat=VCFv4.2\n")
        for key, num, typ in (("GT", "1", "String"), ("DP", "1", "Integer"), ("GQ", "1", "Integer"), ("AD", "R", "Integer")):
            f.write(f'##FORMAT=<ID={key},Number={num},Type={typ},Description="{key}">\n')
        f.write("#CHROM\tPOS\tID\tREF\tALT\tQUAL\tFILTER\tINFO\tFORMAT\t")
        f.write("\t".join(f"Ind{i + 1}" for i in range(N)) + "\n")
        for l in range(L):
            kk = int(k[l])
            if kk == 2:
                ref, alt = ("T", "TA") if l % 10 == 7 else ("T", "A")
            else:
                ref, alt = "TT", ",".join("T" + "ACG"[(a - 1) % 3] * ((a + 2) // 3) for a in range(1, kk))
            keys = fmts[l % len(fmts)]
            cells = []
            for i in range(N):
                v = int(ploidy[i])
                g = G[l, i, :v]
                gt = "/".join(["."] * v) if g[0] < 0 else "/".join(str(int(x)) for x in g)
                vals = [gt]
                for key in keys[1:]:
                    kl = key.lower()
                    if kl == "ad":
                        vals.append(",".join(str(int(x)) for x in rng.integers(0, 30, kk)))
                    else:
                        r = rng.random()
                        if r < 0.05:
                            vals.append(".")
                        elif r < 0.07:
                            vals.append("-1")
                        else:
                            vals.append(str(int(rng.integers(0, 81 if kl == "dp" else 100))))
                if i == N - 1:
                    # every key of the line's last call holds a number, so a
                    # scan from a '.' finds one before the end of the line
                    vals = [x if j == 0 or x != "." else "33" for j, x in enumerate(vals)]
                elif len(keys) > 1 and rng.random() < 0.05:
                    vals = vals[:int(rng.integers(1, len(keys)))]      # a call with fewer keys
                cells.append(":".join(vals))
            qual = "." if l % 7 == 3 else str(int(rng.integers(5, 200)))
            f.write(f"{chroms[l]}\t{pos[l]}\tsnp{l + 1}\t{ref}\t{alt}\t{qual}\t{filt[l]}\t.\t{':'.join(keys)}\t"
                    + "\t".join(cells) + "\n")


def datasets():
    c1 = synth.fmodel(1, 200, 2000, 3, 0.1, 0.05)
    adm = synth.fmodel(2, 120, 400, 4, 0.05, 0.02, admix_alpha=0.5)
    ids = np.repeat(np.arange(4), 30)
    poly = synth.fmodel(3, 120, 300, 3, 0.08, 0.03, ploidy=np.array([2, 2, 4, 6] * 30),
                        n_alleles=np.random.default_rng(0).integers(2, 9, 300), anc_alpha=1.0,
                        loc_ids=ids, loc_alpha=1.0)
    # 7 individuals, one of them without a single typed call
    tiny = synth.fmodel(4, 7, 60, 2, 0.1, 0.05)
    tiny["G"][:, 3, :] = -1
    fmt = synth.fmodel(5, 100, 600, 3, 0.1, 0.05)
    fids = np.repeat(np.arange(4), 20)
    polyfmt = synth.fmodel(6, 80, 200, 3, 0.08, 0.03, ploidy=np.array([2, 2, 4, 6] * 20),
                           n_alleles=np.random.default_rng(1).integers(2, 7, 200), anc_alpha=1.0,
                           loc_ids=fids, loc_alpha=1.0)
    return {
        "fmt": (fmt, synth.indtext(fmt["pop"])),
        "polyfmt": (polyfmt, synth.indtext(fids)),
        "tiny": (tiny, synth.indtext(tiny["pop"])),
        "c1": (c1, synth.indtext(c1["pop"])),
        "adm": (adm, "popA:#1-#60 popB:#61-#120"),
        "poly": (poly, synth.indtext(ids)),
    }


CASES = {
    # name: (dataset, seed, flags)
    "c1_noadmix": ("c1", 1, ["-structure_krange=[3,3]", "-structure_nburnin=100",
                             "-structure_nreps=200", "-structure_nadmburnin=0", "-structure_admix=no"]),
    "c1_noadmix_admburnin": ("c1", 5, ["-structure_krange=[2,2]", "-structure_nburnin=20",
                                       "-structure_nreps=40", "-structure_nadmburnin=10",
                                       "-structure_admix=no"]),
    "adm_admix": ("adm", 7, ["-structure_admix=yes", "-structure_krange=[2,3]", "-structure_nburnin=30",
                             "-structure_nreps=60", "-structure_nruns=2"]),
    "adm_diffalpha": ("adm", 7, ["-structure_admix=yes", "-structure_diffalpha=yes",
                                 "-structure_uniformalpha=no", "-structure_krange=[3,3]",
                                 "-structure_nburnin=20", "-structure_nreps=40"]),
    "poly_admix_loc": ("poly", 7, ["-structure_admix=yes", "-structure_locpriori=yes",
                                   "-structure_krange=[3,3]", "-structure_nburnin=20",
                                   "-structure_nreps=40"]),
    "poly_noadmix_loc": ("poly", 7, ["-structure_admix=no", "-structure_locpriori=yes",
                                     "-structure_krange=[2,3]", "-structure_nburnin=20",
                                     "-structure_nreps=40"]),
    "poly_admix_f": ("poly", 7, ["-structure_admix=yes", "-structure_f=yes", "-structure_krange=[3,3]",
                                 "-structure_nburnin=20", "-structure_nreps=40"]),
    "poly_noadmix_singlef": ("poly", 7, ["-structure_admix=no", "-structure_f=yes",
                                         "-structure_singlef=yes", "-structure_nadmburnin=10",
                                         "-structure_krange=[2,2]", "-structure_nburnin=20",
                                         "-structure_nreps=40"]),
    # edge cases: one cluster; a handful of individuals, one untyped; the
    # general genotype layout without location prior or F model
    "c1_k1": ("c1", 11, ["-structure_krange=[1,2]", "-structure_nburnin=10", "-structure_nreps=20",
                         "-structure_nadmburnin=0", "-structure_admix=no", "-structure_nthinning=3"]),
    "tiny_noadmix": ("tiny", 12, ["-structure_krange=[1,3]", "-structure_nburnin=10", "-structure_nreps=20",
                                  "-structure_nadmburnin=0", "-structure_admix=no"]),
    "tiny_admix": ("tiny", 13, ["-structure_admix=yes", "-structure_krange=[2,2]", "-structure_nburnin=10",
                                "-structure_nreps=20"]),
    "poly_noadmix": ("poly", 14, ["-structure_admix=no", "-structure_krange=[2,2]", "-structure_nburnin=10",
                                  "-structure_nreps=20", "-structure_nadmburnin=5"]),
    # the locus filter (-f_filter with diversity windows) and the per-locus
    # diversity table, which lists the loci that survive; checked by the
    # filter tests rather than by a whole-file comparison with the oracle
    "c1_filter": ("c1", 3, ["-f", "-f_bmaf=[0.15,0.5]", "-f_ptype=[0.96,1]", "-f_ho=[0.1,0.6]",
                            "-structure_krange=[2,2]", "-structure_nburnin=10", "-structure_nreps=20",
                            "-structure_nadmburnin=0", "-structure_admix=no", "-structure_diversity=yes"]),
    # the genotype filter (DP and GQ windows; '.' and -1 values, calls with
    # fewer keys, keys in any order and case): whole-file comparisons
    "fmt_dpgq": ("fmt", 21, ["-f", "-f_dp=[10,60]", "-f_gq=[25,99]", "-structure_krange=[2,2]",
                             "-structure_nburnin=20", "-structure_nreps=40", "-structure_nadmburnin=0",
                             "-structure_admix=no"]),
    "polyfmt_dpgq_ploidy": ("polyfmt", 22, ["-f", "-f_dp=[5,70]", "-f_gq=[15,99]", "-f_ploidy=[2,4]",
                                            "-structure_admix=yes", "-structure_krange=[2,2]",
                                            "-structure_nburnin=10", "-structure_nreps=20"]),
    # the loader's locus tests and the window filter: the loci that survive
    # (the per-locus diversity table) are compared
    "fmt_window": ("fmt", 23, ["-f", "-f_type=snp", "-f_original=yes", "-f_chrprefix=chr1,chr2",
                               "-f_windowsize=4000", "-f_bmaf=[0.05,0.5]", "-f_qual=[20,250]",
                               "-structure_krange=[2,2]", "-structure_nburnin=10", "-structure_nreps=20",
                               "-structure_nadmburnin=0", "-structure_admix=no", "-structure_diversity=yes"]),
    "fmt_window_stat": ("fmt", 24, ["-f", "-f_type=indel", "-f_chrname=chr2,chr10", "-f_windowsize=2500",
                                    "-f_windowstat=ptype", "-f_dp=[10,60]", "-structure_krange=[2,2]",
                                    "-structure_nburnin=10", "-structure_nreps=20", "-structure_nadmburnin=0",
                                    "-structure_admix=no", "-structure_diversity=yes"]),
    # the locus windows and the window filter on polyploid multiallelic data
    "poly_filter": ("poly", 26, ["-f", "-f_k=[3,8]", "-f_he=[0.4,0.78]", "-f_ho=[0.3,0.76]", "-f_ae=[1.6,4.6]",
                                 "-f_ptype=[0.96,1]", "-f_pic=[0.3,0.75]", "-f_I=[0.6,1.68]", "-f_n=[110,120]",
                                 "-structure_admix=no", "-structure_krange=[2,2]", "-structure_nburnin=10",
                                 "-structure_nreps=20", "-structure_nadmburnin=5", "-structure_diversity=yes"]),
    "polyfmt_window": ("polyfmt", 27, ["-f", "-f_windowsize=2000", "-f_windowstat=pic", "-f_he=[0.3,0.9]",
                                       "-f_dp=[5,70]", "-structure_admix=yes", "-structure_krange=[2,2]",
                                       "-structure_nburnin=10", "-structure_nreps=20", "-structure_diversity=yes"]),
    "fmt_window_all": ("fmt", 25, ["-f", "-f_windowsize=3000", "-f_windowstat=ho", "-structure_krange=[2,2]",
                                   "-structure_nburnin=10", "-structure_nreps=20", "-structure_nadmburnin=0",
                                   "-structure_admix=no", "-structure_diversity=yes"]),
}


def main(only=None):
    if not os.path.exists(REF):
        subprocess.check_call(["make", "-C", os.path.join(ROOT, "oracle"), "-j8", "ref"])
    data = datasets()
    for name, (d, ind) in data.items():
        path = os.path.join(HERE, f"{name}.vcf.gz")
        if only and (os.path.exists(path) or all(CASES[c][0] != name for c in only)):
            continue
        with tempfile.NamedTemporaryFile("w", suffix=".vcf", delete=False) as t:
            tmp = t.name
        if name in ("fmt", "polyfmt"):
            write_vcf_fmt(tmp, d, 100 + len(name))
        else:
            synth.write_vcf(tmp, d)
        with open(tmp, "rb") as fi, gzip.GzipFile(path, "wb", mtime=0) as fo:
            shutil.copyfileobj(fi, fo)
        os.unlink(tmp)
    manifest = {}
    if only:
        with open(os.path.join(HERE, "cases.json")) as f:
            manifest = json.load(f)
    for case, (dname, seed, flags) in CASES.items():
        if only and case not in only:
            continue
        out = os.path.join(HERE, case)
        if os.path.isdir(out):
            shutil.rmtree(out)
        os.makedirs(out)
        work = tempfile.mkdtemp()
        vcf = os.path.join(work, "data.vcf")
        with gzip.open(os.path.join(HERE, f"{dname}.vcf.gz"), "rb") as fi, open(vcf, "wb") as fo:
            shutil.copyfileobj(fi, fo)
        ind = data[dname][1]
        args = [REF, f"-g_input={vcf}", "-g_format=vcf", f"-g_output={work}/out", f"-g_seed={seed}",
                f"-g_indtext={ind}"] + COMMON + flags
        # the reference waits for Enter after an error: give it no terminal, and a time limit
        subprocess.run(args, check=True, stdin=subprocess.DEVNULL, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL,
                       timeout=600)
        files = sorted(f for f in os.listdir(work) if f.startswith("out.structure"))
        for f in files:
            shutil.copy(os.path.join(work, f), os.path.join(out, f))
        shutil.rmtree(work)
        manifest[case] = {"data": f"{dname}.vcf.gz", "seed": seed, "indtext": ind, "flags": flags,
                          "files": files}
        print(case, files)
    with open(os.path.join(HERE, "cases.json"), "w") as f:
        json.dump(manifest, f, indent=1)


if __name__ == "__main__":
    main(sys.argv[1:] or None)
