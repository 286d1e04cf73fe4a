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
    return {
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
