"""The drop-in driver against the reference program's own output files.

vcfpop-gb300 takes the reference's flags and writes the reference's files. With
the reference random streams its likelihood trace follows the golden file
(written by the reference binary) at the start of the chain; for every golden
case the files have the reference's layout line for line.
"""
import gzip
import json
import os
import re
import shutil
import subprocess

import pytest

from vcfpop_gb300.build import CLI

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
CASES = json.load(open(os.path.join(GOLD, "cases.json")))
NUM = re.compile(r"-?\d+\.\d+|nan")


def _run(case, tmp, rng, form="plain"):
    c = CASES[case]
    vcf = os.path.join(tmp, "data.vcf")
    with gzip.open(os.path.join(GOLD, c["data"]), "rb") as fi, open(vcf, "wb") as fo:
        shutil.copyfileobj(fi, fo)
    args = [CLI, f"-g_input={vcf}", f"-g_output={tmp}/out", f"-g_seed={c['seed']}", "-g_decimal=15",
            f"-g_indtext={c['indtext']}", "-g_float=single", "-structure", "-structure_writelnl=yes",
            f"-gb300_rng={rng}", f"-gb300_form={form}"] + c["flags"]
    subprocess.run(args, check=True)
    return c


def _shape(text):
    return [NUM.sub("#", ln) for ln in text.replace("\r", "").split("\n")]


@pytest.mark.parametrize("case", sorted(CASES))
def test_cli_files_have_reference_layout(case, tmp_path):
    c = _run(case, str(tmp_path), "counter")
    for f in c["files"]:
        if f == "out.structure.txt":
            continue
        got = open(tmp_path / f, "rb").read().decode()
        want = open(os.path.join(GOLD, case, f), "rb").read().decode()
        assert _shape(got) == _shape(want), f
        assert got.count("\r\n") == want.count("\r\n")


# the genotype filter cases pin the device parse's DP/GQ/ploidy windows and
# the loci the loader's genotype table keeps: a call filtered differently, or
# a locus kept or ordered differently, changes the reference streams' trace
@pytest.mark.parametrize("case", ["c1_noadmix", "adm_admix", "fmt_dpgq", "polyfmt_dpgq_ploidy"])
def test_cli_reference_streams_follow_golden_trace(case, tmp_path):
    c = _run(case, str(tmp_path), "reference")
    f = [x for x in c["files"] if x.endswith(".lnl.txt")][0]
    got = [float(x) for x in NUM.findall(open(tmp_path / f).read())]
    want = [float(x) for x in NUM.findall(open(os.path.join(GOLD, case, f)).read())]
    assert len(got) == len(want)
    for g, w in list(zip(got, want))[:3]:
        assert abs(g - w) <= 1e-5 * abs(w), (g, w)


@pytest.mark.parametrize("case", ["c1_filter", "fmt_window", "fmt_window_stat", "fmt_window_all", "poly_filter",
                                  "polyfmt_window"])
def test_cli_locus_filter_keeps_the_reference_loci(case, tmp_path):
    """-f with locus filters: the diversity table lists the loci the reference
    program kept, by name, in its order. The cases cover the diversity
    windows, the loader's tests on the fixed columns (-f_type, -f_original,
    -f_chrprefix, -f_chrname, -f_qual), the genotype filter, and the window
    filter with three statistics."""
    c = _run(case, str(tmp_path), "counter")
    f = [x for x in c["files"] if x.endswith("_id=1.txt")][0]

    def loci(path):
        lines = open(path, "rb").read().decode().replace("\r", "").split("\n")
        i = next(j for j, ln in enumerate(lines) if ln.startswith("Estimated genetic diversity in each cluster"))
        return [ln.split("\t")[0] for ln in lines[i + 2:] if ln.split("\t")[0] not in ("", "Average")]

    got, want = loci(tmp_path / f), loci(os.path.join(GOLD, case, f))
    assert 0 < len(want) and got == want


def test_cli_tensor_core_form_writes_the_reference_files(tmp_path):
    """-gb300_form=tc on a no-admixture case: the reference's file layout, and
    the first recorded lnP(D) equal to the plain form's (same state, same
    Philox draws) within 1e-5."""
    (tmp_path / "tc").mkdir()
    (tmp_path / "plain").mkdir()
    c = _run("c1_noadmix", str(tmp_path / "tc"), "counter", form="tc")
    _run("c1_noadmix", str(tmp_path / "plain"), "counter", form="plain")
    for f in c["files"]:
        if f == "out.structure.txt":
            continue
        got = open(tmp_path / "tc" / f, "rb").read().decode()
        want = open(os.path.join(GOLD, "c1_noadmix", f), "rb").read().decode()
        assert _shape(got) == _shape(want), f
    f = [x for x in c["files"] if x.endswith(".lnl.txt")][0]
    tc = [float(x) for x in NUM.findall(open(tmp_path / "tc" / f).read())]
    pl = [float(x) for x in NUM.findall(open(tmp_path / "plain" / f).read())]
    assert len(tc) == len(pl) > 0
    assert abs(tc[0] - pl[0]) <= 1e-5 * abs(pl[0]), (tc[0], pl[0])


def test_cli_default_flags_run_the_tensor_core_batch(tmp_path):
    """The reference's default no-admixture K-sweep (-structure_admix=no
    -structure_krange=[1,4], default nadmburnin = 500 admixture burn-in
    sweeps) reaches the tensor-core form without any extra flag: the burn-in
    runs in the plain form, then every run joins the batch. Against the same
    runs forced into the plain form: the admixture burn-in records are equal
    bit for bit, the first single-label record within 1e-5, and the files keep
    the reference's layout."""
    vcf = os.path.join(str(tmp_path), "data.vcf")
    with gzip.open(os.path.join(GOLD, "c1.vcf.gz"), "rb") as fi, open(vcf, "wb") as fo:
        shutil.copyfileobj(fi, fo)
    out = {}
    for form in ("default", "plain"):
        d = tmp_path / form
        d.mkdir()
        args = [CLI, f"-g_input={vcf}", f"-g_output={d}/out", "-g_seed=5", "-g_decimal=15", "-structure",
                "-structure_admix=no", "-structure_krange=[1,4]", "-structure_nburnin=30", "-structure_nreps=40",
                "-structure_nthinning=1",
                "-structure_writelnl=yes"] + ([] if form == "default" else ["-gb300_form=plain"])
        r = subprocess.run(args, check=True, capture_output=True, text=True)
        assert ("tensor-core form" in r.stderr) == (form == "default"), r.stderr
        out[form] = d
    for K in range(1, 5):
        f = f"out.structure.k={K}_rep=1_id={K}.lnl.txt"
        tc = [float(x) for x in NUM.findall(open(out["default"] / f).read())]
        pl = [float(x) for x in NUM.findall(open(out["plain"] / f).read())]
        assert len(tc) == len(pl) == 500 + 30 + 40
        assert tc[:500] == pl[:500]
        assert abs(tc[500] - pl[500]) <= 1e-5 * abs(pl[500])
        g = open(out["default"] / f"out.structure.k={K}_rep=1_id={K}.txt", "rb").read().decode()
        p = open(out["plain"] / f"out.structure.k={K}_rep=1_id={K}.txt", "rb").read().decode()
        assert _shape(g) == _shape(p)


def test_cli_individual_filter_runs_on_the_kept_individuals(tmp_path):
    """-f -f_itype=[0.9,1]: the run's ancestry table lists exactly the
    individuals whose typed-locus count passes the reference's window
    (src/filter.cpp:457-465), in file order."""
    import numpy as np
    from vcfpop_gb300 import synth
    d = synth.fmodel(5, 100, 800, 2, 0.1, 0.02)
    extra = np.random.default_rng(5).random((800, 100)) < 0.3
    extra[:, 1::4] = extra[:, 2::4] = extra[:, 3::4] = False
    d["G"][extra] = -1
    vcf = str(tmp_path / "d.vcf")
    synth.write_vcf(vcf, d)
    L = d["G"].shape[0]
    ntype = (d["G"][:, :, 0] >= 0).sum(axis=0)
    keep = np.where((ntype >= int(0.9 * L + 0.5)) & (ntype <= int(L + 0.5)))[0]
    subprocess.run([CLI, f"-g_input={vcf}", f"-g_output={tmp_path}/out", "-structure", "-f", "-f_itype=[0.9,1]",
                    "-structure_krange=[2,2]", "-structure_nburnin=10", "-structure_nreps=20",
                    "-structure_admix=no", "-structure_nadmburnin=0"], check=True)
    lines = open(tmp_path / "out.structure.k=2_rep=1_id=1.txt", "rb").read().decode().replace("\r", "").split("\n")
    i = next(j for j, ln in enumerate(lines) if ln.startswith("Inferred ancestry of individuals"))
    names = []
    for ln in lines[i + 3:]:
        if not ln.strip():
            break
        names.append(ln.split("\t")[0])
    header = open(vcf).read().split("\n")
    samples = next(h for h in header if h.startswith("#CHROM")).split("\t")[9:]
    assert names == [samples[j] for j in keep]
