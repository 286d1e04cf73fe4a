"""Flag handling of the drop-in driver that needs no GPU: a filter of the
reference that the driver does not implement (-f_pop) is refused before any
data is read, so no run ever clusters data the caller asked to have filtered. The
reference applies its -f_* windows only under -f (src/parameters.cpp:
1336-1343), so without -f they are accepted and have no effect, as there."""
import subprocess

import pytest

from vcfpop_gb300.build import CLI


@pytest.mark.parametrize("flag", ["-f_pop=pop1"])
def test_unimplemented_filters_are_refused(flag, tmp_path):
    r = subprocess.run([CLI, "-structure", f"-g_input={tmp_path}/none.vcf", f"-g_output={tmp_path}/out", "-f", flag],
                       capture_output=True, text=True)
    assert r.returncode == 2
    assert "not implemented" in r.stderr and flag.split("=")[0] in r.stderr
    assert not list(tmp_path.iterdir())


def test_implemented_filters_are_accepted(tmp_path):
    """The implemented windows pass parsing; the run then stops at the
    missing input file, not at a flag."""
    r = subprocess.run([CLI, "-structure", f"-g_input={tmp_path}/none.vcf", f"-g_output={tmp_path}/out", "-f",
                        "-f_bmaf=[0.05,0.5]", "-f_ptype=[0.9,1]", "-f_k=[2,2]", "-f_n=[1,1000]", "-f_he=[0,1]",
                        "-f_ho=[0,1]", "-f_pic=[0,1]", "-f_ae=[1,2]", "-f_I=[0,2]", "-f_itype=[0.5,1]",
                        "-f_iploidy=[2,2]", "-f_pval=[0.001,1]", "-f_dp=[10,100]", "-f_gq=[20,99]",
                        "-f_ploidy=[2,4]", "-f_qual=[30,255]", "-f_model=prcs", "-f_type=snp", "-f_original=yes",
                        "-f_chrprefix=chr1,chr2", "-f_chrname=chr3", "-f_windowsize=1000", "-f_windowstat=pic"],
                       capture_output=True, text=True)
    assert r.returncode == 2
    assert "not implemented" not in r.stderr and "cannot read" in r.stderr


@pytest.mark.parametrize("flag", ["-f_qual=[20,1000]", "-f_gq=[20,101]", "-f_ploidy=[0,4]", "-f_dp=[30,10]",
                                  "-f_type=snv", "-f_original=maybe", "-f_windowsize=0", "-f_windowstat=I",
                                  "-f_model=hwe"])
def test_filter_values_outside_the_reference_ranges_are_refused(flag, tmp_path):
    """The reference's parameter ranges (src/parameters.cpp:695-756: -f_qual
    0..255, -f_gq 0..100, -f_ploidy 1..10, -f_windowsize 1..10^9, choices of
    -f_type, -f_original, -f_windowstat, -f_model) stop the driver before it
    reads any data."""
    r = subprocess.run([CLI, "-structure", f"-g_input={tmp_path}/none.vcf", f"-g_output={tmp_path}/out", "-f", flag],
                       capture_output=True, text=True)
    assert r.returncode == 2
    assert flag.split("=")[0] in r.stderr and "cannot read" not in r.stderr


def test_filters_without_f_are_ignored_as_in_the_reference(tmp_path):
    r = subprocess.run([CLI, "-structure", f"-g_input={tmp_path}/none.vcf", f"-g_output={tmp_path}/out",
                        "-f_dp=[10,100]"], capture_output=True, text=True)
    assert r.returncode == 2
    assert "not implemented" not in r.stderr and "cannot read" in r.stderr


def _imiss_vcf(path):
    """100 diploids x 800 SNPs; every fourth individual misses a further 30%
    of its calls."""
    import numpy as np
    from vcfpop_gb300 import synth
    d = synth.fmodel(5, 100, 800, 2, 0.1, 0.02)
    extra = np.random.default_rng(5).random((800, 100)) < 0.3
    extra[:, 1::4] = extra[:, 2::4] = extra[:, 3::4] = False
    d["G"][extra] = -1
    synth.write_vcf(path, d)
    return d


def test_individual_filter_keeps_the_reference_rule(tmp_path):
    """-f -f_itype=[0.9,1]: an individual stays when its typed-locus count is
    within (int64)(0.9 * L + 0.5) .. (int64)(1 * L + 0.5) (MarkerIndividual,
    src/filter.cpp:457-465). The driver reports the count it kept before it
    needs a GPU; here it is compared with the rule evaluated on the data."""
    import numpy as np
    vcf = str(tmp_path / "d.vcf")
    d = _imiss_vcf(vcf)
    L = d["G"].shape[0]
    ntype = (d["G"][:, :, 0] >= 0).sum(axis=0)
    want = int(((ntype >= int(0.9 * L + 0.5)) & (ntype <= int(1.0 * L + 0.5))).sum())
    assert 60 <= want < 100
    r = subprocess.run([CLI, "-structure", f"-g_input={vcf}", f"-g_output={tmp_path}/out", "-f", "-f_itype=[0.9,1]",
                        "-gb300_device=0"], capture_output=True, text=True)
    assert f"individual filter kept {want} of 100 individuals" in r.stderr, r.stderr


def test_ploidy_window_outside_the_data_removes_everyone(tmp_path):
    """-f_iploidy compares its window with the smallest and largest ploidy of
    the whole data set (src/filter.cpp:467-471), so a window that misses
    either removes every individual, which the reference reports as an
    error; a window covering both keeps everyone."""
    vcf = str(tmp_path / "d.vcf")
    _imiss_vcf(vcf)
    r = subprocess.run([CLI, "-structure", f"-g_input={vcf}", f"-g_output={tmp_path}/out", "-f", "-f_iploidy=[3,4]"],
                       capture_output=True, text=True)
    assert r.returncode == 1 and "all 100 individuals are excluded" in r.stderr
    r = subprocess.run([CLI, "-structure", f"-g_input={vcf}", f"-g_output={tmp_path}/out", "-f", "-f_iploidy=[2,2]"],
                       capture_output=True, text=True)
    assert "individual filter kept 100 of 100 individuals" in r.stderr
