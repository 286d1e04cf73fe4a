"""Flag handling of the drop-in driver that needs no GPU: the reference's
filters that the driver does not implement are refused before any data is
read, so no run ever clusters data the caller asked to have filtered."""
import subprocess

import pytest

from vcfpop_gb300.build import CLI


@pytest.mark.parametrize("flag", ["-f_dp=[10,100]", "-f_gq=[20,99]", "-f_qual=[30,255]", "-f_pval=[0.001,1]",
                                  "-f_itype=[0.5,1]", "-f_iploidy=[2,2]", "-f_windowsize=1000", "-f_ploidy=[2,2]",
                                  "-f_type=snp", "-f_chrprefix=chr"])
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
                        "-f_ho=[0,1]", "-f_pic=[0,1]", "-f_ae=[1,2]", "-f_I=[0,2]"], capture_output=True, text=True)
    assert r.returncode == 2
    assert "not implemented" not in r.stderr and "cannot read" in r.stderr
