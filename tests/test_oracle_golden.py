"""Pin the oracle: its output must equal the reference program's, byte for byte.

The fixtures under tests/golden/ were written by the reference vcfpop binary
(compiled from its own sources) via tests/golden/make_golden.py.
"""
import gzip
import json
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
CASES = json.load(open(os.path.join(GOLD, "cases.json")))


def _summary_table(path):
    lines = open(path, "rb").read().decode().replace("\r", "").split("\n")
    i = next(j for j, ln in enumerate(lines) if ln.startswith("ID\tk\trep"))
    return [ln for ln in lines[i:] if ln.strip()]


@pytest.mark.parametrize("case", sorted(CASES))
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
