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
