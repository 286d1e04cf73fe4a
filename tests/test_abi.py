"""CPU checks of the C ABI and the host logic (no GPU needed)."""
import ctypes
import os
import re

import numpy as np
import pytest

from vcfpop_gb300 import _lib as B
from vcfpop_gb300 import structure as S
from vcfpop_gb300 import synth

from . import orc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol():
    hdr = open(os.path.join(ROOT, "include", "vcfpop_structure.h")).read()
    declared = sorted(set(re.findall(r"\b(vp_[a-z0-9_]+)\s*\(", hdr)))
    assert declared, "no declarations found"
    L = B.lib()
    for name in declared:
        assert hasattr(L, name), f"{name} declared but not exported"
    assert set(declared) == set(B.EXPORTS)


def test_run_seed_matches_reference_hash():
    for g, i in [(1, 1), (7, 3), (0, 1), (123456, 42)]:
        assert S.run_seed(g, i) == orc.lib().orc_hash_ulong_c(g + i)
    assert S.run_seed(1, 1) == 4273950213  # Seed= line of the reference's c1 run file


def _compare_dataset(d, packed):
    ds = S.Dataset.from_synth(d, packed=packed)
    od = orc.Data(d)
    L = ds.L
    assert np.array_equal(ds.order(), od.order(L))
    k_or = od.field(1, np.int32)
    assert len(k_or) == L
    return ds, od


@pytest.mark.parametrize("packed", [True, False])
def test_dataset_prepare_matches_oracle_biallelic(packed):
    d = synth.fmodel(11, 150, 900, 3, 0.1, 0.05)
    _compare_dataset(d, packed)


def test_dataset_prepare_matches_oracle_polyploid():
    rng = np.random.default_rng(1)
    d = synth.fmodel(12, 90, 400, 3, 0.08, 0.03, ploidy=np.array([2, 4, 6] * 30),
                     n_alleles=rng.integers(2, 9, 400), anc_alpha=1.0, loc_ids=np.repeat(np.arange(3), 30),
                     loc_alpha=1.0)
    ds, od = _compare_dataset(d, False)
    assert ds.maxploidy == 6
    assert ds.KT == int(od.field(1, np.int32).sum())


@pytest.mark.parametrize("packed", [True, False])
def test_dataset_prepare_matches_oracle_with_filtered_loci(packed):
    """Seven individuals, one without a typed call: many loci are monomorphic
    and dropped, so the sort order maps over the kept loci only; the library's
    order (input indices), allele counts and offsets equal the oracle's."""
    d = synth.fmodel(4, 7, 60, 2, 0.1, 0.05)
    d["G"][:, 3, :] = -1
    ds, od = _compare_dataset(d, packed)
    assert 0 < ds.L < 60
    order = ds.order()
    assert len(np.unique(order)) == ds.L and order.max() < 60
    k_or = od.field(1, np.int32)
    assert ds.KT == int(k_or.sum())
    # every kept locus is polymorphic among the typed calls
    for l in order:
        g = d["G"][l][d["G"][l][:, 0] >= 0]
        assert len(np.unique(g)) > 1


def test_dataset_rejects_bad_input():
    with pytest.raises(B.VpError):
        S.Dataset(np.array([2, 2], np.int32), np.array([2], np.int32), np.array([1, 0], np.int32), 2,
                  G=np.zeros((1, 2, 2), np.int8))  # populations not grouped


def test_all_monomorphic_rejected():
    G = np.zeros((5, 10, 2), np.int8)
    with pytest.raises(B.VpError, match="monomorphic"):
        S.Dataset(np.full(10, 2, np.int32), np.full(5, 2, np.int32), np.zeros(10, np.int32), 1, G=G)


def test_open_without_gpu_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    d = synth.fmodel(3, 40, 100, 2, 0.1, 0.0)
    ds = S.Dataset.from_synth(d)
    with pytest.raises(B.VpError, match="no CUDA device"):
        S.Context(ds)


def test_pack2_roundtrip():
    d = synth.fmodel(5, 37, 50, 2, 0.1, 0.2)
    P = S.pack2(d["G"])
    for l in range(50):
        for i in range(37):
            code = (int(P[l, i // 16]) >> (2 * (i % 16))) & 3
            g = d["G"][l, i]
            assert code == (3 if g[0] < 0 else int(g[0]) + int(g[1]))


def test_server_without_gpu_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    with pytest.raises(B.VpError, match="no CUDA device"):
        S.Server()


def test_vcf_ingest_without_gpu_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    with pytest.raises(B.VpError, match="no CUDA device"):
        S.vcf_pack2(b"1\t1\t.\tA\tC\t.\tPASS\t.\tGT\t0/1\n", 1)


def test_tuner_entry_points_reject_bad_arguments():
    """vp_tune, vp_tc_configure and vp_tc_config_get check their arguments
    before any device call: no chains, a null chain, a null configuration."""
    L = B.lib()
    cfg = B.VpTcConfig()
    none = (ctypes.c_void_p * 1)()
    assert L.vp_tune(none, 0, 1, ctypes.byref(cfg)) == -1   # VP_E_ARG
    assert L.vp_tune(none, 1, 1, ctypes.byref(cfg)) == -1   # VP_E_ARG
    assert L.vp_tc_configure(none, 1, None) == -1   # VP_E_ARG
    assert L.vp_tc_config_get(none, 0, ctypes.byref(cfg)) == -1   # VP_E_ARG
    assert "chain" in L.vp_last_error().decode()


def test_wait_timeout_diagnostic_without_gpu_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    st, after, err = ctypes.c_int32(0), ctypes.c_int32(0), ctypes.c_double(0)
    assert B.lib().vp_debug_gemm_wait_timeout(ctypes.byref(st), ctypes.byref(after), ctypes.byref(err)) != 0
    assert "no CUDA device" in B.lib().vp_last_error().decode()


class _RecordingLib:
    """Stands in for the library: records close/destroy calls by handle."""

    def __init__(self):
        self.calls = []

    def vp_close(self, h):
        self.calls.append(("close", h))
        return 0

    def vp_chain_destroy(self, h):
        self.calls.append(("destroy", h))
        return 0


def _wrappers(n_chains):
    ctx = S.Context.__new__(S.Context)
    ctx.h = 100
    chains = []
    for j in range(n_chains):
        ch = S.Chain.__new__(S.Chain)
        ch.h, ch.ctx = 200 + j, ctx
        chains.append(ch)
    return ctx, chains


@pytest.mark.parametrize("context_first", [True, False])
def test_chain_wrappers_never_destroy_after_their_context_closed(monkeypatch, context_first):
    """The library's vp_close destroys a context's open chains, so a chain
    wrapper closed after its context must not call vp_chain_destroy on the
    freed chain; closed first, it destroys it as usual."""
    fake = _RecordingLib()
    monkeypatch.setattr(B, "lib", lambda: fake)
    ctx, chains = _wrappers(2)
    order = [ctx] + chains if context_first else chains + [ctx]
    for o in order:
        o.close()
        o.close()                              # idempotent
    expect = [("close", 100)] if context_first else [("destroy", 200), ("destroy", 201), ("close", 100)]
    assert fake.calls == expect
    assert ctx.h is None and all(c.h is None for c in chains)


def test_collected_reference_cycle_never_destroys_after_close(monkeypatch):
    """A failing test's traceback can hold a context and its chains in one
    reference cycle; the collector then runs their finalisers in any order.
    Whatever the order, no chain is destroyed after its context closed."""
    import gc
    fake = _RecordingLib()
    monkeypatch.setattr(B, "lib", lambda: fake)
    ctx, chains = _wrappers(3)
    box = {"ctx": ctx, "chains": chains}
    box["self"] = box                          # the cycle
    ctx.cycle = box
    del ctx, chains, box
    gc.collect()
    names = [c[0] for c in fake.calls]
    assert names.count("close") == 1
    closed_at = names.index("close")
    assert "destroy" not in names[closed_at:]


def test_general_locus_filter_rejects_bad_arguments():
    """vp_locus_filter_general checks its sizes before any device call: a
    ploidy outside 1..10, more individuals than its genotype tables' hash
    maps index (2^28), an allele count outside 1..64."""
    import numpy as np
    L = B.lib()
    f = S.locus_filter_spec()
    G = np.zeros(16, dtype=np.int8)
    k = np.array([2], dtype=np.int32)
    bad_k = np.array([65], dtype=np.int32)
    keep = np.zeros(1, dtype=np.uint8)
    call = lambda n_ind, vmax, kk: L.vp_locus_filter_general(G.ctypes.data, None, 1, n_ind, vmax, kk.ctypes.data,
                                                             ctypes.byref(f), 0, keep.ctypes.data, None)
    assert call(4, 11, k) == B.VP_E_ARG
    assert call((1 << 28) + 1, 2, k) == B.VP_E_ARG
    assert "2^28" in L.vp_last_error().decode()
    assert call(4, 2, bad_k) == B.VP_E_ARG
    assert "alleles" in L.vp_last_error().decode()
