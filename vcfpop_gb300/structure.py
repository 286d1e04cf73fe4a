"""Python front end of the GB300 STRUCTURE sweep, over the C ABI.

Mirrors the reference's run structure (vcfpop src/structure.cpp): a dataset is
prepared once (CalcBayesian's locus filter/sort), uploaded once, and each
(K, replicate) run is a chain whose MCMC state stays on the GPU. Parameter
names and defaults are those of the -structure_* flags.
"""
from __future__ import annotations

import ctypes as C
import sys

import numpy as np

from . import _lib as B

PARAM_FLAGS = {
    # -structure_* flag -> (field, kind)
    "admix": ("admix", "yn"), "locpriori": ("locpriori", "yn"), "f": ("fmodel", "yn"),
    "nburnin": ("nburnin", int), "nreps": ("nreps", int), "nthinning": ("nthinning", int),
    "nadmburnin": ("nadmburnin", int), "writelnl": ("writelnl", "yn"),
    "lambda": ("lambda_", float), "stdlambda": ("stdlambda", float), "maxlambda": ("maxlambda", float),
    "alpha": ("alpha", float), "inferalpha": ("inferalpha", "yn"), "diffalpha": ("diffalpha", "yn"),
    "uniformalpha": ("uniformalpha", "yn"), "stdalpha": ("stdalpha", float), "maxalpha": ("maxalpha", float),
    "alphapriora": ("alphapriora", float), "alphapriorb": ("alphapriorb", float),
    "metrofreq": ("metrofreq", int), "r": ("r", float), "maxr": ("maxr", float), "stdr": ("epsr", float),
    "epseta": ("epseta", float), "epsgamma": ("epsgamma", float), "pmeanf": ("pmeanf", float),
    "pstdf": ("pstdf", float), "stdf": ("stdf", float), "singlef": ("fsame", "yn"),
}


def params(K: int, seed: int, rng: int = B.VP_RNG_COUNTER, form: int = B.VP_FORM_PLAIN, **kw) -> B.VpParams:
    """Build a run's parameters; keyword names are the -structure_* flag names
    (yes/no may be given as bool, "yes"/"no" or 1/0)."""
    p = B.VpParams()
    B.lib().vp_params_default(C.byref(p))
    p.K = K
    p.seed = seed
    p.rng = rng
    p.form = form
    for k, v in kw.items():
        field, kind = PARAM_FLAGS[k]
        if kind == "yn":
            v = 1 if v in (True, 1, "yes") else 0
        setattr(p, field, kind(v) if kind not in ("yn",) else v)
    return p


def run_seed(g_seed: int, run_id: int) -> int:
    """HashULong(g_seed + run id), the reference's per-run seed."""
    return int(B.lib().vp_run_seed(g_seed, run_id))


def pack2(G: np.ndarray) -> np.ndarray:
    """Pack biallelic diploid calls G[L, N, 2] (allele index, -1 missing) into
    2-bit codes (count of allele 1; 3 = missing), 16 calls per uint32."""
    L, N, _ = G.shape
    code = np.where(G[:, :, 0] < 0, 3, G[:, :, 0].astype(np.int64) + G[:, :, 1].astype(np.int64)).astype(np.uint32)
    Nw = (N + 15) // 16
    pad = np.full((L, Nw * 16), 3, dtype=np.uint32)
    pad[:, :N] = code
    pad = pad.reshape(L, Nw, 16)
    shifts = (np.arange(16, dtype=np.uint32) * 2)[None, None, :]
    return np.bitwise_or.reduce(pad << shifts, axis=2).astype(np.uint32)


class Dataset:
    """A prepared dataset (host side): loci filtered and sorted as the reference does."""

    def __init__(self, ploidy, n_alleles, popid, n_pop, G=None, packed2=None, n_ind=None):
        self._keep = []
        ploidy = np.ascontiguousarray(ploidy, dtype=np.int32)
        n_alleles = np.ascontiguousarray(n_alleles, dtype=np.int32)
        popid = np.ascontiguousarray(popid, dtype=np.int32)
        inp = B.VpInput()
        inp.n_ind = len(ploidy)
        inp.n_loc = len(n_alleles)
        if G is not None:
            G = np.ascontiguousarray(G, dtype=np.int8)
            inp.vmax = G.shape[2]
            inp.alleles = G.ctypes.data
            self._keep.append(G)
        if packed2 is not None:
            packed2 = np.ascontiguousarray(packed2, dtype=np.uint32)
            inp.packed2 = packed2.ctypes.data
            inp.vmax = 2
            self._keep.append(packed2)
        inp.ploidy = ploidy.ctypes.data
        inp.n_alleles = n_alleles.ctypes.data
        inp.popid = popid.ctypes.data
        inp.n_pop = n_pop
        self._keep += [ploidy, n_alleles, popid]
        h = C.c_void_p()
        B.check(B.lib().vp_dataset_prepare(C.byref(inp), C.byref(h)))
        self.h = h
        self._keep = []  # the library copied what it needs
        info = B.VpDatasetInfo()
        B.check(B.lib().vp_dataset_info_get(h, C.byref(info)))
        self.N, self.L, self.KT, self.S = info.n_ind, info.n_loc, info.n_alleles_total, info.n_pop
        self.maxploidy, self.maxK, self.packed2, self.coprime = info.maxploidy, info.max_alleles, info.packed2, info.coprime

    @classmethod
    def from_synth(cls, d: dict, n_pop: int | None = None, packed: bool | None = None):
        G, ploidy, k, pop = d["G"], d["ploidy"], d["k"], d["pop"]
        S = int(n_pop if n_pop is not None else pop.max() + 1)
        if packed is None:
            packed = bool((ploidy == 2).all() and (k == 2).all())
        if packed:
            return cls(ploidy, k, pop, S, packed2=pack2(G))
        return cls(ploidy, k, pop, S, G=G)

    def order(self) -> np.ndarray:
        o = np.zeros(self.L, dtype=np.int64)
        B.check(B.lib().vp_dataset_order(self.h, o.ctypes.data))
        return o

    def __del__(self):
        if getattr(self, "h", None) and not sys.is_finalizing():
            B.lib().vp_dataset_free(self.h)
            self.h = None


class Context:
    """The genotype matrix resident on one GPU."""

    def __init__(self, ds: Dataset, device: int = 0):
        h = C.c_void_p()
        B.check(B.lib().vp_open(ds.h, device, C.byref(h)))
        self.h = h
        self.ds = ds

    def sync(self):
        B.check(B.lib().vp_sync(self.h))

    def launches(self) -> int:
        return int(B.lib().vp_launch_count(self.h))

    def tc_pipeline(self, share: int) -> None:
        """Tensor-core sweeps by allele ranges, UpdateP of one range beside
        the likelihood contraction of the range before it with at most
        `share` UpdateP blocks beside a contraction CTA (1-8), or in one pass
        (0)."""
        B.check(B.lib().vp_tc_pipeline(self.h, int(share)))

    def close(self):
        if getattr(self, "h", None):
            B.lib().vp_close(self.h)
            self.h = None

    def __del__(self):
        # at interpreter exit the CUDA runtime may already be gone; the process
        # teardown releases the device memory
        if not sys.is_finalizing():
            self.close()


_DT = {1: np.float32, 2: np.float32, 3: np.uint16, 4: np.int32, 5: np.int32, 6: np.float64, 7: np.float64,
       8: np.int32, 9: np.float64, 10: np.float32, 11: np.float64, 12: np.float64, 13: np.float32, 14: np.float64}


class Chain:
    """One (K, replicate) run with device-resident state."""

    def __init__(self, ctx: Context, p: B.VpParams):
        h = C.c_void_p()
        B.check(B.lib().vp_chain_create(ctx.h, C.byref(p), C.byref(h)))
        self.h = h
        self.ctx = ctx
        self.p = p

    def _size(self, field):
        ds = self.ctx.ds
        K = self.p.K
        return {1: K * ds.KT, 2: ds.N * K, 3: ds.N, 4: K * ds.KT, 5: ds.N * K, 6: ds.N * K, 7: K, 8: 1, 9: 1,
                10: ds.KT, 11: 2 * K, 12: 1 + K + 2 * ds.S * K + ds.S, 13: ds.S * K, 14: ds.N}[field]

    def get(self, name: str) -> np.ndarray:
        f = B.FIELD[name]
        a = np.zeros(self._size(f), dtype=_DT[f])
        B.check(B.lib().vp_chain_get(self.h, f, a.ctypes.data, a.nbytes))
        return a

    def set(self, name: str, value) -> None:
        f = B.FIELD[name]
        a = np.ascontiguousarray(value, dtype=_DT[f]).reshape(-1)
        B.check(B.lib().vp_chain_set(self.h, f, a.ctypes.data, a.nbytes))

    def step(self, name: str) -> None:
        B.check(B.lib().vp_chain_step(self.h, B.STEP[name]))

    def run(self, nsweeps: int) -> None:
        arr = (C.c_void_p * 1)(self.h)
        B.check(B.lib().vp_run(arr, 1, nsweeps))

    def result(self, final: bool = False) -> dict:
        """Results; `final` (after vp_finish) adds the normalised ancestry."""
        return chain_result(self.h, final)

    def write(self, prefix: str, rep: int, run_id: int, ind_names, pop_names, loc_names, decimal: int = 5,
              diversity: bool = False, comma: bool = False, unix: bool = False) -> None:
        """The run's result files in the reference's format (vp_write_structure);
        loc_names in the dataset's input locus order."""
        def arr(names):
            return (C.c_char_p * len(names))(*[n.encode() for n in names])
        keep = [arr(ind_names), arr(pop_names), arr(loc_names)]
        o = B.VpWriteOpts(prefix.encode(), rep, run_id, keep[0], keep[1], keep[2], decimal, int(comma), int(unix),
                          int(diversity))
        B.check(B.lib().vp_write_structure(self.h, C.byref(o)))

    def divergence(self, per_locus: bool = False) -> dict:
        """Heterozygosity H[K], net nucleotide distance D[K, K] (and the
        per-locus heterozygosity [K, L]) of a finished chain, on the device."""
        K, L = self.p.K, self.ctx.ds.L
        H, D = np.zeros(K), np.zeros((K, K))
        Hl = np.zeros((K, L)) if per_locus else None
        B.check(B.lib().vp_chain_divergence(self.h, H.ctypes.data, D.ctypes.data,
                                            None if Hl is None else Hl.ctypes.data))
        return dict(H=H, D=D, Hl=Hl)

    def close(self):
        # a closed context has already destroyed its chains (the collector may
        # finalise the context first when both sit in one reference cycle)
        if getattr(self, "h", None):
            if getattr(self.ctx, "h", None):
                B.lib().vp_chain_destroy(self.h)
            self.h = None

    def __del__(self):
        if not sys.is_finalizing():
            self.close()


def call_filter(dp=None, gq=None, ploidy=None):
    """The genotype filter of -f_dp, -f_gq, -f_ploidy: each window a (min,
    max) pair or None (not used). None when no window is used."""
    if dp is None and gq is None and ploidy is None:
        return None
    cf = B.VpCallFilter()
    for name, w in (("dp", dp), ("gq", gq), ("ploidy", ploidy)):
        if w is not None:
            setattr(cf, name + "_b", 1)
            setattr(cf, name + "_min", int(w[0]))
            setattr(cf, name + "_max", int(w[1]))
    return cf


def vcf_pack2(text: bytes, n_ind: int, device: int = 0, calls=None):
    """Parse the data lines of a biallelic diploid VCF on the device: returns
    (packed [L][ceil(N/16)] uint32 2-bit codes, line offsets [L + 1]). calls:
    a genotype filter (call_filter) applied as the calls are decoded."""
    buf = np.frombuffer(text, dtype=np.uint8)
    # a well-formed line holds 9 fields and n_ind calls of 3 bytes, each after a tab
    L = len(text) // (4 * n_ind + 17) + 1
    packed = np.empty((L, (n_ind + 15) // 16), np.uint32)
    starts = np.empty(L + 1, np.int64)
    n = C.c_int64()
    B.check(B.lib().vp_vcf_pack2_ex(buf.ctypes.data, len(text), n_ind, device, packed.ctypes.data, max(L, 1),
                                    starts.ctypes.data, C.byref(n), C.byref(calls) if calls is not None else None))
    return packed[:n.value], starts[:n.value + 1]


def vcf_parse(text: bytes, n_ind: int, vmax: int, device: int = 0, calls=None):
    """Parse the data lines of a VCF of any ploidy and allele count on the
    device: (alleles [L][N][vmax] int8, ascending, -1 missing; alleles per
    locus [L]; ploidy of each sample's first call [N]; line offsets [L + 1]).
    calls: a genotype filter (call_filter)."""
    buf = np.frombuffer(text, dtype=np.uint8)
    n = C.c_int64()
    B.check(B.lib().vp_vcf_parse(buf.ctypes.data, len(text), n_ind, vmax, device, None, None, None, 0, None,
                                 C.byref(n)))
    L = n.value
    G = np.empty((L, n_ind, vmax), np.int8)
    k = np.empty(L, np.int32)
    ploidy = np.empty(n_ind, np.int32)
    starts = np.empty(L + 1, np.int64)
    if L:
        B.check(B.lib().vp_vcf_parse_ex(buf.ctypes.data, len(text), n_ind, vmax, device, G.ctypes.data,
                                        k.ctypes.data, ploidy.ctypes.data, L, starts.ctypes.data, C.byref(n),
                                        C.byref(calls) if calls is not None else None))
    return G, k, ploidy, starts


LOCUS_STATS = ("n", "k", "ptype", "bmaf", "he", "ho", "pic", "ae", "I", "pval")


def locus_filter_spec(single: bool = True, **windows) -> B.VpLocusFilter:
    """A locus filter from -f_* windows given as name=(min, max), names as in
    LOCUS_STATS (bmaf, k, n, ptype, he, ho, pic, ae, I, pval)."""
    f = B.VpLocusFilter()
    f.single = 1 if single else 0
    for name, (lo, hi) in windows.items():
        if name not in LOCUS_STATS:
            raise ValueError(f"unknown locus statistic {name}")
        setattr(f, f"{name}_b", 1)
        setattr(f, f"{name}_min", lo)
        setattr(f, f"{name}_max", hi)
    return f


def locus_filter(packed: np.ndarray, n_ind: int, f: B.VpLocusFilter, device: int = 0):
    """Per-locus statistics and the pass flags of the -f_* locus filter on the
    device: (keep [L] uint8, stats [L][10])."""
    packed = np.ascontiguousarray(packed, np.uint32)
    L = packed.shape[0]
    keep = np.zeros(L, np.uint8)
    stats = np.zeros((L, len(LOCUS_STATS)))
    B.check(B.lib().vp_locus_filter_pack2(packed.ctypes.data, L, n_ind, C.byref(f), device, keep.ctypes.data,
                                          stats.ctypes.data))
    return keep, stats


def locus_filter_general(G: np.ndarray, n_alleles, f: B.VpLocusFilter, table=None, device: int = 0):
    """The -f_* locus filter on the device for the general genotype layout
    G[L][N][vmax] (any ploidy, up to 64 alleles per locus): (keep [L] uint8,
    stats [L][10]). table: the calls before the genotype filter (same
    layout), whose first appearances order each locus' genotype table."""
    G = np.ascontiguousarray(G, np.int8)
    L, N, vmax = G.shape
    k = np.ascontiguousarray(n_alleles, np.int32)
    T = None if table is None else np.ascontiguousarray(table, np.int8)
    keep = np.zeros(L, np.uint8)
    stats = np.zeros((L, len(LOCUS_STATS)))
    B.check(B.lib().vp_locus_filter_general(G.ctypes.data, None if T is None else T.ctypes.data, L, N, vmax,
                                            k.ctypes.data, C.byref(f), device, keep.ctypes.data, stats.ctypes.data))
    return keep, stats


def chain_result(h, final: bool = False) -> dict:
    r = B.VpResult()
    B.check(B.lib().vp_chain_sizes(h, C.byref(r)))
    out = dict(rout=np.zeros(r.rlen), lnl=np.zeros(max(r.nlnl, 0)), Q=np.zeros(r.N * r.K, np.float32),
               ancestry=np.zeros(r.N * r.K), freqm=np.zeros(r.K * r.KT, np.float32))
    r.rout, r.lnl, r.Q = out["rout"].ctypes.data, out["lnl"].ctypes.data, out["Q"].ctypes.data
    r.ancestry = out["ancestry"].ctypes.data if final else None
    r.freqm = out["freqm"].ctypes.data
    if not final:
        del out["ancestry"]
    B.check(B.lib().vp_chain_result(h, C.byref(r)))
    out.update(K=r.K, N=r.N, nr=r.nr, nburnin=r.nburnin, nreps=r.nreps, nthinning=r.nthinning, seed=r.seed)
    return out


_STATE = {B.VP_REQ_QUEUED: "queued", B.VP_REQ_RUNNING: "running", B.VP_REQ_DONE: "done", B.VP_REQ_FAILED: "failed"}


class Server:
    """Many independent runs on one device: a native scheduler thread admits
    runs by device-memory budget and overlaps them on per-run streams
    (vp_server_open / vp_submit / vp_poll / vp_wait / vp_release)."""

    def __init__(self, device: int = 0, mem_budget: int = 0, max_active: int = 0, chunk: int = 0,
                 batching: bool = True):
        h = C.c_void_p()
        B.check(B.lib().vp_server_open(device, mem_budget, max_active, chunk, C.byref(h)))
        B.check(B.lib().vp_server_set_batching(h, int(batching)))
        self.h = h

    def submit(self, ds: Dataset, p: B.VpParams) -> int:
        rid = C.c_int64()
        # the request keeps its own reference to the dataset: freeing `ds`
        # before the run ends is safe
        B.check(B.lib().vp_submit(self.h, ds.h, C.byref(p), C.byref(rid)))
        return rid.value

    @staticmethod
    def _info(i: B.VpRequestInfo) -> dict:
        return dict(state=_STATE[i.state], rc=i.rc, sweeps_issued=i.sweeps_issued, sweeps_total=i.sweeps_total,
                    device_bytes=i.device_bytes, t_submit=i.t_submit, t_start=i.t_start, t_done=i.t_done,
                    error=i.error.decode())

    def poll(self, rid: int) -> dict:
        i = B.VpRequestInfo()
        B.check(B.lib().vp_poll(self.h, rid, C.byref(i)))
        return self._info(i)

    def wait(self, rid: int, timeout: float = -1.0) -> dict:
        i = B.VpRequestInfo()
        B.check(B.lib().vp_wait(self.h, rid, timeout, C.byref(i)))
        return self._info(i)

    def chain(self, rid: int):
        h = C.c_void_p()
        B.check(B.lib().vp_request_chain(self.h, rid, C.byref(h)))
        return h

    def result(self, rid: int, final: bool = True) -> dict:
        return chain_result(self.chain(rid), final)

    def release(self, rid: int) -> None:
        B.check(B.lib().vp_release(self.h, rid))

    def stats(self) -> dict:
        """Kernel launches the scheduler queued and the run-sweeps they carry."""
        a, b = C.c_int64(), C.c_int64()
        B.check(B.lib().vp_server_stats(self.h, C.byref(a), C.byref(b)))
        return dict(launches=int(a.value), run_sweeps=int(b.value))

    def close(self):
        if getattr(self, "h", None):
            B.lib().vp_server_close(self.h)
            self.h = None

    def __del__(self):
        if not sys.is_finalizing():
            self.close()


def finish(chains: list[Chain]) -> None:
    """Run every remaining sweep and Arrange() the results."""
    arr = (C.c_void_p * len(chains))(*[c.h for c in chains])
    B.check(B.lib().vp_finish(arr, len(chains)))


def _chain_array(chains):
    return (C.c_void_p * len(chains))(*[c.h for c in chains])


class Cohort:
    """Chains of any contexts swept together in shared launches (vp_cohort_*)."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        B.check(B.lib().vp_cohort_open(device, C.byref(h)))
        self.h = h
        self.members = []

    def set(self, chains) -> None:
        arr = (C.c_void_p * max(1, len(chains)))(*[c.h for c in chains])
        B.check(B.lib().vp_cohort_set(self.h, arr, len(chains)))
        self.members = list(chains)

    def run(self, nsweeps: int) -> None:
        B.check(B.lib().vp_cohort_run(self.h, nsweeps))

    def sync(self) -> None:
        B.check(B.lib().vp_cohort_sync(self.h))

    def launches(self) -> tuple[int, int]:
        """(launches queued so far, launches of one sweep)"""
        per = C.c_int32()
        n = B.lib().vp_cohort_launches(self.h, C.byref(per))
        return int(n), int(per.value)

    def close(self) -> None:
        if getattr(self, "h", None):
            B.check(B.lib().vp_cohort_close(self.h))
            self.h = None
            self.members = []

    def __del__(self):
        if getattr(self, "h", None) and not sys.is_finalizing():
            B.lib().vp_cohort_close(self.h)
            self.h = None


def tune(chains: list[Chain], effort: int = 1) -> dict:
    """Autotune the batched sweep of these tensor-core chains (vp_tune): the
    chosen launch configuration and the device times before and after."""
    cfg = B.VpTcConfig()
    B.check(B.lib().vp_tune(_chain_array(chains), len(chains), effort, C.byref(cfg)))
    return cfg.as_dict()


def tc_configure(chains: list[Chain], **kw) -> None:
    """Set the batch's launch configuration (vp_tc_configure); unnamed fields
    keep their current values."""
    cfg = B.VpTcConfig()
    B.check(B.lib().vp_tc_config_get(_chain_array(chains), len(chains), C.byref(cfg)))
    for k, v in kw.items():
        setattr(cfg, k, v)
    B.check(B.lib().vp_tc_configure(_chain_array(chains), len(chains), C.byref(cfg)))


def tc_config(chains: list[Chain]) -> dict:
    cfg = B.VpTcConfig()
    B.check(B.lib().vp_tc_config_get(_chain_array(chains), len(chains), C.byref(cfg)))
    return cfg.as_dict()


def run_chains(chains: list[Chain], nsweeps: int | None = None) -> None:
    """Advance chains that share a context together (shared launches, one graph)."""
    arr = (C.c_void_p * len(chains))(*[c.h for c in chains])
    if nsweeps is None:
        B.check(B.lib().vp_finish(arr, len(chains)))
    else:
        B.check(B.lib().vp_run(arr, len(chains), nsweeps))
