"""ctypes handle on the oracle (oracle/_build/liborc.so): test infrastructure.

The oracle is the CPU restatement of the reference's STRUCTURE path, pinned
byte-for-byte to the reference program by tests/test_oracle_golden.py. Tests
compare the GPU library against it, never the other way round.
"""
import ctypes as C
import os
import sys
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBPATH = os.path.join(ROOT, "oracle", "_build", "liborc.so")
_lib = None


class OrcParams(C.Structure):
    _fields_ = [("K", C.c_int32), ("admix", C.c_int32), ("locpriori", C.c_int32), ("fmodel", C.c_int32),
                ("nburnin", C.c_int32), ("nreps", C.c_int32), ("nthinning", C.c_int32), ("nadmburnin", C.c_int32),
                ("writelnl", C.c_int32),
                ("lambda_", C.c_double), ("stdlambda", C.c_double), ("maxlambda", C.c_double),
                ("inferlambda", C.c_int32), ("difflambda", C.c_int32),
                ("alpha", C.c_double), ("stdalpha", C.c_double), ("maxalpha", C.c_double),
                ("alphapriora", C.c_double), ("alphapriorb", C.c_double),
                ("metrofreq", C.c_int32), ("inferalpha", C.c_int32), ("diffalpha", C.c_int32),
                ("uniformalpha", C.c_int32),
                ("r", C.c_double), ("maxr", C.c_double), ("epsr", C.c_double), ("epseta", C.c_double),
                ("epsgamma", C.c_double), ("pmeanf", C.c_double), ("pstdf", C.c_double), ("stdf", C.c_double),
                ("fsame", C.c_int32), ("seed", C.c_uint64)]


def lib():
    global _lib
    if _lib is None:
        subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "all"])
        L = C.CDLL(LIBPATH)
        P = C.c_void_p
        L.orc_data_build.restype = P
        L.orc_data_build.argtypes = [C.c_int32, C.c_int64, C.c_int32, P, P, P, P, C.c_int32]
        L.orc_data_view.restype = P
        L.orc_data_view.argtypes = [P]
        L.orc_data_order.restype = C.POINTER(C.c_int64)
        L.orc_data_order.argtypes = [P]
        L.orc_data_free.argtypes = [P]
        L.orc_chain_new.restype = P
        L.orc_chain_new.argtypes = [P, C.POINTER(OrcParams)]
        L.orc_chain_free.argtypes = [P]
        for f in ["orc_init", "orc_sweep", "orc_arrange", "orc_run", "orc_update_p", "orc_update_q",
                  "orc_update_q_noadmix", "orc_update_q_admix", "orc_update_q_metro", "orc_update_locpriori",
                  "orc_update_z", "orc_update_z_noadmix", "orc_update_z_admix", "orc_update_alpha", "orc_update_a",
                  "orc_update_f", "orc_record"]:
            getattr(L, f).argtypes = [P]
            getattr(L, f).restype = None
        L.orc_record_lnl.argtypes = [P]
        L.orc_record_lnl.restype = C.c_double
        L.orc_loglik_noadmix.argtypes = [P, P]
        L.orc_field.restype = P
        L.orc_field.argtypes = [P, C.c_int, C.POINTER(C.c_int64)]
        L.orc_data_field.restype = P
        L.orc_data_field.argtypes = [P, C.c_int, C.POINTER(C.c_int64)]
        L.orc_m.restype = C.POINTER(C.c_int32)
        L.orc_m.argtypes = [P]
        L.orc_nlnl.restype = C.POINTER(C.c_int32)
        L.orc_nlnl.argtypes = [P]
        L.orc_write_structure.argtypes = [P, C.c_char_p, C.c_int, C.c_int, P, P, P, C.c_int, C.c_int]
        L.orc_write_structure.restype = C.c_int
        L.orc_r.restype = C.POINTER(C.c_double)
        L.orc_r.argtypes = [P]
        L.orc_binaryq.restype = C.POINTER(C.c_int32)
        L.orc_binaryq.argtypes = [P]
        L.orc_sweep_many.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_int]
        L.orc_sweep_many.restype = None
        L.orc_divergence.argtypes = [P, P, C.c_int64, C.c_int64, C.c_int, P, P, P]
        L.orc_divergence.restype = None
        L.orc_vcf_pack2.argtypes = [P, C.c_size_t, C.c_int, P, C.c_int64]
        L.orc_vcf_pack2_ex.argtypes = [P, C.c_size_t, C.c_int, P, C.c_int64, C.POINTER(CallFilter)]
        L.orc_vcf_pack2_ex.restype = C.c_int64
        L.orc_locus_filter_pack2.argtypes = [P, C.c_int64, C.c_int, P, P, P]
        L.orc_locus_filter_general.argtypes = [P, P, C.c_int64, C.c_int, C.c_int, P, P, P, P]
        L.orc_locus_filter_general.restype = None
        L.orc_locus_filter_pack2.restype = None
        L.orc_vcf_pack2.restype = C.c_int64
        L.orc_hash_ulong_c.restype = C.c_uint32
        L.orc_hash_ulong_c.argtypes = [C.c_uint64]
        _lib = L
    return _lib


FIELD_DT = {1: np.float32, 2: np.float32, 3: np.uint16, 4: np.int32, 5: np.int64, 6: np.float64, 7: np.float64,
            10: np.float32, 11: np.float64, 12: np.float64, 13: np.float32, 14: np.float64, 15: np.float64,
            16: np.float64, 17: np.float64, 18: np.float64, 19: np.float64, 20: np.float64, 21: np.int64,
            22: np.float32}
NAMES = dict(FREQ=1, Q=2, Z=3, NI=4, MI=5, LL=6, ALPHA=7, FREQA=10, f=11, F=12, DI=13, METRO=14, ETA=15,
             GAMMA=16, ALPHALOCAL=17, SUMALPHA=18, ROUT=19, LNL=20, MISUM=21, FREQM=22)


class Data:
    def __init__(self, d: dict, n_pop=None):
        G = np.ascontiguousarray(d["G"], dtype=np.int8)
        self.G = G
        self.ploidy = np.ascontiguousarray(d["ploidy"], dtype=np.int32)
        self.k = np.ascontiguousarray(d["k"], dtype=np.int32)
        self.pop = np.ascontiguousarray(d["pop"], dtype=np.int32)
        self.S = int(n_pop if n_pop is not None else self.pop.max() + 1)
        L, N, vmax = G.shape
        self.h = lib().orc_data_build(N, L, vmax, G.ctypes.data, self.ploidy.ctypes.data, self.k.ctypes.data,
                                      self.pop.ctypes.data, self.S)
        self.view = lib().orc_data_view(self.h)
        self.N = N

    def order(self, L):
        return np.ctypeslib.as_array(lib().orc_data_order(self.h), shape=(L,)).copy()

    def field(self, f, dt):
        n = C.c_int64()
        p = lib().orc_data_field(self.view, f, C.byref(n))
        return np.ctypeslib.as_array(C.cast(p, C.POINTER(np.ctypeslib.as_ctypes_type(dt))), shape=(n.value,)).copy()

    def __del__(self):
        if getattr(self, "h", None) and not sys.is_finalizing():
            lib().orc_data_free(self.h)
            self.h = None


def params(K, seed, **kw):
    p = OrcParams()
    p.K = K
    p.nburnin, p.nreps, p.nthinning, p.nadmburnin = 1000, 10000, 10, 500
    p.lambda_, p.stdlambda, p.maxlambda = 1, 0.3, 10
    p.alpha, p.stdalpha, p.maxalpha, p.alphapriora, p.alphapriorb = 1, 0.025, 10, 0.05, 0.001
    p.metrofreq, p.inferalpha, p.diffalpha, p.uniformalpha = 10, 1, 0, 1
    p.r, p.maxr, p.epsr, p.epseta, p.epsgamma = 1, 20, 0.1, 0.025, 0.025
    p.pmeanf, p.pstdf, p.stdf, p.fsame = 0.01, 0.05, 0.05, 0
    p.seed = seed
    alias = dict(f="fmodel", singlef="fsame", stdr="epsr", **{"lambda": "lambda_"})
    for k, v in kw.items():
        setattr(p, alias.get(k, k), int(v) if isinstance(v, bool) else v)
    return p


class Chain:
    def __init__(self, data: Data, p: OrcParams):
        self.data = data
        self.p = p
        self.h = lib().orc_chain_new(data.view, C.byref(p))

    def init(self):
        lib().orc_init(self.h)

    def field(self, name):
        f = NAMES[name]
        n = C.c_int64()
        ptr = lib().orc_field(self.h, f, C.byref(n))
        if not ptr or n.value == 0:
            return np.zeros(0, FIELD_DT[f])
        return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(np.ctypeslib.as_ctypes_type(FIELD_DT[f]))),
                                     shape=(n.value,))

    def get(self, name):
        return self.field(name).copy()

    def set(self, name, v):
        a = self.field(name)
        a[:] = np.asarray(v, dtype=a.dtype).reshape(-1)

    @property
    def m(self):
        return lib().orc_m(self.h)[0]

    @m.setter
    def m(self, v):
        lib().orc_m(self.h)[0] = v

    @property
    def r(self):
        return lib().orc_r(self.h)[0]

    def step(self, name):
        getattr(lib(), "orc_" + name)(self.h)

    def loglik(self):
        out = np.zeros(self.data.N * self.p.K)
        lib().orc_loglik_noadmix(self.h, out.ctypes.data)
        return out

    def __del__(self):
        if getattr(self, "h", None) and not sys.is_finalizing():
            lib().orc_chain_free(self.h)
            self.h = None


def divergence(freqm, k, K, per_locus=False):
    """The reference's H, D (and per-locus H) on mean frequencies [K][KT]."""
    freqm = np.ascontiguousarray(freqm, np.float32)
    k = np.ascontiguousarray(k, np.int32)
    L, KT = len(k), int(k.sum())
    H, D = np.zeros(K), np.zeros((K, K))
    Hl = np.zeros((K, L)) if per_locus else None
    lib().orc_divergence(freqm.ctypes.data, k.ctypes.data, L, KT, K, H.ctypes.data, D.ctypes.data,
                         None if Hl is None else Hl.ctypes.data)
    return dict(H=H, D=D, Hl=Hl)


class CallFilter(C.Structure):
    """The layout of orc_call_filter (and of vp_call_filter)."""
    _fields_ = [(n, C.c_int32) for n in ("dp_b", "dp_min", "dp_max", "gq_b", "gq_min", "gq_max", "ploidy_b",
                                         "ploidy_min", "ploidy_max")]


def call_filter(dp=None, gq=None, ploidy=None):
    cf = CallFilter()
    for name, w in (("dp", dp), ("gq", gq), ("ploidy", ploidy)):
        if w is not None:
            setattr(cf, name + "_b", 1)
            setattr(cf, name + "_min", int(w[0]))
            setattr(cf, name + "_max", int(w[1]))
    return cf


def vcf_pack2(text: bytes, n_ind: int, max_loci: int, calls=None):
    """The oracle's biallelic diploid VCF genotype parse: (packed, lines) or
    raises naming the first unsupported line. calls: a genotype filter
    (call_filter)."""
    packed = np.zeros((max_loci, (n_ind + 15) // 16), np.uint32)
    buf = np.frombuffer(text, dtype=np.uint8)
    n = lib().orc_vcf_pack2_ex(buf.ctypes.data, len(text), n_ind, packed.ctypes.data, max_loci,
                               C.byref(calls) if calls is not None else None)
    if n < 0:
        raise ValueError(f"data line {-n} is not biallelic diploid 0/1 data")
    return packed[:n]


class LocusFilter(C.Structure):
    """The layout of orc_locus_filter (and of vp_locus_filter)."""
    _fields_ = [(n, C.c_int32) for n in ("bmaf_b", "k_b", "n_b", "ptype_b", "he_b", "ho_b", "pic_b", "ae_b", "I_b",
                                         "k_min", "k_max", "n_min", "n_max", "single")] + \
               [(n, C.c_double) for n in ("bmaf_min", "bmaf_max", "ptype_min", "ptype_max", "he_min", "he_max",
                                          "ho_min", "ho_max", "pic_min", "pic_max", "ae_min", "ae_max", "I_min",
                                          "I_max")] + \
               [("pval_b", C.c_int32), ("pval_min", C.c_double), ("pval_max", C.c_double)]


def locus_filter_pack2(packed, n_ind, f):
    packed = np.ascontiguousarray(packed, np.uint32)
    L = packed.shape[0]
    keep = np.zeros(L, np.uint8)
    stats = np.zeros((L, 10))
    lib().orc_locus_filter_pack2(packed.ctypes.data, L, n_ind, C.byref(f), keep.ctypes.data, stats.ctypes.data)
    return keep, stats


def locus_filter_general(G, n_alleles, f, table=None):
    """The oracle's locus filter for the general genotype layout G[L][N][vmax]."""
    G = np.ascontiguousarray(G, np.int8)
    L, N, vmax = G.shape
    k = np.ascontiguousarray(n_alleles, np.int32)
    T = None if table is None else np.ascontiguousarray(table, np.int8)
    keep = np.zeros(L, np.uint8)
    stats = np.zeros((L, 10))
    lib().orc_locus_filter_general(G.ctypes.data, None if T is None else T.ctypes.data, L, N, vmax, k.ctypes.data,
                                   C.byref(f), keep.ctypes.data, stats.ctypes.data)
    return keep, stats
