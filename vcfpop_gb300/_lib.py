"""ctypes binding of libvcfpop_structure.so (declared in include/vcfpop_structure.h).

This is the same binding a Python caller of the reference's STRUCTURE path would
add: plain pointers and sizes, integer status codes turned into exceptions.
The library is the product path; there is no Python or CPU fallback, so a
missing or unloadable library raises.
"""
import ctypes as C
import os

from .build import LIB

VP_RNG_REFERENCE, VP_RNG_COUNTER = 0, 1
VP_FORM_PLAIN, VP_FORM_TC = 0, 1
VP_OK, VP_E_ARG, VP_E_CUDA, VP_E_MEM, VP_E_STATE, VP_E_NODEV = 0, -1, -2, -3, -4, -5

STEP = dict(UPDATEP=1, UPDATEQ=2, LOCPRIORI=3, UPDATEZ=4, ALPHA=5, UPDATEA=6, UPDATEF=7, RECORD=8, NEXT=9,
            LOGLIK=10)
FIELD = dict(FREQ=1, Q=2, Z=3, NI=4, MI=5, LL=6, ALPHA=7, M=8, LNL=9, FREQA=10, FF=11, LOCP=12, DI=13, METRO=14)


class VpInput(C.Structure):
    _fields_ = [("n_ind", C.c_int32), ("n_loc", C.c_int64), ("vmax", C.c_int32),
                ("alleles", C.c_void_p), ("packed2", C.c_void_p), ("ploidy", C.c_void_p),
                ("n_alleles", C.c_void_p), ("popid", C.c_void_p), ("n_pop", C.c_int32),
                ("table_poly", C.c_void_p), ("table_ngeno", C.c_void_p)]


class VpDatasetInfo(C.Structure):
    _fields_ = [("n_ind", C.c_int32), ("n_pop", C.c_int32), ("maxploidy", C.c_int32), ("max_alleles", C.c_int32),
                ("packed2", C.c_int32), ("n_loc", C.c_int64), ("n_alleles_total", C.c_int64), ("coprime", C.c_int64)]


class VpParams(C.Structure):
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
                ("epsgamma", C.c_double),
                ("pmeanf", C.c_double), ("pstdf", C.c_double), ("stdf", C.c_double),
                ("fsame", C.c_int32), ("seed", C.c_uint64), ("rng", C.c_int32), ("form", C.c_int32)]


class VpResult(C.Structure):
    _fields_ = [("K", C.c_int32), ("N", C.c_int32), ("S", C.c_int32), ("nburnin", C.c_int32), ("nreps", C.c_int32),
                ("nthinning", C.c_int32), ("nr", C.c_int32), ("nlnl", C.c_int32), ("rlen", C.c_int32),
                ("KT", C.c_int64), ("seed", C.c_uint64),
                ("rout", C.c_void_p), ("lnl", C.c_void_p), ("Q", C.c_void_p), ("ancestry", C.c_void_p),
                ("freqm", C.c_void_p)]


class VpRequestInfo(C.Structure):
    _fields_ = [("state", C.c_int32), ("rc", C.c_int32), ("sweeps_issued", C.c_int64), ("sweeps_total", C.c_int64),
                ("device_bytes", C.c_int64), ("t_submit", C.c_double), ("t_start", C.c_double),
                ("t_done", C.c_double), ("error", C.c_char * 256)]


VP_REQ_QUEUED, VP_REQ_RUNNING, VP_REQ_DONE, VP_REQ_FAILED = 0, 1, 2, 3


class VpLocusFilter(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("bmaf_b", "k_b", "n_b", "ptype_b", "he_b", "ho_b", "pic_b", "ae_b", "I_b",
                                         "k_min", "k_max", "n_min", "n_max", "single")] + \
               [(n, C.c_double) for n in ("bmaf_min", "bmaf_max", "ptype_min", "ptype_max", "he_min", "he_max",
                                          "ho_min", "ho_max", "pic_min", "pic_max", "ae_min", "ae_max", "I_min",
                                          "I_max")] + \
               [("pval_b", C.c_int32), ("pval_min", C.c_double), ("pval_max", C.c_double)]


class VpCallFilter(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("dp_b", "dp_min", "dp_max", "gq_b", "gq_min", "gq_max", "ploidy_b",
                                         "ploidy_min", "ploidy_max")]


class VpTcConfig(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("bk", "row_tiles", "cols", "piece", "stages", "splits", "group_major",
                                         "count_stages", "count_group_major", "candidates")] + \
               [(n, C.c_float) for n in ("ms_likelihood", "ms_counts", "ms_likelihood_default", "ms_counts_default")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class VpWriteOpts(C.Structure):
    _fields_ = [("prefix", C.c_char_p), ("rep", C.c_int32), ("id", C.c_int32),
                ("ind_names", C.POINTER(C.c_char_p)), ("pop_names", C.POINTER(C.c_char_p)),
                ("loc_names", C.POINTER(C.c_char_p)), ("decimal", C.c_int32), ("comma", C.c_int32),
                ("unix_lb", C.c_int32), ("diversity", C.c_int32)]


class VpError(RuntimeError):
    pass


_lib = None

# every exported symbol of include/vcfpop_structure.h
EXPORTS = ["vp_dataset_prepare", "vp_dataset_info_get", "vp_dataset_order", "vp_dataset_free", "vp_open",
           "vp_close", "vp_sync", "vp_params_default", "vp_run_seed", "vp_chain_create", "vp_chain_destroy",
           "vp_run", "vp_finish", "vp_chain_sizes", "vp_chain_result", "vp_chain_divergence", "vp_chain_step", "vp_chain_get",
           "vp_chain_set", "vp_launch_count", "vp_last_error", "vp_tc_status", "vp_debug_gemm_bf16", "vp_debug_gemm_e4m3", "vp_debug_gemm_time", "vp_stream", "vp_prof_enable", "vp_prof_read", "vp_loglik_packed2",
           "vp_loglik_packed2_noalloc", "vp_server_open", "vp_submit", "vp_poll", "vp_wait", "vp_request_chain",
           "vp_release", "vp_server_close", "vp_vcf_pack2", "vp_locus_filter_pack2", "vp_release_memory",
           "vp_tune", "vp_tc_configure", "vp_tc_config_get", "vp_debug_gemm_wait_timeout", "vp_write_structure",
           "vp_cohort_open", "vp_cohort_set", "vp_cohort_run", "vp_cohort_sync", "vp_cohort_stream",
           "vp_cohort_launches", "vp_cohort_close", "vp_server_set_batching", "vp_server_stats",
           "vp_vcf_parse", "vp_tc_pipeline", "vp_vcf_pack2_ex", "vp_vcf_parse_ex",
           "vp_genotype_table", "vp_locus_filter_general"]


def lib():
    """Load the library (building it first if this tree has not)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        from .build import build
        build()
    L = C.CDLL(LIB)
    P = C.c_void_p
    L.vp_dataset_prepare.argtypes = [C.POINTER(VpInput), C.POINTER(P)]
    L.vp_genotype_table.argtypes = [C.POINTER(VpInput), P, P]
    L.vp_locus_filter_general.argtypes = [P, P, C.c_int64, C.c_int32, C.c_int32, P, C.POINTER(VpLocusFilter), C.c_int,
                                          P, P]
    L.vp_dataset_info_get.argtypes = [P, C.POINTER(VpDatasetInfo)]
    L.vp_dataset_order.argtypes = [P, P]
    L.vp_dataset_free.argtypes = [P]
    L.vp_dataset_free.restype = None
    L.vp_open.argtypes = [P, C.c_int, C.POINTER(P)]
    L.vp_close.argtypes = [P]
    L.vp_sync.argtypes = [P]
    L.vp_params_default.argtypes = [C.POINTER(VpParams)]
    L.vp_params_default.restype = None
    L.vp_run_seed.argtypes = [C.c_int64, C.c_int32]
    L.vp_run_seed.restype = C.c_uint64
    L.vp_chain_create.argtypes = [P, C.POINTER(VpParams), C.POINTER(P)]
    L.vp_chain_destroy.argtypes = [P]
    L.vp_run.argtypes = [C.POINTER(P), C.c_int32, C.c_int32]
    L.vp_finish.argtypes = [C.POINTER(P), C.c_int32]
    L.vp_chain_sizes.argtypes = [P, C.POINTER(VpResult)]
    L.vp_chain_result.argtypes = [P, C.POINTER(VpResult)]
    L.vp_chain_divergence.argtypes = [P, P, P, P]
    L.vp_chain_step.argtypes = [P, C.c_int32]
    L.vp_chain_get.argtypes = [P, C.c_int32, P, C.c_size_t]
    L.vp_chain_set.argtypes = [P, C.c_int32, P, C.c_size_t]
    L.vp_launch_count.argtypes = [P]
    L.vp_launch_count.restype = C.c_int64
    L.vp_last_error.restype = C.c_char_p
    L.vp_tc_status.argtypes = [P]
    L.vp_tune.argtypes = [C.POINTER(P), C.c_int32, C.c_int32, C.POINTER(VpTcConfig)]
    L.vp_tc_configure.argtypes = [C.POINTER(P), C.c_int32, C.POINTER(VpTcConfig)]
    L.vp_tc_config_get.argtypes = [C.POINTER(P), C.c_int32, C.POINTER(VpTcConfig)]
    L.vp_tc_pipeline.argtypes = [P, C.c_int]
    L.vp_debug_gemm_bf16.argtypes = [P, P, P] + [C.c_int32] * 9 + [P]
    L.vp_debug_gemm_time.argtypes = [C.c_int32] * 13 + [P]
    L.vp_debug_gemm_e4m3.argtypes = [P, P] + [C.c_int32] * 7 + [P]
    L.vp_debug_gemm_wait_timeout.argtypes = [C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_double)]
    L.vp_release_memory.argtypes = [C.c_int]
    L.vp_stream.argtypes = [P]
    L.vp_stream.restype = P
    L.vp_prof_enable.argtypes = [P, C.c_int]
    L.vp_prof_read.argtypes = [P, P, P]
    L.vp_loglik_packed2.argtypes = [P, C.c_int32, C.c_int64, P, C.c_int32, P, P]
    L.vp_loglik_packed2_noalloc.argtypes = [P, C.c_int32, C.c_int64, P, C.c_int32, P, P]
    L.vp_server_open.argtypes = [C.c_int, C.c_int64, C.c_int32, C.c_int32, C.POINTER(P)]
    L.vp_submit.argtypes = [P, P, C.POINTER(VpParams), C.POINTER(C.c_int64)]
    L.vp_poll.argtypes = [P, C.c_int64, C.POINTER(VpRequestInfo)]
    L.vp_wait.argtypes = [P, C.c_int64, C.c_double, C.POINTER(VpRequestInfo)]
    L.vp_request_chain.argtypes = [P, C.c_int64, C.POINTER(P)]
    L.vp_release.argtypes = [P, C.c_int64]
    L.vp_server_close.argtypes = [P]
    L.vp_vcf_pack2.argtypes = [P, C.c_size_t, C.c_int32, C.c_int, P, C.c_int64, P, P]
    L.vp_vcf_parse.argtypes = [P, C.c_size_t, C.c_int32, C.c_int32, C.c_int, P, P, P, C.c_int64, P, P]
    L.vp_vcf_pack2_ex.argtypes = [P, C.c_size_t, C.c_int32, C.c_int, P, C.c_int64, P, P, C.POINTER(VpCallFilter)]
    L.vp_vcf_parse_ex.argtypes = [P, C.c_size_t, C.c_int32, C.c_int32, C.c_int, P, P, P, C.c_int64, P, P,
                                  C.POINTER(VpCallFilter)]
    L.vp_locus_filter_pack2.argtypes = [P, C.c_int64, C.c_int32, C.POINTER(VpLocusFilter), C.c_int, P, P]
    L.vp_write_structure.argtypes = [P, C.POINTER(VpWriteOpts)]
    L.vp_cohort_open.argtypes = [C.c_int, C.POINTER(P)]
    L.vp_cohort_set.argtypes = [P, C.POINTER(P), C.c_int32]
    L.vp_cohort_run.argtypes = [P, C.c_int32]
    L.vp_cohort_sync.argtypes = [P]
    L.vp_cohort_stream.argtypes = [P]
    L.vp_cohort_stream.restype = P
    L.vp_cohort_launches.argtypes = [P, C.POINTER(C.c_int32)]
    L.vp_cohort_launches.restype = C.c_int64
    L.vp_cohort_close.argtypes = [P]
    L.vp_server_set_batching.argtypes = [P, C.c_int32]
    L.vp_server_stats.argtypes = [P, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    _lib = L
    return L


def check(rc):
    if rc != 0:
        raise VpError(f"vcfpop_structure error {rc}: {lib().vp_last_error().decode()}")
    return rc
