#!/usr/bin/env python
"""Benchmark of the STRUCTURE sweep on GB300: genotype-cluster updates/s.

Default workload (c3, the batched K-sweep the metric is quoted on): N = 10,000
diploid individuals x L = 200,000 biallelic SNPs drawn from an 8-population
F-model (F = 0.03, ancestral frequencies Beta(0.5, 0.5), 1% missing calls),
seeded synthetic data; K = 1..10 x 10 replicates = 100 no-admixture chains
sharing the genotype matrix. One step = one MCMC sweep of all 100 chains; one
genotype-cluster update = one (individual, locus, cluster) term, so a step is
N * L * sum(K) updates.

  --form tc     the tensor-core split-BF16 form (default)
  --form plain  the FP32 SIMT form of the same sweep
  --workload c1|c2|c4   one chain of that case (vcfpop_gb300/workloads.py);
                a step is one sweep
  --workload c5 the serving stream: independent runs arriving at 50/s through
                the native scheduler, against the same runs one at a time
  --impl reference  the CPU baseline: the reference algorithm's C port on the
                host cores on a bounded sample of the workload

Prints one JSON line (rank 0).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_IND, N_LOC, N_POP, FST, MISSING = 10_000, 200_000, 8, 0.03, 0.01
KS = [k for k in range(1, 11) for _ in range(10)]
METRIC = "genotype-cluster updates/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=150)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--form", default="tc", choices=["tc", "plain"])
    ap.add_argument("--loci", type=int, default=N_LOC)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-sweeps", type=int, default=10)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="c3: skip the plain-form comparison sweeps")
    ap.add_argument("--tune", type=int, default=2, choices=[0, 1, 2],
                    help="c3: autotuner effort for the batched contractions before warm-up (0: built-in defaults)")
    ap.add_argument("--workload", default="c3", choices=["c1", "c2", "c3", "c4", "c5"])
    ap.add_argument("--no-serving", action="store_true", help="c3: skip the c5 serving stream")
    ap.add_argument("--no-extra", action="store_true", help="c3: skip the compact c2 and c4 results")
    ap.add_argument("--no-labels", action="store_true", help="c3: skip the FP64 label check")
    ap.add_argument("--requests", type=int, default=120, help="c5: runs in the stream")
    ap.add_argument("--c5-scale", type=float, default=0.1, help="c5: scale of the N, L and run-length ranges")
    return ap.parse_args()


# ---------------------------------------------------------------- data
def gen_packed_gpu(seed, N, L, P=N_POP, F=FST, miss=MISSING, chunk=20_000):
    """F-model genotypes drawn on the GPU, returned as host 2-bit codes [L][ceil(N/16)]."""
    import torch
    torch.manual_seed(seed)
    dev = "cuda"
    g = torch.Generator(device=dev).manual_seed(seed)
    anc = torch.distributions.Beta(torch.full((L,), 0.5, device=dev), torch.full((L,), 0.5, device=dev)).sample()
    f = (1 - F) / F
    a = (anc * f).clamp_min(1e-3).expand(P, L)
    b = ((1 - anc) * f).clamp_min(1e-3).expand(P, L)
    popf = torch.distributions.Beta(a, b).sample()  # [P, L]
    pop = (torch.arange(N, device=dev) * P) // N
    Nw = (N + 15) // 16
    out = np.empty((L, Nw), dtype=np.uint32)
    shifts = (torch.arange(16, device=dev, dtype=torch.int64) * 2)
    for l0 in range(0, L, chunk):
        l1 = min(L, l0 + chunk)
        p = popf[:, l0:l1][pop]  # [N, Lc]
        u = torch.rand((2, N, l1 - l0), device=dev, generator=g)
        c1 = (u[0] < p).to(torch.int64) + (u[1] < p).to(torch.int64)
        m = torch.rand((N, l1 - l0), device=dev, generator=g) < miss
        code = torch.where(m, torch.full_like(c1, 3), c1).t().contiguous()  # [Lc, N]
        pad = torch.full((l1 - l0, Nw * 16), 3, dtype=torch.int64, device=dev)
        pad[:, :N] = code
        words = (pad.view(l1 - l0, Nw, 16) << shifts).sum(dim=2).to(torch.int64) & 0xFFFFFFFF
        out[l0:l1] = words.to(torch.int64).cpu().numpy().astype(np.uint32)
    return out, pop.cpu().numpy().astype(np.int32)


def gen_sample_cpu(seed, N, L):
    from vcfpop_gb300 import synth
    return synth.fmodel(seed, N, L, N_POP, FST, MISSING)


# ---------------------------------------------------------------- clocks
class Clocks:
    """nvidia-smi clock and throttle-reason samples taken during the timed region."""

    def __init__(self, index=0):
        self.rows, self.proc, self.index = [], None, index

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for n, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


# ---------------------------------------------------------------- CPU leg
class CpuPort:
    """The oracle -- the reference algorithm's C port -- on N x `loci` of the
    same F-model, 100 chains, one chain at a time per host thread (the
    reference's run-level parallelism)."""

    def __init__(self, loci, chains_k, seed=7, threads=None, n_ind=N_IND):
        from tests import orc
        import ctypes as C
        self.orc = orc
        self.n_ind = n_ind
        self.d = gen_sample_cpu(seed, n_ind, loci)
        self.od = orc.Data(self.d)
        self.L = self.od.field(1, np.int32).size
        self.threads = threads or os.cpu_count()
        self.chains = [orc.Chain(self.od, orc.params(K, 1000 + j, admix=0, nadmburnin=0, nburnin=1000, nreps=2000))
                       for j, K in enumerate(chains_k)]
        self.arr = (C.c_void_p * len(self.chains))(*[c.h for c in self.chains])
        self.upd_sweep = n_ind * self.L * sum(chains_k)
        orc.lib().orc_sweep_many(self.arr, len(self.chains), 0, self.threads, 1)   # init

    def sweep(self, n=1):
        t0 = time.perf_counter()
        self.orc.lib().orc_sweep_many(self.arr, len(self.chains), n, self.threads, 0)
        return time.perf_counter() - t0


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    # a step: one sweep of the 100 chains on 1,000 individuals x 8,000 loci of
    # the same F-model (each chain's frequency table at the size of about 4% of
    # the full one, so its reads leave the core's caches as at full size)
    cp = CpuPort(8000, KS, n_ind=1000)
    cores, L = cp.threads, cp.L
    for _ in range(args.warmup):
        cp.sweep()
    t = [cp.sweep() for _ in range(args.steps)]
    rates = [cp.upd_sweep / x for x in t]
    value = float(np.median(rates))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "updates/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * float(np.median(t)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64/f32 (reference CPU)",
            "data": "synthetic F-model, seeded",
            "config": {"workload": f"K-sweep K=1..10 x 10 replicates, sample N={cp.n_ind} of {N_IND} individuals "
                                   f"x L={L} of {N_LOC} loci", "chains": len(KS), "host_threads": cores},
            "cpu_baseline": {"value": value, "unit": "updates/s", "cores": cores, "kind": "port",
                             "sample": f"N={cp.n_ind} x {L} loci, 100 chains, one sweep per step"},
            "e2e": {"value": value, "unit": "updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- VCF ingest
def vcf_text(packed, N):
    """A biallelic diploid VCF data section (GT only) with the given calls."""
    L = packed.shape[0]
    shifts = (np.arange(16, dtype=np.uint32) * 2)
    codes = ((packed[:, :, None] >> shifts) & 3).reshape(L, -1)[:, :N].astype(np.uint8)
    table = np.frombuffer(b"0/0\t0/1\t1/1\t./.\t", dtype=np.uint8).reshape(4, 4)
    body = table[codes]                          # [L, N, 4]
    body[:, -1, 3] = ord("\n")
    out = bytearray()
    for l in range(L):
        out += f"1\t{l + 1}\t.\tA\tC\t.\tPASS\t.\tGT\t".encode()
        out += body[l].tobytes()
    return bytes(out)


def vcf_ingest(packed, N, args, rank, loci=20000):
    """Device ingest of a VCF data section of `loci` lines of this dataset
    (vp_vcf_pack2: upload from host memory, parse, packed matrix back) and,
    as its CPU baseline, the oracle's line-by-line parse on one core."""
    from vcfpop_gb300 import structure as S
    text = vcf_text(packed[:loci], N)
    S.vcf_pack2(text[:text.index(b"\n", len(text) // 8) + 1], N)   # warm-up on whole lines (context, allocator)
    reps = 3
    t0 = time.perf_counter()
    for _ in range(reps):
        got, _ = S.vcf_pack2(text, N)
    dev = (time.perf_counter() - t0) / reps
    out = {"what": f"{loci} lines x {N} samples, {len(text) / 1e9:.2f} GB of VCF text, GT only",
           "device_ms": dev * 1e3, "device_gbs": len(text) / dev / 1e9,
           "exact": bool(np.array_equal(got, packed[:loci]))}
    if rank == 0 and not args.no_cpu_baseline:
        from tests import orc
        t0 = time.perf_counter()
        ref = orc.vcf_pack2(text, N, loci)
        cpu = time.perf_counter() - t0
        out.update({"cpu_baseline_ms": cpu * 1e3, "cpu_baseline_gbs": len(text) / cpu / 1e9,
                    "cpu_baseline_kind": "port (the oracle's line-by-line GT parse, one core)",
                    "cpu_equal": bool(np.array_equal(ref, got))})
    return out


# ---------------------------------------------------------------- locus filter
def locus_filter_leg(packed, N, args, rank, sample=20000):
    """The -f_* locus filter (vp_locus_filter_pack2: statistics and pass
    flags of every locus, copies included) on the whole packed matrix, and as
    its CPU baseline the oracle's restatement on one core over a sample of
    loci, scaled to the same count."""
    from vcfpop_gb300 import structure as S
    f = S.locus_filter_spec(bmaf=(0.05, 0.5), ptype=(0.9, 1.0), he=(0.05, 0.5))
    S.locus_filter(packed[:1000], N, f)               # warm-up
    reps = 3
    t0 = time.perf_counter()
    for _ in range(reps):
        keep, _ = S.locus_filter(packed, N, f)
    dev = (time.perf_counter() - t0) / reps
    out = {"what": f"{packed.shape[0]} loci x {N} samples ({packed.nbytes / 1e9:.2f} GB packed), "
                   f"-f_bmaf=[0.05,0.5] -f_ptype=[0.9,1] -f_he=[0.05,0.5]",
           "device_ms": dev * 1e3, "device_gbs": packed.nbytes / dev / 1e9, "kept": int(keep.sum())}
    if rank == 0 and not args.no_cpu_baseline:
        from tests import orc
        o = orc.LocusFilter()
        for name, _ in orc.LocusFilter._fields_:
            setattr(o, name, getattr(f, name))
        n = min(sample, packed.shape[0])
        t0 = time.perf_counter()
        okeep, _ = orc.locus_filter_pack2(packed[:n], N, o)
        cpu = (time.perf_counter() - t0) * packed.shape[0] / n
        out.update({"cpu_baseline_ms": cpu * 1e3, "cpu_baseline_kind": f"port (the oracle on one core, {n} loci, scaled)",
                    "cpu_equal_on_sample": bool(np.array_equal(okeep, keep[:n]))})
    return out


def locus_filter_general_leg(d, with_cpu, sample=2000):
    """The -f_* locus filter for the general genotype layout
    (vp_locus_filter_general: each locus' genotype table in order of first
    appearance, its statistics and the HWE test, copies included) on a
    polyploid multiallelic dataset, and as its CPU baseline the oracle on one
    core over a sample of loci, scaled to the same count."""
    from vcfpop_gb300 import structure as S
    f = S.locus_filter_spec(single=False, k=(3, 8), he=(0.3, 0.9), ptype=(0.9, 1.0), pval=(0.001, 1.0))
    G, k = d["G"], d["k"]
    S.locus_filter_general(G[:200], k[:200], f)        # warm-up
    reps = 3
    t0 = time.perf_counter()
    for _ in range(reps):
        keep, _ = S.locus_filter_general(G, k, f)
    dev = (time.perf_counter() - t0) / reps
    L, N, vmax = G.shape
    out = {"what": f"{L} loci x {N} individuals (ploidy {sorted(set(int(x) for x in d['ploidy']))}, "
                   f"{int(k.min())}-{int(k.max())} alleles; {G.nbytes / 1e9:.2f} GB of allele copies), "
                   f"-f_k=[3,8] -f_he=[0.3,0.9] -f_ptype=[0.9,1] -f_pval=[0.001,1]",
           "device_ms": dev * 1e3, "device_gbs": G.nbytes / dev / 1e9, "kept": int(keep.sum())}
    if with_cpu:
        from tests import orc
        o = orc.LocusFilter()
        for name, _ in orc.LocusFilter._fields_:
            setattr(o, name, getattr(f, name))
        n = min(sample, L)
        t0 = time.perf_counter()
        okeep, _ = orc.locus_filter_general(G[:n], k[:n], o)
        cpu = (time.perf_counter() - t0) * L / n
        out.update({"cpu_baseline_ms": cpu * 1e3, "cpu_baseline_kind": f"port (the oracle on one core, {n} loci, scaled)",
                    "cpu_equal_on_sample": bool(np.array_equal(okeep, keep[:n]))})
    return out


# ---------------------------------------------------------------- output reductions
def output_reductions(ctx, ds, args, rank):
    """WriteStructure's heterozygosity / net-distance / per-locus diversity
    reductions of one finished K = 10 chain on this dataset: the device call
    (vp_chain_divergence, copies included) and, as its CPU baseline, the
    reference loops restated in the oracle, on the same mean frequencies."""
    from vcfpop_gb300 import structure as S
    K = 10
    ch = S.Chain(ctx, S.params(K, S.run_seed(1, 999), admix=0, nadmburnin=0, nburnin=0, nreps=1, nthinning=1))
    S.finish([ch])
    ch.divergence(per_locus=True)
    t0 = time.perf_counter()
    reps = 5
    for _ in range(reps):
        got = ch.divergence(per_locus=True)
    dev_ms = (time.perf_counter() - t0) / reps * 1e3
    out = {"what": f"H[K], D[K,K] and per-locus H[K,L] of one K={K} chain, L={ds.L}, KT={ds.KT}",
           "device_ms": dev_ms, "kernels": "k_divergence_pairs, k_divergence_finish, k_heterozygosity"}
    if rank == 0 and not args.no_cpu_baseline:
        from tests import orc
        fm = ch.result(final=True)["freqm"]
        k = np.full(ds.L, 2, np.int32)
        t0 = time.perf_counter()
        ref = orc.divergence(fm, k, K, per_locus=True)
        out["cpu_baseline_ms"] = (time.perf_counter() - t0) * 1e3
        out["cpu_baseline_kind"] = "port (the reference's WriteStructure loops, one core)"
        out["max_abs_diff_D"] = float(np.abs(ref["D"] - got["D"]).max())
    ch.close()
    return out


# ---------------------------------------------------------------- c1, c2, c4: one chain
SINGLE_DESC = {
    "c1": "N=200 diploids, 3 pops, L=2,000 biallelic SNPs, F=0.1, 5% missing; K=3 no-admixture, 1,000 + 2,000 sweeps",
    "c2": "N=2,000 x L=50,000 biallelic, Q~Dir(0.5), F=0.05, 2% missing; K=5 admixture, alpha inferred, 5,000 + 10,000 sweeps",
    "c4": "N=5,000 autopolyploids (ploidy 2/4/6 at 2:1:1), 20 locations, L=20,000 loci with 2-8 alleles, F=0.08, "
          "3% missing; K=8 admixture + location prior, 10,000 + 10,000 sweeps",
}


def _single(name):
    from vcfpop_gb300 import workloads as W
    d, run = getattr(W, name)()
    run = dict(run)
    K = run.pop("K")
    return d, K, run


def _sweep_bytes(ds, K, admix):
    """Algorithmic bytes of the dominant kernel per launch: the genotype
    matrix, the frequencies (and counts written back for the admixture form)
    and the per-individual outputs."""
    bg = ds.L * ((ds.N + 15) // 16) * 4 if ds.packed2 else ds.L * ds.N * ds.maxploidy
    if admix:
        return bg + 8 * K * ds.KT + 8 * ds.N * K
    return bg + 4 * K * ds.KT + 8 * ds.N * K


def cpu_sample_single(d, K, run, budget_s=12.0, max_sweeps=400):
    """The oracle (the reference algorithm's C port), one chain on one core,
    on the full dataset of the case: sweeps until about budget_s seconds."""
    from tests import orc
    import ctypes as C
    od = orc.Data(d)
    L = od.field(1, np.int32).size
    p = orc.params(K, 1000, **run)
    ch = orc.Chain(od, p)
    arr = (C.c_void_p * 1)(ch.h)
    orc.lib().orc_sweep_many(arr, 1, 0, 1, 1)
    orc.lib().orc_sweep_many(arr, 1, 1, 1, 0)        # warm-up sweep
    n, t0 = 0, time.perf_counter()
    while n < max_sweeps and (time.perf_counter() - t0) < budget_s:
        orc.lib().orc_sweep_many(arr, 1, 1, 1, 0)
        n += 1
    dt = time.perf_counter() - t0
    N = d["G"].shape[1]
    return N * L * K * n / dt, n, dt


def bench_single(args):
    import torch
    import ctypes as C
    from vcfpop_gb300 import _lib as B
    from vcfpop_gb300 import structure as S
    from vcfpop_gb300 import replicas as R
    rank, world, local = R.env()
    torch.cuda.set_device(local)
    R.init("nccl")
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    d, K, run = _single(args.workload)
    ds = S.Dataset.from_synth(d)
    admix = bool(run.get("admix"))
    upd = ds.N * ds.L * K
    lib = B.lib()
    ctx = S.Context(ds, local)
    ch = S.Chain(ctx, S.params(K, S.run_seed(1, 1), **run))
    arr = (C.c_void_p * 1)(ch.h)
    total = run["nburnin"] + run["nreps"] + (run.get("nadmburnin", 0) if not admix and not run.get("locpriori") else 0)
    B.check(lib.vp_run(arr, 1, args.warmup))
    ctx.sync()
    # time enough sweeps for a region of about a second (within the run's length)
    t0 = time.perf_counter()
    B.check(lib.vp_run(arr, 1, 5))
    ctx.sync()
    per = (time.perf_counter() - t0) / 5
    left = total - args.warmup - 5 - 8
    n = int(max(args.steps, min(left, 1.0 / max(per, 1e-6))))
    n = max(1, min(n, left))
    stream = torch.cuda.ExternalStream(lib.vp_stream(ctx.h))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = ctx.launches()
    n = int(R.max_over_ranks(n) if world > 1 else n)   # every replica times the same number of sweeps
    R.barrier()
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        e0.record(stream)
        B.check(lib.vp_run(arr, 1, n))
        e1.record(stream)
        torch.cuda.synchronize()
        R.barrier()
    launches = ctx.launches() - l0
    ms = R.max_over_ranks(e0.elapsed_time(e1)) / n
    # dominant kernel: average launch duration over a few more sweeps
    lib.vp_prof_enable(ctx.h, 1)
    dom, cnt = 0.0, 0
    msv, nl = C.c_double(), C.c_int32()
    for _ in range(6):
        B.check(lib.vp_run(arr, 1, 1))
        B.check(lib.vp_prof_read(ctx.h, C.byref(msv), C.byref(nl)))
        dom += msv.value
        cnt += nl.value
    dom_ms = dom / max(cnt, 1)
    byts = _sweep_bytes(ds, K, admix)
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = byts / (dom_ms / 1e3) / 1e9
    l2 = byts < 120e6
    roof = {"bound": "hbm", "kernel": "k_update_z_admix_ctr (per-copy labels)" if admix else "k_loglik / k_loglik_fma (likelihood stream)",
            "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in peaks else "fallback", "traffic": None,
            "avg_launch_ms": dom_ms, "bytes_per_launch": byts,
            "note": "working set fits in L2 (129 MB): the fraction is against HBM bandwidth but served from L2" if l2 else ""}
    ch.close()
    ctx.close()

    # end to end: open from host buffers, create, run, read results, close
    e2e = None
    if not args.no_e2e:
        r2 = dict(run)
        full = args.workload == "c1"
        if not full:
            r2["nburnin"], r2["nreps"] = 500, 500
        e_sweeps = r2["nburnin"] + r2["nreps"] + (r2.get("nadmburnin", 0) if not admix and not r2.get("locpriori") else 0)
        times = []
        for it in range(2):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            cx = S.Context(ds, local)
            c2 = S.Chain(cx, S.params(K, S.run_seed(1, 2), **r2))
            S.finish([c2])
            res = c2.result(final=True)
            c2.close()
            cx.close()
            times.append(time.perf_counter() - t0)
            assert np.isfinite(res["rout"]).all()
        tt = R.max_over_ranks(min(times[1:]) if len(times) > 1 else times[0])
        h2d = (ds.L * ((ds.N + 15) // 16) * 4 if ds.packed2 else ds.L * ds.N * ds.maxploidy) + ds.L * 12 + ds.N * 12
        d2h = 8 * (ds.N * K * 2 + ds.KT * K) + 64
        e2e = {"value": upd * e_sweeps * world / tt, "unit": "updates/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "step": ("one complete run" if full else f"a run of {e_sweeps} sweeps (500 + 500)") +
                       ": open context from pinned host buffers, create the chain, every sweep, Arrange, read Q, "
                       "ancestry, mean frequencies and lnL, close", "time_to_result_s": tt}
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        v, ns, dt = cpu_sample_single(d, K, run)
        cpu = {"value": v, "unit": "updates/s", "cores": 1, "kind": "port",
               "sample": f"the same dataset, one chain on one host core, {ns} sweeps in {dt:.1f} s"}
    line = {"metric": METRIC, "value": upd * world / (ms / 1e3), "unit": "updates/s", "n_gpus": world, "steps": n,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (lnP(D) accumulations in f64)",
            "data": "synthetic F-model, seeded (vcfpop_gb300/workloads.py)",
            "config": {"workload": f"{args.workload}: {SINGLE_DESC[args.workload]}; one step = one sweep",
                       "form": "plain", "chains": 1, "updates_per_step": upd,
                       "l2": "working set smaller than L2" if l2 else "inputs larger than L2",
                       "parallelism": f"replicas x{world}" if world > 1 else "1 GPU"},
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clk.summary()}
    if rank == 0:
        print(json.dumps(line), flush=True)
    R.finish()


def single_compact(name, local, peaks, cpu_budget_s=0.0):
    """One chain of c2 or c4 in brief, for the default line: device-timed
    sweeps (CUDA events on the library's stream, about half a second), the
    dominant kernel's HBM roofline, and optionally the oracle on one core."""
    import torch
    import ctypes as C
    from vcfpop_gb300 import _lib as B
    from vcfpop_gb300 import structure as S
    t_data = time.perf_counter()
    d, K, run = _single(name)
    t_data = time.perf_counter() - t_data
    ds = S.Dataset.from_synth(d)
    admix = bool(run.get("admix"))
    upd = ds.N * ds.L * K
    lib = B.lib()
    ctx = S.Context(ds, local)
    ch = S.Chain(ctx, S.params(K, S.run_seed(1, 1), **run))
    arr = (C.c_void_p * 1)(ch.h)
    B.check(lib.vp_run(arr, 1, 3))
    ctx.sync()
    t0 = time.perf_counter()
    B.check(lib.vp_run(arr, 1, 5))
    ctx.sync()
    n = int(max(10, min(400, 0.5 / max((time.perf_counter() - t0) / 5, 1e-6))))
    stream = torch.cuda.ExternalStream(lib.vp_stream(ctx.h))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    l0 = ctx.launches()
    e0.record(stream)
    B.check(lib.vp_run(arr, 1, n))
    e1.record(stream)
    torch.cuda.synchronize()
    launches = ctx.launches() - l0
    ms = e0.elapsed_time(e1) / n
    lib.vp_prof_enable(ctx.h, 1)
    dom, cnt = 0.0, 0
    msv, nl = C.c_double(), C.c_int32()
    for _ in range(6):
        B.check(lib.vp_run(arr, 1, 1))
        B.check(lib.vp_prof_read(ctx.h, C.byref(msv), C.byref(nl)))
        dom += msv.value
        cnt += nl.value
    dom_ms = dom / max(cnt, 1)
    byts = _sweep_bytes(ds, K, admix)
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = byts / (dom_ms / 1e3) / 1e9
    ch.close()
    ctx.close()
    out = {"workload": f"{name}: {SINGLE_DESC[name]}; one step = one sweep", "value": upd / (ms / 1e3),
           "unit": "updates/s", "ms_per_step": ms, "steps": n, "warmup": 3, "gpu_launches": launches,
           "roofline": {"bound": "hbm", "kernel": "k_update_z_admix_ctr (per-copy labels)" if admix else
                        "k_loglik / k_loglik_fma (likelihood stream)", "achieved": achieved, "peak": peak, "unit": "GB/s",
                        "frac": achieved / peak, "avg_launch_ms": dom_ms, "bytes_per_launch": byts},
           "data_seconds": t_data}
    if cpu_budget_s > 0:
        v, ns, dt = cpu_sample_single(d, K, run, budget_s=cpu_budget_s)
        out["cpu_baseline"] = {"value": v, "unit": "updates/s", "cores": 1, "kind": "port",
                               "sample": f"the same dataset, one chain on one host core, {ns} sweeps in {dt:.1f} s"}
    if name == "c4":
        out["locus_filter_general"] = locus_filter_general_leg(d, cpu_budget_s > 0)
    return out


def reference_single(args):
    if int(os.environ.get("RANK", "0")) != 0:
        return
    d, K, run = _single(args.workload)
    v, ns, dt = cpu_sample_single(d, K, run, budget_s=60.0, max_sweeps=max(args.steps, 1))
    N, L = d["G"].shape[1], d["G"].shape[0]
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "updates/s", "n_gpus": args.gpus,
            "steps": ns, "warmup": 1, "ms_per_step": 1e3 * dt / ns, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64/f32 (reference CPU)", "data": "synthetic F-model, seeded",
            "config": {"workload": f"{args.workload}: {SINGLE_DESC[args.workload]}; one step = one sweep",
                       "chains": 1, "host_threads": 1},
            "cpu_baseline": {"value": v, "unit": "updates/s", "cores": 1, "kind": "port",
                             "sample": f"one chain, {ns} sweeps in {dt:.1f} s"},
            "e2e": {"value": v, "unit": "updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- c5: serving
def serve_stream(args, local, rank):
    """The c5 stream through the serving loop (vp_server): every run submitted
    at its arrival time with up to 64 active, then the same runs one at a
    time (the reference's schedule). Returns both summaries, the runs, their
    updates and the bytes uploaded."""
    from vcfpop_gb300 import structure as S
    from vcfpop_gb300 import workloads as W
    reqs = W.c5_requests(args.requests, seed=5 + rank, scale=args.c5_scale)
    runs = []
    for q in reqs:
        packed, pop = gen_packed_gpu(q["seed"], q["N"], q["L"], P=q["pops"], F=0.05, miss=0.02)
        ds = S.Dataset(np.full(q["N"], 2, np.int32), np.full(q["L"], 2, np.int32), pop, q["pops"], packed2=packed)
        p = S.params(q["K"], q["seed"], admix=q["admix"], nburnin=q["nburnin"], nreps=q["nreps"], nadmburnin=0)
        runs.append((q, ds, p))
    upd = sum(ds.N * ds.L * q["K"] * (q["nburnin"] + q["nreps"]) for q, ds, p in runs)
    h2d = sum(ds.L * ((ds.N + 15) // 16) * 4 + ds.L * 12 + ds.N * 12 for q, ds, p in runs)

    def serve(max_active, batching=True):
        srv = S.Server(device=local, max_active=max_active, chunk=16, batching=batching)
        ids = [None] * len(runs)
        t0 = time.perf_counter()

        def feeder():
            for j, (q, ds, p) in enumerate(runs):
                dt = t0 + q["t"] - time.perf_counter()
                if dt > 0:
                    time.sleep(dt)
                ids[j] = srv.submit(ds, p)

        th = threading.Thread(target=feeder)
        th.start()
        th.join()
        infos, lnl = [], []
        for rid in ids:
            inf = srv.wait(rid, 600.0)
            assert inf["state"] == "done", inf
            lnl.append(srv.result(rid)["rout"][0])
            infos.append(inf)
            srv.release(rid)
        st = srv.stats()
        srv.close()
        ttr = np.array([i["t_done"] - i["t_submit"] for i in infos])
        span = max(i["t_done"] for i in infos) - min(i["t_submit"] for i in infos)
        assert np.isfinite(lnl).all()
        return {"updates_per_s": upd / span, "makespan_s": span, "p50_s": float(np.percentile(ttr, 50)),
                "p99_s": float(np.percentile(ttr, 99)), "max_active": max_active, "batching": batching,
                "launches": st["launches"], "run_sweeps": st["run_sweeps"],
                "launches_per_run_sweep": st["launches"] / max(1, st["run_sweeps"])}

    conc = serve(64)
    conc["unbatched"] = serve(64, batching=False)
    alone = serve(1)
    return conc, alone, runs, upd, h2d


def c5_desc(args, nruns):
    return (f"c5 serving: {nruns} independent runs, Poisson arrivals at 50/s, N log-uniform "
            f"[{int(100 * args.c5_scale)}, {int(20000 * args.c5_scale)}], L log-uniform "
            f"[{int(1000 * args.c5_scale)}, {int(200000 * args.c5_scale)}], K uniform 2..12, "
            f"admixture p=0.5, {int(2000 * args.c5_scale)}-{int(20000 * args.c5_scale)} sweeps "
            f"(ranges x{args.c5_scale} of the full case)")


def bench_serve(args):
    import torch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    torch.cuda.set_device(local)
    with Clocks(local) as clk:
        conc, alone, runs, upd, h2d = serve_stream(args, local, rank)
    line = {"metric": METRIC, "value": conc["updates_per_s"] * world, "unit": "updates/s", "n_gpus": world,
            "steps": 1, "warmup": 0, "ms_per_step": conc["makespan_s"] * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (lnP(D) accumulations in f64)",
            "data": "synthetic F-model per run, seeded",
            "config": {"workload": c5_desc(args, len(runs)) + "; one step = the whole stream",
                       "form": "plain", "runs": len(runs), "updates_per_step": upd, "parallelism": "1 GPU"},
            "serving": {"concurrent": conc, "one_at_a_time": alone},
            "roofline": None, "cpu_baseline": None,
            "e2e": {"value": conc["updates_per_s"] * world, "unit": "updates/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": 8 * len(runs),
                    "step": "every run submitted from host buffers at its arrival time, uploaded, run, lnL read back"},
            "gpu_launches": None, "clocks": clk.summary()}
    if rank == 0:
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- GPU leg
def lnp_rel_err(chains):
    """Largest relative error of the chains' last lnP(D) against the FP64
    evaluation of the same state: without admixture Record's lnP(D) is the sum
    of Ni x ln p over clusters, loci and alleles."""
    worst = 0.0
    for c in chains:
        ni, p = c.get("NI"), c.get("FREQ")
        m = ni > 0
        want = float(np.sum(ni[m].astype(np.float64) * np.log(p[m].astype(np.float64))))
        worst = max(worst, abs(float(c.get("LNL")[0]) - want) / abs(want))
    return worst


def recorded_lnp_err(ctx):
    """The batched form's recorded lnP(D) on the full-size data: 10 chains
    (K = 1..10) that record every sweep, against the FP64 evaluation."""
    from vcfpop_gb300 import _lib as B
    from vcfpop_gb300 import structure as S
    chains = [S.Chain(ctx, S.params(K, S.run_seed(2, K), form=B.VP_FORM_TC, admix=0, nadmburnin=0, nburnin=0,
                                    nreps=100, nthinning=1, writelnl=1)) for K in range(1, 11)]
    S.run_chains(chains, 2)
    err = lnp_rel_err(chains)
    for c in chains:
        c.close()
    return err


def philox_first_uniform(seed, a, b):
    """The first float uniform of the device's counter stream Philox(seed;
    a, b, 0) for an array of b: Philox-4x32-10 (Salmon et al., SC 2011) with
    the key (seed low, seed high) and the counter (a, b, 0, 0), its first
    output word w mapped to ((w >> 8) + 1) / 2^24."""
    M = np.uint64(0xFFFFFFFF)
    k0, k1 = np.uint64(seed & 0xFFFFFFFF), np.uint64((seed >> 32) & 0xFFFFFFFF)
    b = np.asarray(b, np.uint64)
    c0, c1 = np.full_like(b, a), b.copy()
    c2, c3 = np.zeros_like(b), np.zeros_like(b)
    for _ in range(10):
        p0 = np.uint64(0xD2511F53) * c0
        p1 = np.uint64(0xCD9E8D57) * c2
        c0, c1, c2, c3 = ((p1 >> np.uint64(32)) ^ c1 ^ k0) & M, p1 & M, ((p0 >> np.uint64(32)) ^ c3 ^ k1) & M, p0 & M
        k0 = (k0 + np.uint64(0x9E3779B9)) & M
        k1 = (k1 + np.uint64(0xBB67AE85)) & M
    return ((c0 >> np.uint64(8)).astype(np.float64) + 1.0) / 16777216.0


def label_parity(chains, packed, loci_chunk=4000):
    """The likelihoods and labels of the chains' last sweep against FP64: for
    every (chain, individual, cluster) LL is evaluated again in FP64 from the
    packed genotypes and the frequencies that sweep used (torch FP64 GEMMs on
    the device, per chunk of loci), and a label is drawn from each FP64 row
    with the same counter-stream uniform the sweep used (the categorical draw
    of both forms: weights exp(LL - max), below 2^-23 floored at 1e-10, plus
    1e-10 per cluster). Returns the largest |LL - LL64| and relative error,
    and the labels that differ from the FP64 draws."""
    import torch
    dev = "cuda"
    N = int(chains[0].ctx.ds.N)
    L = packed.shape[0]
    Ks = [c.p.K for c in chains]
    R = sum(Ks)
    lnp = torch.empty((R, 2 * L), dtype=torch.float64, device=dev)
    r = 0
    for c, K in zip(chains, Ks):
        f = torch.from_numpy(c.get("FREQ").reshape(K, 2 * L)).to(dev).double()
        lnp[r:r + K] = torch.where(f > 0, torch.log(f.clamp_min(1e-300)), torch.full_like(f, -709.0895657128241))
        r += K
    LL64 = torch.zeros((N, R), dtype=torch.float64, device=dev)
    shifts = torch.arange(16, dtype=torch.int64, device=dev) * 2
    for l0 in range(0, L, loci_chunk):
        l1 = min(L, l0 + loci_chunk)
        w = torch.from_numpy(packed[l0:l1].view(np.int32)).to(dev).to(torch.int64) & 0xFFFFFFFF
        code = ((w[:, :, None] >> shifts) & 3).reshape(l1 - l0, -1)[:, :N].t()          # [N, Lc]
        typed = code != 3
        c1 = torch.where(typed, code, torch.zeros_like(code)).double()
        c0 = torch.where(typed, 2 - code, torch.zeros_like(code)).double()
        LL64 += c0 @ lnp[:, 2 * l0:2 * l1:2].t() + c1 @ lnp[:, 2 * l0 + 1:2 * l1:2].t()
    out = {"draws": 0, "flips": 0, "ll_max_abs_err": 0.0, "ll_max_rel_err": 0.0}
    r = 0
    for c, K in zip(chains, Ks):
        ll = torch.from_numpy(c.get("LL").reshape(N, K)).to(dev)
        ref = LL64[:, r:r + K]
        err = (ll - ref).abs()
        out["ll_max_abs_err"] = max(out["ll_max_abs_err"], float(err.max()))
        out["ll_max_rel_err"] = max(out["ll_max_rel_err"], float((err / ref.abs()).max()))
        m_used = int(c.get("M")[0]) - 1
        u = torch.from_numpy(philox_first_uniform(int(c.p.seed), 3 | (m_used << 4), np.arange(N))).to(dev)
        d = ref - ref.max(dim=1, keepdim=True).values
        e = torch.where(d < -23, torch.full_like(d, 1e-10), torch.exp(d))
        cum = torch.cumsum(e, dim=1)
        t = u * (cum[:, -1] + 1e-10 * K)
        z64 = torch.where((t[:, None] < cum).any(dim=1), (t[:, None] >= cum).sum(dim=1), torch.full_like(t, K - 1,
                                                                                                     dtype=torch.int64))
        z = torch.from_numpy(c.get("Z").astype(np.int64)).to(dev)
        out["flips"] += int((z != z64).sum())
        out["draws"] += N
        r += K
    del LL64, lnp
    torch.cuda.empty_cache()
    return out


def plain_form_leg(ctx, lib, upd_step, world, peaks, packed=None, steps=3):
    """The same 100 chains in the plain FP32 form on the same context: a few
    timed sweeps (after one untimed), for the batched-over-plain ratio; then
    two sweeps with the likelihood stream's launches timed (its HBM
    roofline) and, given the packed genotypes, the FP64 label check."""
    import ctypes as C
    import torch
    from vcfpop_gb300 import _lib as B
    from vcfpop_gb300 import replicas as R
    from vcfpop_gb300 import structure as S
    chains = [S.Chain(ctx, S.params(K, S.run_seed(1, j + 1), form=B.VP_FORM_PLAIN, admix=0, nadmburnin=0,
                                    nburnin=1000, nreps=2000)) for j, K in enumerate(KS)]
    arr = (C.c_void_p * len(chains))(*[c.h for c in chains])
    B.check(lib.vp_run(arr, len(chains), 1))
    ctx.sync()
    stream = torch.cuda.ExternalStream(lib.vp_stream(ctx.h))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    R.barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    B.check(lib.vp_run(arr, len(chains), steps))
    e1.record(stream)
    torch.cuda.synchronize()
    ms = R.max_over_ranks(e0.elapsed_time(e1)) / steps
    err = lnp_rel_err(chains)
    # the likelihood stream (k_loglik, one launch per chain and sweep)
    lib.vp_prof_enable(ctx.h, 1)
    msv, nl = C.c_double(), C.c_int32()
    dom, cnt = 0.0, 0
    for _ in range(2):
        B.check(lib.vp_run(arr, len(chains), 1))
        B.check(lib.vp_prof_read(ctx.h, C.byref(msv), C.byref(nl)))
        dom += msv.value
        cnt += nl.value
    dom_ms = dom / max(cnt, 1)
    L = ctx.ds.L
    byts = sum(N_IND * L / 4 + 4 * K * 2 * L + 8 * N_IND * K for K in KS) / len(KS)
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = byts / (dom_ms / 1e3) / 1e9
    roof = {"bound": "hbm", "kernel": "k_loglik / k_loglik_fma (likelihood stream)", "achieved": achieved, "peak": peak,
            "unit": "GB/s", "frac": achieved / peak, "avg_launch_ms": dom_ms, "bytes_per_launch": byts,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in peaks else "fallback",
            "bytes_what": "packed genotypes N*L/4 + frequencies 4*K*2L + per-individual output 8*N*K, per chain"}
    labels = label_parity(chains, packed) if packed is not None else None
    for c in chains:
        c.close()
    return {"value": upd_step * world / (ms / 1e3), "ms_per_step": ms, "steps": steps, "warmup": 1,
            "lnp_rel_err_max": err, "roofline": roof, "labels": labels}


def main():
    args = parse()
    if args.impl == "reference":
        if args.workload in ("c1", "c2", "c4"):
            return reference_single(args)
        if args.workload == "c5":
            print(json.dumps({"impl": "reference", "unavailable": "c5 reference arm: the reference runs one request "
                              "at a time; bench.py --workload c5 reports that schedule on the GPU beside the "
                              "concurrent one"}), flush=True)
            return
        return reference_arm(args)
    if args.workload in ("c1", "c2", "c4"):
        return bench_single(args)
    if args.workload == "c5":
        return bench_serve(args)
    import torch
    import ctypes as C
    from vcfpop_gb300 import replicas as R
    rank, world, local = R.env()
    torch.cuda.set_device(local)
    R.init("nccl")
    from vcfpop_gb300 import _lib as B
    from vcfpop_gb300 import structure as S

    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        peaks = {}
    form = B.VP_FORM_TC if args.form == "tc" else B.VP_FORM_PLAIN

    packed, pop = gen_packed_gpu(1234 + rank, N_IND, args.loci)
    ingest = vcf_ingest(packed, N_IND, args, rank)
    lfilter = locus_filter_leg(packed, N_IND, args, rank)
    ds = S.Dataset(np.full(N_IND, 2, np.int32), np.full(args.loci, 2, np.int32), pop, N_POP, packed2=packed)
    order = ds.order()
    if not np.array_equal(order, np.arange(len(order))):
        packed = packed[order]      # the dataset's locus order (monomorphic loci dropped)
    sumK = sum(KS)
    upd_step = N_IND * ds.L * sumK

    def make(ctx):
        return [S.Chain(ctx, S.params(K, S.run_seed(1, j + 1), form=form, admix=0, nadmburnin=0,
                                      nburnin=1000, nreps=2000)) for j, K in enumerate(KS)]

    ctx = S.Context(ds, local)
    chains = make(ctx)
    lib = B.lib()
    tuning = None
    if form == B.VP_FORM_TC and args.tune:
        t0 = time.perf_counter()
        tuning = S.tune(chains, args.tune)
        tuning["effort"] = args.tune
        tuning["seconds"] = time.perf_counter() - t0
    lib.vp_prof_enable(ctx.h, 1)
    arr = (C.c_void_p * len(chains))(*[c.h for c in chains])
    for _ in range(args.warmup):
        B.check(lib.vp_run(arr, len(chains), 1))
    ctx.sync()
    stream = torch.cuda.ExternalStream(lib.vp_stream(ctx.h))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    R.barrier()
    torch.cuda.synchronize()
    l0 = ctx.launches()
    dom_ms, dom_n = 0.0, 0
    ms, nl = C.c_double(), C.c_int32()
    with Clocks(local) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            B.check(lib.vp_run(arr, len(chains), 1))
            B.check(lib.vp_prof_read(ctx.h, C.byref(ms), C.byref(nl)))
            dom_ms += ms.value
            dom_n += nl.value
        e1.record(stream)
        torch.cuda.synchronize()
        R.barrier()
    launches = ctx.launches() - l0
    total_ms = R.max_over_ranks(e0.elapsed_time(e1))   # the slowest replica sets the job time
    tc_err = lib.vp_tc_status(ctx.h)
    ms_step = total_ms / args.steps
    value = upd_step * world / (ms_step / 1e3)

    # dominant kernel roofline
    dom_avg_ms = dom_ms / max(dom_n, 1)
    if form == B.VP_FORM_TC:
        A = 2 * ds.L
        flops = 2.0 * N_IND * A * sumK  # algorithmic: the likelihood contraction [N x A] . [A x sumK]
        achieved = flops / (dom_avg_ms / 1e3) / 1e12
        # the burst peak when the timed region ran at the maximum clock with
        # no throttle reason (a short region), else the sustained one
        ck = clk.summary()
        at_max = (ck.get("sm_mhz") and ck.get("sm_max_mhz") and ck["sm_mhz"] >= 0.97 * ck["sm_max_mhz"]
                  and not ck.get("reasons"))
        key = "bf16_tflops" if at_max else "bf16_tflops_sustained"
        peak = peaks.get(key, 1900.0 if at_max else 1700.0)
        rpad = (sumK + 191) // 192 * 192
        executed = 2 * flops * (rpad / sumK) / (dom_avg_ms / 1e3) / 1e12
        roof = {"bound": "tensor", "kernel": "k_gemm_bf16 (likelihood contraction)", "achieved": achieved,
                "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "peak_source": f"MEASURED_PEAKS.json {key}" if key in peaks else "fallback",
                "peak_choice": "burst: timed region at max SM clock, no throttle reason" if at_max else
                               "sustained: clocks below max or a throttle reason during the timed region",
                "executed_tflops": executed, "executed_frac": executed / peak,
                "executed_what": "hi and lo MMAs over the cluster rows padded to 192-row column groups",
                "traffic": None}
    else:
        # per likelihood-stream launch (one chain): packed genotypes + frequencies + per-individual output
        byts = [N_IND * ds.L / 4 + 4 * K * 2 * ds.L + 8 * N_IND * K for K in KS]
        achieved = sum(byts) / len(byts) / (dom_avg_ms / 1e3) / 1e9
        peak = peaks.get("hbm_gbs", 6800.0)
        roof = {"bound": "hbm", "kernel": "k_loglik / k_loglik_fma (likelihood stream)", "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in peaks else "fallback", "traffic": None}
    roof["avg_launch_ms"] = dom_avg_ms
    # the batched UpdateP of the same sweeps: Dirichlet draws per second, from
    # CUDA events around its launch inside the sweep graph (after the timed
    # steps; the chains run a few more of their sweeps)
    updatep = pipeline = None
    if form == B.VP_FORM_TC:
        # the same chains' next sweeps by allele ranges (UpdateP of one range
        # beside the contraction of the range before it), for comparison
        # with the timed one-pass sweeps
        cfg = S.tc_config(chains)
        ctx.tc_pipeline(2)
        for _ in range(2):
            B.check(lib.vp_run(arr, len(chains), 1))
        ctx.sync()
        n1 = 10
        e0.record(stream)
        for _ in range(n1):
            B.check(lib.vp_run(arr, len(chains), 1))
        e1.record(stream)
        torch.cuda.synchronize()
        ranges_ms = e0.elapsed_time(e1) / n1
        ctx.tc_pipeline(0)
        pipeline = {"ms_per_step": ms_step, "ms_per_step_by_ranges": ranges_ms, "ranges": cfg["splits"],
                    "what": "timed sweeps in one pass (UpdateP of every locus, then the whole likelihood "
                            "contraction) against the same chains' next sweeps by allele ranges (UpdateP of a "
                            "range beside the contraction slice of the range before it, at most 2 UpdateP "
                            "blocks beside a contraction CTA)"}
        lib.vp_prof_enable(ctx.h, 2)
        up_ms = []
        for it in range(4):
            B.check(lib.vp_run(arr, len(chains), 1))
            B.check(lib.vp_prof_read(ctx.h, C.byref(ms), C.byref(nl)))
            if it:
                up_ms.append(ms.value / max(nl.value, 1))
        lib.vp_prof_enable(ctx.h, 1)
        draws = sumK * ds.KT
        up = float(np.median(up_ms))
        # algorithmic bytes: Ni read, Freq and the two W rows written (4 bytes each per draw, W 2 + 2)
        up_bytes = draws * (4 + 4 + 2 + 2)
        updatep = {"kernel": "tc::k_update_p_tc", "gamma_draws_per_sweep": draws, "avg_launch_ms": up,
                   "draws_per_s": draws / (up / 1e3), "gbs": up_bytes / (up / 1e3) / 1e9,
                   "bound": "instruction issue (Philox-4x32-10 block + two Marsaglia-Tsang gammas per biallelic locus)"}
    tfile = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tfile):
        try:
            tr = json.load(open(tfile)).get(args.form)
            if tr:
                roof["traffic"] = tr["bytes_per_launch_at_full_size"]
        except Exception:
            pass
    sweep_ll_err = lnp_rel_err(chains)
    labels = None
    if not args.no_labels:
        t0 = time.perf_counter()
        labels = {args.form: label_parity(chains, packed)}
        labels["seconds"] = time.perf_counter() - t0
    for c in chains:
        c.close()
    lnp_err = None
    if form == B.VP_FORM_TC:
        lnp_err = {"max": recorded_lnp_err(ctx), "chains": 10, "bound": 1e-6,
                   "what": "lnP(D) recorded by the batched form on full-size data (K=1..10, thinning 1, 2 sweeps)",
                   "against": "FP64 sum of Ni x ln p over the same state, Record's lnP(D) (structure.cpp:1902-1938)",
                   "sweep_ll_max": sweep_ll_err,
                   "sweep_ll_what": "the 100 timed chains' per-sweep sum of the likelihood contraction (FP32 "
                                    "accumulation), used for the label draws only"}
    plain = None
    if form == B.VP_FORM_TC and not args.no_plain:
        plain = plain_form_leg(ctx, lib, upd_step, world, peaks, packed if labels is not None else None)
        lnp_err["plain_max"] = plain.pop("lnp_rel_err_max")
        if labels is not None:
            labels["plain"] = plain.pop("labels")
    elif form != B.VP_FORM_TC:
        lnp_err = {"max": sweep_ll_err, "chains": len(chains), "bound": 1e-6,
                   "against": "FP64 sum of Ni x ln p over the same state, Record's lnP(D) (structure.cpp:1902-1938)"}
    outputs = output_reductions(ctx, ds, args, rank)
    ctx.close()

    # ---- end to end through the C ABI: upload from pinned host memory, create
    # the chains, sweep, read every chain's likelihood back, close
    e2e_steps, e2e_ms = 5, []   # the median of five: single steps vary by several ms
    h2d = ds.L * ((N_IND + 15) // 16) * 4 + ds.L * (4 + 8) + N_IND * (8 + 4)
    d2h = 8 * len(KS)
    for it in range(0 if args.no_e2e else e2e_steps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        cx = S.Context(ds, local)
        cs = make(cx)
        a2 = (C.c_void_p * len(cs))(*[c.h for c in cs])
        B.check(lib.vp_run(a2, len(cs), args.e2e_sweeps))
        lnl = [c.get("LNL")[0] for c in cs]
        for c in cs:
            c.close()
        cx.close()
        dt = time.perf_counter() - t0
        if it:
            e2e_ms.append(dt * 1e3)
        assert all(np.isfinite(lnl))
    e2e_value = upd_step * args.e2e_sweeps * world / (np.median(e2e_ms) / 1e3) if e2e_ms else None
    # one more step, untimed, with a wait after each phase: where the time
    # outside the sweeps goes (the first vp_run call builds the batch's
    # operands and counts the initial labels before its sweep)
    phases = None
    if not args.no_e2e:
        ph, t = {}, time.perf_counter()

        def mark(name):
            nonlocal t
            torch.cuda.synchronize()
            now = time.perf_counter()
            ph[name] = round((now - t) * 1e3, 3)
            t = now

        cx = S.Context(ds, local)
        mark("open_upload")
        cs = make(cx)
        mark("create_chains")
        a2 = (C.c_void_p * len(cs))(*[c.h for c in cs])
        B.check(lib.vp_run(a2, len(cs), 1))
        mark("batch_build_and_first_sweep")
        B.check(lib.vp_run(a2, len(cs), args.e2e_sweeps - 1))
        mark(f"next_{args.e2e_sweeps - 1}_sweeps")
        lnl = [c.get("LNL")[0] for c in cs]
        mark("read_lnl")
        for c in cs:
            c.close()
        cx.close()
        mark("close")
        phases = ph

    # the c5 serving stream (p50/p99 time-to-result, concurrent vs one at a
    # time) and the single-chain cases in brief
    serving = None
    if not args.no_serving:
        conc, alone, sruns, supd, _ = serve_stream(args, local, rank)
        serving = {"workload": c5_desc(args, len(sruns)), "updates": supd, "concurrent": conc,
                   "one_at_a_time": alone, "form": "plain"}
    extra = None
    if not args.no_extra:
        extra = {name: single_compact(name, local, peaks, cpu_budget_s=0.0 if args.no_cpu_baseline else 5.0)
                 for name in ("c2", "c4")}
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cp = CpuPort(8000, KS)
        cp.sweep()
        dt = cp.sweep()
        cpu = {"value": cp.upd_sweep / dt, "unit": "updates/s", "cores": cp.threads, "kind": "port",
               "sample": f"N={N_IND} x {cp.L} loci sample, 100 chains (K=1..10 x 10), one timed sweep "
                         f"after one warm-up sweep, {dt:.1f} s"}

    line = {"metric": METRIC, "value": value, "unit": "updates/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "likelihood bf16 hi+lo x bf16 counts -> f32; counts e4m3 x e4m3 -> f32 (exact); lnP(D) in f64" if form else "f32",
            "data": "synthetic F-model (8 pops, F=0.03, Beta(0.5,0.5) ancestry, 1% missing), seeded",
            "config": {"workload": f"batched K-sweep: N={N_IND}, L={ds.L} biallelic SNPs, K=1..10 x 10 replicates "
                                   f"= 100 no-admixture chains, one sweep of all chains per step",
                       "form": args.form, "chains": len(KS), "sum_K": sumK, "updates_per_step": upd_step,
                       "l2": "inputs larger than L2 (packed genotypes 0.5 GB; count operands 7.8 GB bf16 + 3.9 GB e4m3)",
                       "parallelism": f"replicas x{world}" if world > 1 else "1 GPU"},
            "roofline": roof, "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "updates/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "step": f"open context from pinned host buffers + create 100 chains + {args.e2e_sweeps} sweeps "
                            f"+ read every chain's lnL + close (launch configuration from the tuner's cache)", "ms_per_step": float(np.median(e2e_ms)) if e2e_ms else None,
                    "phases_ms": phases},
            "gpu_launches": launches, "clocks": clk.summary(), "tc_error_flag": tc_err, "lnp_rel_err": lnp_err,
            "plain_form": plain, "batched_over_plain": value / plain["value"] if plain else None,
            "labels": labels, "serving": serving, "single_chain": extra,
            "tuning": tuning, "updatep": updatep, "pipeline": pipeline,
            "outputs": outputs, "ingest": ingest, "locus_filter": lfilter}
    if rank == 0:
        print(json.dumps(line), flush=True)
    R.finish()


if __name__ == "__main__":
    main()
