"""The STRUCTURE workloads the throughput and latency figures are quoted on,
as seeded synthetic data with the shapes and distributions of each case.

  c1  N=200 diploids, 3 source populations, L=2,000 biallelic SNPs, F=0.1,
      5% missing; K=3 without admixture, 1,000 burn-in + 2,000 sweeps
  c2  N=2,000 x L=50,000, Q ~ Dir(0.5), F=0.05, 2% missing; K=5 with
      admixture and alpha inferred, 5,000 burn-in + 10,000 sweeps
  c3  N=10,000 x L=200,000, 8 populations, F=0.03, 1% missing; K=1..10 x 10
      replicates without admixture (bench.py draws it on the GPU)
  c4  N=5,000 autopolyploids (ploidy 2/4/6 in ratio 2:1:1) at 20 locations,
      L=20,000 loci with 2-8 alleles, Dirichlet F-model F=0.08 over Dir(1),
      location ancestry Dir(1), Q_i ~ Dir(2 x location ancestry), 3% missing;
      K=8 with admixture and the location prior, 10,000 + 10,000 sweeps
  c5  a stream of independent runs (Poisson arrivals; N, L log-uniform; K
      uniform; admixture with probability 1/2; run length uniform)

Each function returns the data (a synth dict) and the run parameters as
-structure_* flag names.
"""
from __future__ import annotations

import numpy as np

from . import synth


def c1(seed: int = 1):
    d = synth.fmodel(seed, 200, 2000, 3, 0.1, 0.05)
    run = dict(K=3, admix=0, locpriori=0, f=0, nburnin=1000, nreps=2000, nadmburnin=0)
    return d, run


def c2(seed: int = 2):
    d = synth.fmodel(seed, 2000, 50_000, 5, 0.05, 0.02, admix_alpha=0.5, per_locus_origin=True)
    run = dict(K=5, admix=1, locpriori=0, f=0, inferalpha=1, nburnin=5000, nreps=10_000)
    return d, run


def c4(seed: int = 4):
    rng = np.random.default_rng(seed)
    N, L, S = 5000, 20_000, 20
    ploidy = np.array([2, 2, 4, 6] * (N // 4), np.int32)
    loc = np.repeat(np.arange(S), N // S).astype(np.int32)
    d = synth.fmodel(seed, N, L, 8, 0.08, 0.03, ploidy=ploidy, n_alleles=rng.integers(2, 9, L), anc_alpha=1.0,
                     loc_ids=loc, loc_alpha=1.0, q_scale=2.0, per_locus_origin=True)
    run = dict(K=8, admix=1, locpriori=1, f=0, nburnin=10_000, nreps=10_000)
    return d, run


def c5_requests(n: int, seed: int = 5, rate: float = 50.0, scale: float = 0.1):
    """n runs of the serving stream: arrival times (s, Poisson at `rate`) and
    shapes. `scale` shrinks N, L and the run length ranges together (1.0 is
    N in [100, 20,000], L in [1,000, 200,000], 2,000-20,000 sweeps)."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n))
    t -= t[0]

    def logu(lo, hi):
        return int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))

    out = []
    for j in range(n):
        N = max(16, logu(100 * scale, 20_000 * scale)) if scale < 1 else logu(100, 20_000)
        L = max(100, logu(1000 * scale, 200_000 * scale)) if scale < 1 else logu(1000, 200_000)
        K = int(rng.integers(2, 13))
        admix = int(rng.random() < 0.5)
        sweeps = int(rng.integers(int(2000 * scale), int(20_000 * scale) + 1))
        nburnin = sweeps // 2
        out.append(dict(t=float(t[j]), N=N, L=L, K=K, admix=admix, nburnin=nburnin, nreps=sweeps - nburnin,
                        seed=int(rng.integers(1, 2 ** 31)), pops=int(rng.integers(2, 9))))
    return out
