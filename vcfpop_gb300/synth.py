"""Seeded synthetic genotype data for the STRUCTURE workloads.

The reference ships no VCF examples for its Bayesian clustering path, so every
workload here is drawn from the F-model it infers (Falush et al. 2003):
ancestral allele frequencies, population frequencies drifted from them by F,
then genotypes sampled from each individual's source population (no-admixture)
or per allele copy from its ancestry vector Q (admixture).

Genotypes are returned as an int8 array ``G[L, N, v]`` of allele indices per
copy (-1 = missing), alleles within an individual sorted ascending, which is
how the reference stores an unphased genotype (``src/function.h:57``).
"""
from __future__ import annotations

import numpy as np


def _drift(rng, anc, F):
    """Population frequencies ~ Dirichlet(anc * (1-F)/F) per locus (Beta for k=2)."""
    f = (1.0 - F) / F
    a = np.maximum(anc * f, 1e-3)
    g = rng.gamma(a)
    s = g.sum(axis=-1, keepdims=True)
    s[s == 0] = 1.0
    return g / s


def fmodel(seed: int, n_ind: int, n_loc: int, n_pop: int, F: float,
           missing: float, admix_alpha: float | None = None,
           ploidy=2, n_alleles=2, anc_alpha: float = 0.5,
           loc_ids=None, loc_alpha: float | None = None, q_scale: float = 2.0,
           per_locus_origin: bool = False):
    """Draw one F-model dataset.

    ploidy: int, or array of per-individual ploidies.
    n_alleles: int, or array of per-locus allele counts.
    admix_alpha: None for discrete populations (equal sizes), else Q_i ~ Dir(alpha).
    loc_ids/loc_alpha: location ancestry Dir(loc_alpha) and Q_i ~ Dir(q_scale * loc ancestry).
    per_locus_origin: draw the source population of every allele copy at every
      locus from Q_i (the admixture model); otherwise one source per copy
      slot of an individual across all loci (the committed golden fixtures
      were drawn that way).
    Returns dict(G=int8[L,N,vmax], pop=int32[N], ploidy=int32[N], k=int32[L], Q=float[N,P]).
    """
    rng = np.random.default_rng(seed)
    ploidy = np.broadcast_to(np.asarray(ploidy, dtype=np.int32), (n_ind,)).copy()
    k = np.broadcast_to(np.asarray(n_alleles, dtype=np.int32), (n_loc,)).copy()
    kmax = int(k.max())
    vmax = int(ploidy.max())
    # ancestral frequencies: Beta(a,a) for k=2, Dirichlet(a) otherwise (padded)
    anc = np.zeros((n_loc, kmax))
    for kk in np.unique(k):
        idx = np.where(k == kk)[0]
        anc[np.ix_(idx, np.arange(kk))] = rng.dirichlet(np.full(kk, anc_alpha), size=len(idx))
    popf = np.stack([_drift(rng, anc, F) for _ in range(n_pop)])  # [P, L, kmax]
    popf[:, anc == 0] = 0.0
    if admix_alpha is None and loc_ids is None:
        pop = (np.arange(n_ind) * n_pop) // n_ind
        Q = np.eye(n_pop)[pop]
    elif loc_ids is not None:
        nloc_s = int(loc_ids.max()) + 1
        la = rng.dirichlet(np.full(n_pop, loc_alpha), size=nloc_s)
        Q = np.stack([rng.dirichlet(np.maximum(q_scale * la[s], 1e-3)) for s in loc_ids])
        pop = np.asarray(loc_ids, dtype=np.int32)
    else:
        Q = rng.dirichlet(np.full(n_pop, admix_alpha), size=n_ind)
        pop = np.zeros(n_ind, dtype=np.int32)
    G = np.full((n_loc, n_ind, vmax), -1, dtype=np.int8)
    cumQ = np.cumsum(Q, axis=1)
    cumf = np.cumsum(popf, axis=2)  # [P, L, kmax]
    # inverse-CDF draws, one threshold at a time: the origin is the number of
    # cumulative ancestry proportions below u, the allele the number of
    # cumulative frequencies of the origin below ua (capped at k - 1)
    for c in range(vmax):
        has = ploidy > c
        if per_locus_origin:
            chunk = max(1, (1 << 22) // max(1, n_ind * kmax))        # loci per pair of uniform draws
            sub = max(1, (1 << 18) // max(1, n_ind))                  # loci per cache-sized pass
            for l0 in range(0, n_loc, chunk):
                l1 = min(n_loc, l0 + chunk)
                u = rng.random((l1 - l0, n_ind))
                ua = rng.random((l1 - l0, n_ind))
                for r0 in range(0, l1 - l0, sub):
                    r1 = min(l1 - l0, r0 + sub)
                    src = np.zeros((r1 - r0, n_ind), np.int32)                                 # [rows, N]
                    for p in range(n_pop - 1):
                        src += u[r0:r1] > cumQ[:, p][None, :]
                    idx = src + (np.arange(r1 - r0, dtype=np.int32) * n_pop)[:, None]          # (locus, origin)
                    al = np.zeros((r1 - r0, n_ind), np.int8)
                    for a in range(kmax - 1):
                        thr = np.ascontiguousarray(cumf[:, l0 + r0:l0 + r1, a].T).reshape(-1)  # [rows * P]
                        al += ua[r0:r1] > np.take(thr, idx)
                    al = np.minimum(al, (k[l0 + r0:l0 + r1] - 1)[:, None])
                    G[l0 + r0:l0 + r1, has, c] = al[:, has]
            continue
        u = rng.random(n_ind)
        src = np.zeros(n_ind, np.int64)                                           # origin of this copy
        for p in range(n_pop - 1):
            src += u > cumQ[:, p]
        ua = rng.random((n_loc, n_ind))
        al = np.zeros((n_loc, n_ind), np.int64)
        for a in range(kmax - 1):
            al += ua > cumf[src, :, a].T                                            # [L, N]
        al = np.minimum(al, (k - 1)[:, None])
        G[:, has, c] = al[:, has]
    miss = rng.random((n_loc, n_ind)) < missing
    G[miss] = -1
    # unphased: sort the copies of each call ascending, missing stays missing
    Gs = np.where(G < 0, 127, G)
    Gs.sort(axis=2)
    G = np.where(Gs == 127, -1, Gs).astype(np.int8)
    return dict(G=G, pop=np.asarray(pop, dtype=np.int32), ploidy=ploidy, k=k, Q=Q)


def write_vcf(path: str, data: dict, pop_names=None):
    """Write a dataset as an uncompressed VCF (GT only)."""
    G, ploidy, k = data["G"], data["ploidy"], data["k"]
    L, N, _ = G.shape
    bases = ["A", "C", "G", "T"]
    with open(path, "w") as f:
        f.write("##fileformat=VCFv4.2\n")
        f.write('##FORMAT=<ID=GT,Number=1,Type=String,Description="Genotype">\n')
        f.write("#CHROM\tPOS\tID\tREF\tALT\tQUAL\tFILTER\tINFO\tFORMAT\t")
        f.write("\t".join(f"Ind{i + 1}" for i in range(N)) + "\n")
        for l in range(L):
            kk = int(k[l])
            alt = ",".join(bases[(a) % 4] + ("A" * (a // 4)) if a else "" for a in range(1, kk))
            ref = "T" if kk == 2 else "TT"
            alt = "A" if kk == 2 else ",".join("T" + "ACG"[(a - 1) % 3] * ((a + 2) // 3) for a in range(1, kk))
            cells = []
            for i in range(N):
                v = int(ploidy[i])
                g = G[l, i, :v]
                if g[0] < 0:
                    cells.append("/".join(["."] * v))
                else:
                    cells.append("/".join(str(int(x)) for x in g))
            f.write(f"1\t{l + 1}\tsnp{l + 1}\t{ref}\t{alt}\t.\tPASS\t.\tGT\t" + "\t".join(cells) + "\n")


def indtext(pop: np.ndarray, names=None) -> str:
    """vcfpop -g_indtext string assigning consecutive individual ranges to populations."""
    pop = np.asarray(pop)
    parts = []
    n = len(pop)
    i = 0
    while i < n:
        j = i
        while j + 1 < n and pop[j + 1] == pop[i]:
            j += 1
        nm = names[pop[i]] if names else f"pop{pop[i] + 1}"
        parts.append((nm, i + 1, j + 1))
        i = j + 1
    byname = {}
    for nm, a, b in parts:
        byname.setdefault(nm, []).append(f"#{a}-#{b}")
    return " ".join(f"{nm}:{','.join(r)}" for nm, r in byname.items())
