"""Seeded synthetic PLINK cohorts for the tests (structured populations,
MCAR missingness, covariates with causal SNP effects)."""
from __future__ import annotations

from dataclasses import dataclass
from pathlib import Path
from typing import Optional

import numpy as np

from oracle import lfmm_oracle as O


@dataclass
class Cohort:
    codes: np.ndarray      # (p, n) uint8 PLINK codes
    packed: np.ndarray     # (p, ceil(n/4)) uint8
    raw: np.ndarray        # (n, p) float with NaN
    x: np.ndarray          # (n, d) covariates
    u_true: np.ndarray     # (n, k_pop) admixture proportions
    causal: np.ndarray
    b_true: np.ndarray     # (p, d)

    @property
    def n(self):
        return self.codes.shape[1]

    @property
    def p(self):
        return self.codes.shape[0]


def simulate(n: int, p: int, *, k_pop: int = 2, fst: float = 0.1, miss: float = 0.01, d: int = 1,
             n_causal: int = 20, effect: float = 0.3, seed: int = 42, f_lo: float = 0.05, f_hi: float = 0.5,
             pop_effect: float = 0.4, monomorphic: int = 0) -> Cohort:
    rng = np.random.default_rng(seed)
    q = rng.dirichlet(np.full(k_pop, 0.5), size=n)
    f_anc = rng.uniform(f_lo, f_hi, size=p)
    a = f_anc * (1 - fst) / fst
    b = (1 - f_anc) * (1 - fst) / fst
    f_pop = rng.beta(a[None, :], b[None, :], size=(k_pop, p))
    f_ind = np.clip(q @ f_pop, 0.0, 1.0)
    g = rng.binomial(2, f_ind).astype(np.int16)              # (n, p)
    if monomorphic:
        g[:, :monomorphic] = rng.integers(0, 3, size=monomorphic)[None, :]
    causal = rng.choice(np.arange(monomorphic, p), size=min(n_causal, p - monomorphic), replace=False)
    b_true = np.zeros((p, d))
    b_true[causal] = effect * rng.choice([-1.0, 1.0], size=(len(causal), d))
    gm = g - g.mean(axis=0)
    sd = g.std(axis=0)
    sd[sd == 0] = 1.0
    gs = gm / sd
    pop = q @ rng.normal(size=(k_pop, d))
    x = pop_effect * pop / (pop.std(axis=0) + 1e-12) + gs[:, causal] @ b_true[causal] + rng.normal(size=(n, d))
    gmiss = g.copy()
    gmiss[rng.random((n, p)) < miss] = 255
    codes = O.genotypes_to_codes(gmiss.T)
    packed = O.pack_codes(codes)
    raw = O.DECODE_TABLE[codes].T.copy()
    return Cohort(codes, packed, raw, x, q, causal, b_true)


def write_plink(cohort: Cohort, prefix: Path, x_names: Optional[list] = None) -> Path:
    prefix = Path(prefix)
    with open(prefix.with_suffix(".bed"), "wb") as f:
        f.write(O.BED_MAGIC)
        f.write(cohort.packed.tobytes())
    with open(prefix.with_suffix(".bim"), "w") as f:
        for j in range(cohort.p):
            f.write(f"{1 + j // 1000}\trs{j}\t0\t{1000 + j * 10}\tA\tG\n")
    with open(prefix.with_suffix(".fam"), "w") as f:
        for i in range(cohort.n):
            f.write(f"FAM{i}\tIND{i}\t0\t0\t0\t-9\n")
    return prefix.with_suffix(".bed")
