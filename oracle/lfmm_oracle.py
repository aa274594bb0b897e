"""CPU oracle for the streaming LFMM2 hot path -- TEST INFRASTRUCTURE ONLY.

This module is the oracle, never the product.  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py`` (its ``cpu_baseline`` leg and
its ``--impl reference`` arm) may import it.  The product path lives in
``schnellfmm_gb300`` and runs on the GPU only.

It restates, in FP64 NumPy, the algorithm of schnelLFMM v0.3.2 (a Rust crate
that cannot be built here: no cargo/rustc).  Every function cites the
reference file:line it follows.  Two forms are provided:

* ``ref_*`` -- a faithful restatement of the reference CPU path, including
  its n x n matrices (``M = D_lambda Q^T``, ``P_U``, ``I - P_U``, ``H_X``) and
  its per-chunk BLAS calls.  Used as the timed CPU baseline ("port") and to
  cross-check the thin form at small sizes.
* ``thin_*`` / ``oracle64_*`` -- the same mathematics without any n x n
  object (``P = Q D_lambda Q^T = I - Q_d (I - D_d) Q_d^T``), fed with the same
  random sketch as the GPU path.  This is the FP64 precision oracle.

Parity status: the decode, counting, mean/scale, subset, histogram/median,
GIF and covariate-centring rules are pinned by the reference's own unit-test
known answers (``tests/golden/reference_kats.json`` and the CPU tests).  The
engine's default random streams are a counter-based SplitMix64 generator
shared by this oracle and the GPU.  The reference's streams
(ChaCha8Rng::seed_from_u64 sampled by Normal(0, 1) for the sketches and by
Uniform(0, 1) for the CV masks) are restated in ``chacha8_normal_matrix`` and
``mask_uniform`` from the published algorithms; the ChaCha block function is
pinned by the RFC 8439 test vector, the rest is "parity unpinned" (no test of
the reference checks Omega or mask values).  RNG-dependent quantities are
compared at the subspace / statistical level.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field
from pathlib import Path
from typing import List, Optional, Sequence, Tuple

import numpy as np

# ---------------------------------------------------------------------------
# PLINK codec  (src/bed.rs)
# ---------------------------------------------------------------------------

BED_MAGIC = bytes([0x6C, 0x1B, 0x01])  # src/bed.rs:9

NORM_CENTER_ONLY = 0  # src/bed.rs:19-26 (SnpNorm::CenterOnly, library default)
NORM_EIGENSTRAT = 1   # src/bed.rs:19-26 (SnpNorm::Eigenstrat, CLI default)


def bytes_per_snp(n_physical: int) -> int:
    """ceil(n/4) bytes per SNP row (src/bed.rs:143-145)."""
    return (n_physical + 3) // 4


def unpack_codes(packed: np.ndarray, n_physical: int) -> np.ndarray:
    """2-bit codes, SNP-major: returns uint8 array (p, n_physical).

    Sample s of a SNP row sits in byte s//4 at bit offset 2*(s%4)
    (src/bed.rs:262-281)."""
    packed = np.asarray(packed, dtype=np.uint8)
    p, bps = packed.shape
    codes = np.empty((p, bps, 4), dtype=np.uint8)
    for k in range(4):
        codes[:, :, k] = (packed >> (2 * k)) & 0x03
    return codes.reshape(p, bps * 4)[:, :n_physical]


def pack_codes(codes: np.ndarray) -> np.ndarray:
    """Inverse of unpack_codes; padding codes are 0b00 (src/bed.rs:398-434)."""
    codes = np.asarray(codes, dtype=np.uint8)
    p, n = codes.shape
    bps = bytes_per_snp(n)
    padded = np.zeros((p, bps * 4), dtype=np.uint8)
    padded[:, :n] = codes
    padded = padded.reshape(p, bps, 4)
    out = np.zeros((p, bps), dtype=np.uint8)
    for k in range(4):
        out |= (padded[:, :, k] & 3) << (2 * k)
    return out


def genotypes_to_codes(g: np.ndarray) -> np.ndarray:
    """Encode table 0->00, 1->10, 2->11, missing(anything else)->01 (src/bed.rs:405-414).

    ``g`` is (p, n) with values in {0,1,2} or 255/-1 for missing."""
    g = np.asarray(g)
    codes = np.full(g.shape, 1, dtype=np.uint8)
    codes[g == 0] = 0
    codes[g == 1] = 2
    codes[g == 2] = 3
    return codes


DECODE_TABLE = np.array([0.0, np.nan, 1.0, 2.0])  # src/bed.rs:16


def decode_raw(packed: np.ndarray, n_physical: int,
               sample_keep: Optional[Sequence[int]] = None) -> np.ndarray:
    """Raw decode to {0,1,2,NaN}, returned sample-major (n_out, p)
    (src/bed.rs:262-281, decode_raw_single_snp)."""
    codes = unpack_codes(packed, n_physical)
    if sample_keep is not None:
        codes = codes[:, np.asarray(sample_keep, dtype=np.int64)]
    return DECODE_TABLE[codes].T.copy()


def compute_scale(mean: np.ndarray, norm: int) -> np.ndarray:
    """Per-SNP scale from the mean, same operation order as
    src/bed.rs:382-395: p = mean/2; twopq = 2*p*(1-p)."""
    mean = np.asarray(mean, dtype=np.float64)
    p = mean / 2.0
    twopq = (2.0 * p) * (1.0 - p)
    if norm == NORM_CENTER_ONLY:
        return np.where(twopq < 1e-20, 0.0, 1.0)
    denom = np.sqrt(twopq)
    with np.errstate(divide="ignore"):
        return np.where(denom > 1e-10, 1.0 / np.where(denom > 0, denom, 1.0), 0.0)


@dataclass
class SnpStats:
    counts: np.ndarray   # (p, 4) int32: c0, c1 (het), c2 (hom alt), cmiss
    mean: np.ndarray     # (p,) f64, bit-exact with src/bed.rs:349-361
    scale: np.ndarray    # (p,) f64, bit-exact with src/bed.rs:382-395
    tss: np.ndarray      # (p,) f64, sum of squared standardised values


def snp_stats(raw: np.ndarray, norm: int) -> SnpStats:
    """Allele counts, mean over observed calls, scale and TSS per SNP.

    The mean is sum/n_valid in FP64 (src/bed.rs:349-361); the sum of
    0/1/2 values is exact, so ``S1 / n_obs`` is bit-identical.  TSS is
    s^2 * (S2 - S1^2/n_obs), i.e. ||y_hat||^2 of the standardised column."""
    obs = ~np.isnan(raw)
    c0 = np.sum(raw == 0.0, axis=0)
    c1 = np.sum(raw == 1.0, axis=0)
    c2 = np.sum(raw == 2.0, axis=0)
    cm = np.sum(~obs, axis=0)
    counts = np.stack([c0, c1, c2, cm], axis=1).astype(np.int32)
    s1 = (c1 + 2 * c2).astype(np.int64)
    s2 = (c1 + 4 * c2).astype(np.int64)
    nobs = (c0 + c1 + c2).astype(np.int64)
    with np.errstate(invalid="ignore", divide="ignore"):
        mean = np.where(nobs > 0, s1.astype(np.float64) / np.maximum(nobs, 1).astype(np.float64), 0.0)
    scale = compute_scale(mean, norm)
    num = nobs * s2 - s1 * s1            # exact integer
    with np.errstate(invalid="ignore", divide="ignore"):
        css = np.where(nobs > 0, num.astype(np.float64) / np.maximum(nobs, 1), 0.0)
    tss = scale * scale * css
    return SnpStats(counts, mean, scale, tss)


def decode_standardized(raw: np.ndarray, norm: int,
                        fill: Optional[np.ndarray] = None) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """decode_single_snp (src/bed.rs:300-379) on an already raw-decoded
    (n, p) block: optional per-entry fill of NaNs, mean over non-NaN,
    scale, centre, NaN -> 0.  Returns (y_hat, mean, scale)."""
    y = raw.copy()
    if fill is not None:
        nan = np.isnan(y)
        y[nan] = fill[nan]
    obs = ~np.isnan(y)
    n_valid = obs.sum(axis=0)
    s = np.where(obs, y, 0.0).sum(axis=0)
    mean = np.where(n_valid > 0, s / np.maximum(n_valid, 1), 0.0)
    scale = compute_scale(mean, norm)
    out = np.where(obs, (y - mean) * scale, 0.0)
    return out, mean, scale


def fill_missing_with_column_means(raw: np.ndarray) -> np.ndarray:
    """src/parallel.rs:53-71 (MeanRaw fill, raw dosage scale)."""
    y = raw.copy()
    obs = ~np.isnan(y)
    n_obs = obs.sum(axis=0)
    s = np.where(obs, y, 0.0).sum(axis=0)
    mean = np.where(n_obs > 0, s / np.maximum(n_obs, 1), 0.0)
    y[~obs] = np.broadcast_to(mean, y.shape)[~obs]
    return y


# ---------------------------------------------------------------------------
# Subsets  (src/bed.rs:50-57, 162-171; src/parallel.rs:113-122)
# ---------------------------------------------------------------------------

def subset_indices(n_snps: int, rate: Optional[float] = None,
                   indices: Optional[Sequence[int]] = None) -> np.ndarray:
    """All / Rate(r): step = ceil(1/r), indices 0, step, 2*step... / Indices."""
    if indices is not None:
        return np.asarray(indices, dtype=np.int64)
    if rate is None:
        return np.arange(n_snps, dtype=np.int64)
    step = int(math.ceil(1.0 / rate))
    return np.arange(0, n_snps, step, dtype=np.int64)


def subset_snp_count(n_snps: int, rate: Optional[float] = None,
                     indices: Optional[Sequence[int]] = None) -> int:
    if indices is not None:
        return len(indices)
    if rate is None:
        return n_snps
    step = int(math.ceil(1.0 / rate))
    return (n_snps + step - 1) // step


# ---------------------------------------------------------------------------
# Random streams: counter-based SplitMix64 (shared with the GPU path)
# ---------------------------------------------------------------------------

_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def _mix64(z: np.ndarray) -> np.ndarray:
    z = np.asarray(z, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def rng_key(seed: int) -> np.uint64:
    with np.errstate(over="ignore"):
        return _mix64(np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + _GAMMA)


def rng_u64(seed: int, counter: np.ndarray) -> np.ndarray:
    """u64 = mix64(key(seed) + (counter+1)*GAMMA): the SplitMix64 sequence
    started at state key(seed), addressable by counter."""
    key = rng_key(seed)
    c = np.asarray(counter, dtype=np.uint64)
    with np.errstate(over="ignore"):
        return _mix64(key + (c + np.uint64(1)) * _GAMMA)


def rng_uniform(seed: int, counter: np.ndarray) -> np.ndarray:
    """U[0,1) with 53 random bits: (u64 >> 11) * 2^-53."""
    return (rng_u64(seed, counter) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


def rng_normal_matrix(seed: int, rows: int, cols: int) -> np.ndarray:
    """Standard normal (rows x cols), element (i, c) is draw i*cols+c in
    row-major order like ``Array2::from_shape_fn`` (src/rsvd.rs:44-46).
    Box-Muller on draws 2k (radius) and 2k+1 (angle)."""
    idx = np.arange(rows * cols, dtype=np.uint64)
    u1 = ((rng_u64(seed, 2 * idx) >> np.uint64(11)).astype(np.float64) + 1.0) * (2.0 ** -53)
    u2 = (rng_u64(seed, 2 * idx + np.uint64(1)) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)
    z = np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)
    return z.reshape(rows, cols)


# ---------------------------------------------------------------------------
# The reference's sketch stream (src/rsvd.rs:44-46, src/nmf.rs:291-293):
# ChaCha8Rng::seed_from_u64(seed) sampled by rand_distr's Normal(0, 1) into an
# Array2 in row-major order.  Restated from the published algorithms (the
# crates, rand_core 0.6.4 / rand_chacha 0.3.1 / rand_distr 0.4.3 per
# Cargo.lock, are not in the reference tree):
#   ChaCha block function -- Bernstein 2008 / RFC 8439 s2.3, 64-bit block
#     counter in words 12-13, 64-bit stream id in words 14-15;
#   seed_from_u64 -- 8 PCG32 XSH-RR outputs (O'Neill 2014) as the key words;
#   Normal -- ZIGNOR ziggurat, 256 strips (Doornik 2005).
# ---------------------------------------------------------------------------

_CHACHA_CONST = (0x61707865, 0x3320646E, 0x79622D32, 0x6B206574)   # "expand 32-byte k"
_MASK32 = 0xFFFFFFFF


def chacha_blocks(state: np.ndarray, rounds: int) -> np.ndarray:
    """ChaCha block function over B input states at once: ``state`` is
    (B, 16) uint32, the result (B, 16) uint32 is rounds/2 double rounds
    (columns, then diagonals) plus the input state (RFC 8439 s2.3)."""
    x = [state[:, i].astype(np.uint32) for i in range(16)]

    def rotl(v, r):
        return (v << np.uint32(r)) | (v >> np.uint32(32 - r))

    def qr(a, b, c, d):
        x[a] = x[a] + x[b]; x[d] = rotl(x[d] ^ x[a], 16)
        x[c] = x[c] + x[d]; x[b] = rotl(x[b] ^ x[c], 12)
        x[a] = x[a] + x[b]; x[d] = rotl(x[d] ^ x[a], 8)
        x[c] = x[c] + x[d]; x[b] = rotl(x[b] ^ x[c], 7)

    with np.errstate(over="ignore"):
        for _ in range(rounds // 2):
            qr(0, 4, 8, 12); qr(1, 5, 9, 13); qr(2, 6, 10, 14); qr(3, 7, 11, 15)
            qr(0, 5, 10, 15); qr(1, 6, 11, 12); qr(2, 7, 8, 13); qr(3, 4, 9, 14)
        return np.stack(x, axis=1) + state.astype(np.uint32)


def pcg32_seed_words(seed: int) -> List[int]:
    """seed_from_u64: the LCG state is stepped (multiplier
    6364136223846793005, increment 11634580027462260723) before each of 8
    XSH-RR outputs, which become the 8 little-endian key words."""
    s = seed & 0xFFFFFFFFFFFFFFFF
    words = []
    for _ in range(8):
        s = (s * 6364136223846793005 + 11634580027462260723) & 0xFFFFFFFFFFFFFFFF
        xorshifted = (((s >> 18) ^ s) >> 27) & _MASK32
        rot = s >> 59
        words.append(((xorshifted >> rot) | (xorshifted << ((32 - rot) & 31))) & _MASK32)
    return words


def chacha8_u64(seed: int, count: int, start_block: int = 0) -> np.ndarray:
    """``count`` consecutive 64-bit outputs of ChaCha8Rng::seed_from_u64(seed)
    from block ``start_block`` on: the keystream's 32-bit words in order, two
    per output, low word first."""
    blocks = (2 * count + 15) // 16
    st = np.zeros((blocks, 16), dtype=np.uint32)
    st[:, 0:4] = _CHACHA_CONST
    st[:, 4:12] = pcg32_seed_words(seed)
    ctr = np.arange(start_block, start_block + blocks, dtype=np.uint64)
    st[:, 12] = (ctr & np.uint64(_MASK32)).astype(np.uint32)
    st[:, 13] = (ctr >> np.uint64(32)).astype(np.uint32)
    words = chacha_blocks(st, 8).reshape(-1).astype(np.uint64)
    return (words[0::2] | (words[1::2] << np.uint64(32)))[:count]


ZIG_R = 3.6541528853610088
ZIG_V = 0.00492867323399


def _gauss_pdf(x: float) -> float:
    return math.exp(-x * x / 2.0)


def ziggurat_tables() -> Tuple[List[float], List[float]]:
    """Strip edges x_0..x_256 and f(x_i) of the 256-strip ziggurat:
    x_0 = V / f(R) (the base strip's equivalent width), x_1 = R,
    x_{i+1} = f^-1(V / x_i + f(x_i)), x_256 = 0 (Doornik 2005)."""
    x = [0.0] * 257
    x[0] = ZIG_V / _gauss_pdf(ZIG_R)
    x[1] = ZIG_R
    for i in range(2, 256):
        x[i] = math.sqrt(-2.0 * math.log(ZIG_V / x[i - 1] + _gauss_pdf(x[i - 1])))
    x[256] = 0.0
    return x, [_gauss_pdf(v) for v in x]


class _U64Stream:
    def __init__(self, seed: int, hint: int):
        self.seed, self.pos, self.block = seed, 0, 0
        self.buf = np.zeros(0, dtype=np.uint64)
        self._more(max(hint, 8))

    def _more(self, count: int):
        count = (count + 7) // 8 * 8                     # whole blocks
        nxt = chacha8_u64(self.seed, count, self.block)
        self.block += count // 8
        self.buf = np.concatenate([self.buf[self.pos:], nxt])
        self.pos = 0

    def next(self) -> int:
        if self.pos == self.buf.size:
            self._more(max(1024, self.buf.size // 4))
        v = int(self.buf[self.pos])
        self.pos += 1
        return v


def _bits_to_f64(b: int) -> float:
    return float(np.array([b], dtype=np.uint64).view(np.float64)[0])


def chacha8_normal_matrix(seed: int, rows: int, cols: int, stats: Optional[dict] = None) -> np.ndarray:
    """Array2::from_shape_fn((rows, cols), |_| Normal::new(0, 1).sample(&mut
    ChaCha8Rng::seed_from_u64(seed))) (src/rsvd.rs:44-46).  Per draw: a u64
    gives strip i (low 8 bits) and u in [-1, 1) (top 52 bits as the mantissa
    of [2, 4), minus 3); x = u x_i is accepted if |x| < x_{i+1}; strip 0 falls
    back to the tail beyond R (two open (0, 1) uniforms per try, top 52 bits
    in [1, 2) minus 1 - 2^-53, until -2 ln b >= (ln a / R)^2); other strips
    accept if f_{i+1} + (f_i - f_{i+1}) U < f(x), U = (u64 >> 11) 2^-53.
    ``stats`` (optional) counts the tail and wedge branches taken."""
    xt, ft = ziggurat_tables()
    rng = _U64Stream(seed, rows * cols + rows * cols // 64 + 16)
    out = np.empty(rows * cols)
    tails = wedges = 0
    for e in range(rows * cols):
        while True:
            bits = rng.next()
            i = bits & 0xFF
            u = _bits_to_f64((1024 << 52) | (bits >> 12)) - 3.0
            x = u * xt[i]
            if abs(x) < xt[i + 1]:
                break
            if i == 0:
                tails += 1
                tx, ty = 1.0, 0.0
                while -2.0 * ty < tx * tx:
                    a = _bits_to_f64((1023 << 52) | (rng.next() >> 12)) - (1.0 - 2.0 ** -53)
                    b = _bits_to_f64((1023 << 52) | (rng.next() >> 12)) - (1.0 - 2.0 ** -53)
                    tx = math.log(a) / ZIG_R
                    ty = math.log(b)
                x = tx - ZIG_R if u < 0.0 else ZIG_R - tx
                break
            wedges += 1
            if ft[i + 1] + (ft[i] - ft[i + 1]) * ((rng.next() >> 11) * 2.0 ** -53) < _gauss_pdf(x):
                break
        out[e] = 0.0 + 1.0 * x
    if stats is not None:
        stats.update(tails=tails, wedges=wedges)
    return out.reshape(rows, cols)


def sketch_normal(rng: str, seed: int, rows: int, cols: int) -> np.ndarray:
    """Gaussian sketch from the named stream: "counter" (the engine's
    default) or "chacha8" (the reference's)."""
    if rng == "counter":
        return rng_normal_matrix(seed, rows, cols)
    if rng == "chacha8":
        return chacha8_normal_matrix(seed, rows, cols)
    raise ValueError(f"unknown stream {rng!r}")


# ---------------------------------------------------------------------------
# Covariates and Step 0  (src/lib.rs:102-117, src/precompute.rs:30-88)
# ---------------------------------------------------------------------------

def center_covariates(x: np.ndarray, scale: bool) -> np.ndarray:
    """Column-centre; optionally divide by sd with (n-1) denominator,
    skipped when sd <= 1e-14 (src/lib.rs:102-117)."""
    x = np.asarray(x, dtype=np.float64)
    n = x.shape[0]
    xs = x - x.mean(axis=0, keepdims=True)
    if scale:
        for j in range(xs.shape[1]):
            col = xs[:, j]
            sd = math.sqrt(float(col @ col) / (n - 1.0))
            if sd > 1e-14:
                xs[:, j] = col / sd
    return xs


class SingularMatrixError(RuntimeError):
    pass


def _is_exactly_singular(a: np.ndarray) -> bool:
    """LAPACK getrf reports singularity only on an exactly zero pivot."""
    try:
        import scipy.linalg as sla
        lu, piv = sla.lu_factor(a, check_finite=False)
        return bool(np.any(np.diag(lu) == 0.0))
    except Exception:
        return True


def safe_inv(a: np.ndarray, name: str = "matrix") -> Tuple[np.ndarray, bool]:
    """Inverse with Tikhonov fallback eps = 1e-8 * max|diag| (>= 1e-300)
    when the LU factorisation hits an exactly zero pivot
    (src/testing.rs:996-1024).  Returns (inverse, regularised?)."""
    a = np.asarray(a, dtype=np.float64)
    if not _is_exactly_singular(a):
        return np.linalg.inv(a), False
    diag_max = max(float(np.max(np.abs(np.diag(a)))) if a.size else 0.0, 1e-300)
    eps = 1e-8 * diag_max
    a_reg = a + eps * np.eye(a.shape[0])
    if _is_exactly_singular(a_reg):
        raise SingularMatrixError(f"{name} inversion failed even with epsilon={eps:.2e} regularization")
    return np.linalg.inv(a_reg), True


@dataclass
class PrecomputedFull:
    """src/precompute.rs:10-21 (the n x n form)."""
    q_full: np.ndarray
    d_lambda: np.ndarray
    d_lambda_inv: np.ndarray
    m: np.ndarray
    ridge_inv: np.ndarray


def precompute_full(xs: np.ndarray, lam: float) -> PrecomputedFull:
    """src/precompute.rs:30-88: full SVD of X, d_lambda = sqrt(lam/(lam+s^2))
    for j < d (1 beyond), M = D_lambda Q^T, ridge_inv = (X^T X + lam I)^-1."""
    if lam <= 0.0:
        raise ValueError(f"Ridge penalty lambda must be positive, got {lam}")
    n, d = xs.shape
    q_full, sigma, _ = np.linalg.svd(xs, full_matrices=True)
    d_lambda = np.ones(n)
    for j in range(min(len(sigma), d)):
        d_lambda[j] = math.sqrt(lam / (lam + sigma[j] * sigma[j]))
    d_lambda_inv = 1.0 / d_lambda
    m = d_lambda[:, None] * q_full.T
    xtx = xs.T @ xs + lam * np.eye(d)
    ridge_inv, _ = safe_inv(xtx, "X^T X + lambda I (ridge)")
    return PrecomputedFull(q_full, d_lambda, d_lambda_inv, m, ridge_inv)


@dataclass
class PrecomputedThin:
    """Thin Step 0: Q_d (n x r) and d_d (r) with P = I - Q_d (1-d_d) Q_d^T."""
    q_d: np.ndarray
    d_d: np.ndarray
    ridge_inv: np.ndarray

    def apply_p(self, a: np.ndarray) -> np.ndarray:
        return a - self.q_d @ ((1.0 - self.d_d)[:, None] * (self.q_d.T @ a))

    def apply_pinv(self, a: np.ndarray) -> np.ndarray:
        return a - self.q_d @ ((1.0 - 1.0 / self.d_d)[:, None] * (self.q_d.T @ a))


def precompute_thin(xs: np.ndarray, lam: float) -> PrecomputedThin:
    if lam <= 0.0:
        raise ValueError(f"Ridge penalty lambda must be positive, got {lam}")
    n, d = xs.shape
    q, sigma, _ = np.linalg.svd(xs, full_matrices=False)
    keep = sigma > (sigma.max() if sigma.size else 0.0) * 1e-12
    q_d = q[:, keep]
    s = sigma[keep]
    d_d = np.sqrt(lam / (lam + s * s))
    ridge_inv, _ = safe_inv(xs.T @ xs + lam * np.eye(d), "X^T X + lambda I (ridge)")
    return PrecomputedThin(q_d, d_d, ridge_inv)


# ---------------------------------------------------------------------------
# Randomized SVD  (src/rsvd.rs:26-177)
# ---------------------------------------------------------------------------

def _qr_q(a: np.ndarray) -> np.ndarray:
    q, _ = np.linalg.qr(a)
    return q


def rsvd_ref(y_est: np.ndarray, pre: PrecomputedFull, k: int, l: int, q_iter: int,
             omega: np.ndarray, chunk: int) -> np.ndarray:
    """Faithful restatement of estimate_factors_streaming (src/rsvd.rs:26-177)
    over a standardised (n, p_est) matrix, chunked like the reference."""
    n, p = y_est.shape
    mt_omega = pre.m.T @ omega                                     # :51
    chunks = [(s, min(s + chunk, p)) for s in range(0, p, chunk)]
    z = np.zeros((p, l))
    for s, e in chunks:                                            # :61-69
        z[s:e] = y_est[:, s:e].T @ mt_omega
    q_z = _qr_q(z)                                                 # :75
    for _ in range(q_iter):                                        # :79-134
        a_qz = np.zeros((n, l))
        for s, e in chunks:                                        # :88-97
            a_qz += pre.m @ (y_est[:, s:e] @ q_z[s:e])
        mt_q = pre.m.T @ _qr_q(a_qz)                               # :104-107
        z = np.zeros((p, l))
        for s, e in chunks:                                        # :117-125
            z[s:e] = y_est[:, s:e].T @ mt_q
        q_z = _qr_q(z)                                             # :131
    b = np.zeros((n, l))
    for s, e in chunks:                                            # :144-153
        b += pre.m @ (y_est[:, s:e] @ q_z[s:e])
    u_small, _, _ = np.linalg.svd(b, full_matrices=False)          # :162
    return pre.q_full @ (pre.d_lambda_inv[:, None] * u_small[:, :k])  # :168-172


def rsvd_thin(y_est: np.ndarray, pre: PrecomputedThin, k: int, l: int, q_iter: int,
              omega: np.ndarray) -> np.ndarray:
    """Same algorithm in the thin formulation: the reference's sketch
    M^T Omega = Q D Omega is replaced by P Omega (P = Q D Q^T), forward
    passes accumulate P (Y Q_z) (= Q A Q_z), and U_hat = P^-1 U(P Y Q_z).
    Identical latent subspace in exact arithmetic for the same sketch."""
    z = y_est.T @ pre.apply_p(omega)
    q_z = _qr_q(z)
    for _ in range(q_iter):
        s = pre.apply_p(y_est @ q_z)
        q_s = _qr_q(s)
        z = y_est.T @ pre.apply_p(q_s)
        q_z = _qr_q(z)
    b = pre.apply_p(y_est @ q_z)
    u_b, _, _ = np.linalg.svd(b, full_matrices=False)
    return pre.apply_pinv(u_b[:, :k])


# ---------------------------------------------------------------------------
# Association testing  (src/testing.rs)
# ---------------------------------------------------------------------------

HIST_BINS = 100_000      # src/testing.rs:124
HIST_WIDTH = 0.001       # src/testing.rs:125
GIF_DIVISOR = 0.4549     # src/testing.rs:169


class TsqHistogram:
    """Streaming t^2 histogram, bins of width 0.001, last bin clamps
    (src/testing.rs:114-225)."""

    def __init__(self, d: int):
        self.counts = np.zeros((d, HIST_BINS), dtype=np.uint64)
        self.total = np.zeros(d, dtype=np.uint64)

    def add_chunk(self, tstats: np.ndarray) -> None:
        """tstats (chunk, d); skip non-finite t^2 (src/testing.rs:135-149)."""
        t_sq = np.asarray(tstats, dtype=np.float64) ** 2
        for j in range(t_sq.shape[1]):
            v = t_sq[:, j]
            v = v[np.isfinite(v)]
            b = np.minimum(np.floor(v / HIST_WIDTH), HIST_BINS - 1).astype(np.int64)
            self.counts[j] += np.bincount(b, minlength=HIST_BINS).astype(np.uint64)
            self.total[j] += np.uint64(v.size)

    def median_for_trait(self, j: int) -> float:
        """Cumulative walk (src/testing.rs:179-224): odd count -> centre of
        the bin holding element n//2; even -> mean of the centres of the
        bins holding elements n/2-1 and n/2."""
        n = int(self.total[j])
        if n == 0:
            return 0.0
        even = n % 2 == 0
        target = n // 2 - 1 if even else n // 2
        cum = np.cumsum(self.counts[j].astype(np.int64))
        b1 = int(np.searchsorted(cum, target, side="right"))
        if not even:
            return (b1 + 0.5) * HIST_WIDTH
        b2 = int(np.searchsorted(cum, target + 1, side="right"))
        return ((b1 + 0.5) * HIST_WIDTH + (b2 + 0.5) * HIST_WIDTH) / 2.0

    def compute_gif(self) -> Tuple[np.ndarray, float]:
        """gif_raw = 1 if median < 1e-10 else median/0.4549; calibration uses
        max(gif_raw, 1); reported gif is the mean of raw values
        (src/testing.rs:159-176)."""
        d = self.counts.shape[0]
        raw = np.empty(d)
        for j in range(d):
            med = self.median_for_trait(j)
            raw[j] = 1.0 if med < 1e-10 else med / GIF_DIVISOR
        return np.maximum(raw, 1.0), float(raw.sum() / d)


def t_test(coef: np.ndarray, sigma2: np.ndarray, ctc_inv_jj: float) -> np.ndarray:
    """src/testing.rs:1036-1048 (the p-value there is discarded)."""
    with np.errstate(invalid="ignore", divide="ignore"):
        se = np.sqrt(sigma2 * ctc_inv_jj)
        t = coef / se
    bad = ~(se >= 1e-300) | ~np.isfinite(se) | ~np.isfinite(t)
    return np.where(bad, 0.0, t)


def calibrate_p(t: np.ndarray, gif_per_trait: np.ndarray) -> np.ndarray:
    """p = 2 Phi(-|t| / sqrt(GIF_j)) (src/testing.rs:685-728); statrs'
    Normal cdf(x) = 0.5 erfc(-x/sqrt 2), so p = erfc(|z|/sqrt 2)."""
    from scipy.special import erfc
    z = np.asarray(t) / np.sqrt(np.asarray(gif_per_trait))[None, :]
    return 2.0 * (0.5 * erfc(np.abs(z) / math.sqrt(2.0)))


@dataclass
class AssocResults:
    beta: np.ndarray       # (p, d)
    tstat: np.ndarray      # (p, d)
    pvalue: np.ndarray     # (p, d)
    r2: np.ndarray         # (p, 3): r2_cov, r2_latent, r2_resid
    gif_per_trait: np.ndarray
    gif: float
    hist: Optional[TsqHistogram] = None
    extra: dict = field(default_factory=dict)


def check_df(n: int, d: int, k: int) -> float:
    """df = n - 1 - d - K must be positive (src/testing.rs:272-279)."""
    if n <= 1 + d + k:
        raise ValueError(
            f"Insufficient degrees of freedom: n={n} samples but 1+d+K=1+{d}+{k}={1 + d + k}.")
    return float(n - 1 - d - k)


def _per_snp_stats(y: np.ndarray, coefs: np.ndarray, rss: np.ndarray, ss_cov: np.ndarray,
                   tss: np.ndarray, ctc_inv_diag: np.ndarray, df: float, d: int):
    sigma2 = rss / df
    t = np.empty((y.shape[1], d))
    for j in range(d):
        t[:, j] = t_test(coefs[1 + j], sigma2, ctc_inv_diag[j])
    r2 = np.zeros((y.shape[1], 3))
    ok = tss > 1e-300                                             # src/testing.rs:394-404
    ss_lat = np.maximum(tss - rss - ss_cov, 0.0)
    r2[ok, 0] = ss_cov[ok] / tss[ok]
    r2[ok, 1] = ss_lat[ok] / tss[ok]
    r2[ok, 2] = rss[ok] / tss[ok]
    return t, r2


def assoc_ref(y_full: np.ndarray, xs: np.ndarray, u_hat: np.ndarray, pre: PrecomputedFull,
              chunk: int) -> AssocResults:
    """Faithful restatement of test_associations_fused (src/testing.rs:252-528)
    with its n x n P_U, I - P_U and H_X."""
    n, p = y_full.shape
    d = xs.shape[1]
    k = u_hat.shape[1]
    df = check_df(n, d, k)
    utu_inv, _ = safe_inv(u_hat.T @ u_hat, "U_hat^T U_hat")
    p_u = u_hat @ utu_inv @ u_hat.T
    xtr = pre.ridge_inv @ xs.T
    i_minus_pu = np.eye(n) - p_u
    c = np.hstack([np.ones((n, 1)), xs, u_hat])
    ctc_inv, _ = safe_inv(c.T @ c, "C^T C")
    h = ctc_inv @ c.T
    xtx_inv, _ = safe_inv(xs.T @ xs, "X^T X")
    hx = xs @ xtx_inv @ xs.T
    ctc_inv_diag = np.array([ctc_inv[1 + j, 1 + j] for j in range(d)])
    hist = TsqHistogram(d)
    beta = np.empty((p, d))
    tstat = np.empty((p, d))
    r2 = np.empty((p, 3))
    for s in range(0, p, chunk):
        e = min(s + chunk, p)
        ch = y_full[:, s:e]
        b = xtr @ (i_minus_pu @ ch)                                  # :360-362
        coefs = h @ ch                                               # :365
        res = ch - c @ coefs                                         # :366-367
        fx = hx @ ch                                                 # :374
        rss = np.einsum("ij,ij->j", res, res)
        tss = np.einsum("ij,ij->j", ch, ch)
        ss_cov = np.einsum("ij,ij->j", fx, fx)
        t, r2c = _per_snp_stats(ch, coefs, rss, ss_cov, tss, ctc_inv_diag, df, d)
        hist.add_chunk(t)
        beta[s:e] = b.T
        tstat[s:e] = t
        r2[s:e] = r2c
    gif_per_trait, gif = hist.compute_gif()
    return AssocResults(beta, tstat, calibrate_p(tstat, gif_per_trait), r2, gif_per_trait, gif, hist)


def assoc_oracle64(y_full: np.ndarray, xs: np.ndarray, u_hat: np.ndarray, ridge_inv: np.ndarray,
                   chunk: int = 4096) -> AssocResults:
    """Same per-SNP statistics with O(n (1+d+K)) work per SNP instead of the
    n x n projectors: coefs = H y, RSS = ||y - C coefs||^2,
    SS_cov = ||X (X^T X)^-1 X^T y||^2, beta = R X^T (y - U (U^T U)^-1 U^T y)."""
    n, p = y_full.shape
    d = xs.shape[1]
    k = u_hat.shape[1]
    df = check_df(n, d, k)
    utu_inv, _ = safe_inv(u_hat.T @ u_hat, "U_hat^T U_hat")
    c = np.hstack([np.ones((n, 1)), xs, u_hat])
    ctc_inv, _ = safe_inv(c.T @ c, "C^T C")
    xtx_inv, _ = safe_inv(xs.T @ xs, "X^T X")
    ctc_inv_diag = np.array([ctc_inv[1 + j, 1 + j] for j in range(d)])
    hist = TsqHistogram(d)
    beta = np.empty((p, d))
    tstat = np.empty((p, d))
    r2 = np.empty((p, 3))
    for s in range(0, p, chunk):
        e = min(s + chunk, p)
        ch = y_full[:, s:e]
        coefs = ctc_inv @ (c.T @ ch)
        res = ch - c @ coefs
        rss = np.einsum("ij,ij->j", res, res)
        tss = np.einsum("ij,ij->j", ch, ch)
        xty = xs.T @ ch
        ss_cov = np.einsum("ij,ij->j", xty, xtx_inv @ xty)
        resid_u = ch - u_hat @ (utu_inv @ (u_hat.T @ ch))
        b = ridge_inv @ (xs.T @ resid_u)
        t, r2c = _per_snp_stats(ch, coefs, rss, ss_cov, tss, ctc_inv_diag, df, d)
        hist.add_chunk(t)
        beta[s:e] = b.T
        tstat[s:e] = t
        r2[s:e] = r2c
    gif_per_trait, gif = hist.compute_gif()
    return AssocResults(beta, tstat, calibrate_p(tstat, gif_per_trait), r2, gif_per_trait, gif, hist)


# ---------------------------------------------------------------------------
# NMF imputation  (src/nmf.rs, src/parallel.rs:219-321, src/testing.rs:423-487)
# ---------------------------------------------------------------------------

def normalize_w(w: np.ndarray, h: np.ndarray, eps: float) -> None:
    """L1-normalise W columns (if norm > eps) and scale H rows by the norm
    (src/nmf.rs:259-271)."""
    k = w.shape[1]
    for j in range(k):
        col_norm = float(np.sum(w[:, j]))
        if col_norm > eps:
            inv = 1.0 / col_norm
            w[:, j] *= inv
            if h.shape[0] == k:
                h[j, :] *= col_norm


def nmf_init_from_random_probe(raw_est: np.ndarray, k: int, seed: int, rng: str = "counter"):
    """src/nmf.rs:279-362: Omega' from seed+1e6 (``rng`` names the stream),
    Z = Y_meanraw^T Omega', W = |Omega' Vt[:k]^T|, H = max(0, W^+ Y_meanraw)."""
    n, p = raw_est.shape
    l = k + 10
    omega = sketch_normal(rng, seed + 1_000_000, n, l)
    y = fill_missing_with_column_means(raw_est)
    z = y.T @ omega
    _, _, vt = np.linalg.svd(z, full_matrices=False)
    w = np.abs(omega @ vt[:k, :].T)
    inv_wtw, _ = safe_inv(w.T @ w, "W_init^T W_init")
    w_pinv = inv_wtw @ w.T
    h = np.maximum(w_pinv @ y, 0.0)
    return w, h


def mask_uniform(rng: str, seed: int, ctr: np.ndarray) -> np.ndarray:
    """Hold-out uniforms: draw ``ctr`` of the stream keyed by ``seed``.
    "counter": (u64 >> 11) 2^-53 of the SplitMix64 counter stream;
    "chacha8": rand_distr's Uniform(0, 1) on ChaCha8Rng::seed_from_u64(seed),
    (u64 >> 12) 2^-52 of output ``ctr`` (src/nmf.rs:433-434,
    src/testing.rs:437-438)."""
    ctr = np.asarray(ctr, dtype=np.uint64)
    if rng == "counter":
        return rng_uniform(seed, ctr)
    if rng != "chacha8":
        raise ValueError(f"unknown stream {rng!r}")
    if ctr.size == 0:
        return np.zeros(ctr.shape)
    draws = chacha8_u64(seed, int(ctr.max()) + 1)
    return (draws[ctr] >> np.uint64(12)).astype(np.float64) * (2.0 ** -52)


def nmf_cv_error_masked(raw_est: np.ndarray, w: np.ndarray, h: np.ndarray, mask_seed: int,
                        cv_rate: float, chunk: int, rng: str = "counter") -> Tuple[float, float, int]:
    """src/nmf.rs:379-455: per chunk, one uniform per (col,row) in
    column-major order (missing included) from stream mask_seed+chunk_seq;
    masked iff u < cv_rate and observed."""
    n, p = raw_est.shape
    nmf_err = mean_err = 0.0
    cnt = 0
    for seq, s in enumerate(range(0, p, chunk)):
        e = min(s + chunk, p)
        y = raw_est[:, s:e]
        obs = ~np.isnan(y)
        n_obs = obs.sum(axis=0)
        col_mean = np.where(n_obs > 0, np.where(obs, y, 0.0).sum(axis=0) / np.maximum(n_obs, 1), 0.0)
        recon = w @ h[:, s:e]
        ctr = np.arange((e - s) * n, dtype=np.uint64).reshape(e - s, n).T   # counter = col*n + row
        u = mask_uniform(rng, mask_seed + seq, ctr)
        m = (u < cv_rate) & obs
        nmf_err += float(np.abs(y[m] - recon[m]).sum())
        mean_err += float(np.abs(y[m] - np.broadcast_to(col_mean, y.shape)[m]).sum())
        cnt += int(m.sum())
    if cnt == 0:
        return 0.0, 0.0, 0
    return nmf_err / cnt, mean_err / cnt, cnt


@dataclass
class NmfResult:
    w: np.ndarray
    h: np.ndarray
    cv_mae_per_iter: List[float]
    cv_mae_mean_impute: float
    total_mask_count: int


def nmf_impute_estimation(raw_est: np.ndarray, k: int, n_iter: int, eps: float, cv_rate: float,
                          seed: int, chunk: int, rng: str = "counter") -> NmfResult:
    """src/nmf.rs:80-249 on a raw (n, p_est) matrix with NaNs."""
    w, h = nmf_init_from_random_probe(raw_est, k, seed, rng)
    w = np.maximum(w, eps)
    h = np.maximum(h, eps)
    normalize_w(w, h, eps)
    nan = np.isnan(raw_est)
    cv, mean_mae, total = [], 0.0, 0
    for it in range(n_iter):
        y = raw_est.copy()
        y[nan] = (w @ h)[nan]                                        # NmfRawInRam fill
        num_w = y @ h.T
        hh = h @ h.T
        denom = w @ hh
        upd = denom > eps
        w = np.where(upd, w * np.divide(num_w, denom, out=np.ones_like(denom), where=upd), w)
        w = np.maximum(w, eps)
        normalize_w(w, h, eps)
        wtw = w.T @ w
        y = raw_est.copy()
        y[nan] = (w @ h)[nan]
        num_h = w.T @ y
        denom_h = wtw @ h
        upd = denom_h > eps
        h = np.where(upd, h * np.divide(num_h, denom_h, out=np.ones_like(denom_h), where=upd), h)
        h = np.maximum(h, eps)
        normalize_w(w, h, eps)
        mae, mmae, c = nmf_cv_error_masked(raw_est, w, h, seed + it, cv_rate, chunk, rng)
        cv.append(mae)
        mean_mae = mmae
        total += c
    return NmfResult(w, h, cv, mean_mae, total)


def nmf_onthefly_fill(raw: np.ndarray, w: np.ndarray, w_pinv: np.ndarray) -> np.ndarray:
    """NmfOnTheFly (src/parallel.rs:249-282): mean-fill, H = max(0, W^+ Y),
    fill values W H at the NaNs."""
    y = fill_missing_with_column_means(raw)
    h = np.maximum(w_pinv @ y, 0.0)
    return w @ h


def nmf_gwas_cv(raw: np.ndarray, w: np.ndarray, w_pinv: np.ndarray, cv_rate: float, seed: int,
                chunk: int, rng: str = "counter") -> Tuple[float, float, int]:
    """GWAS-phase CV (src/testing.rs:423-487): per block, one draw per
    OBSERVED entry in column-major order from stream seed+seq (the k-th
    observed entry uses counter k); leave-out mean fill; H = max(0, W^+ Y);
    MAE of W H and of the mean fill at the masked positions."""
    n, p = raw.shape
    nmf_err = mean_err = 0.0
    cnt = 0
    for seq, s in enumerate(range(0, p, chunk)):
        e = min(s + chunk, p)
        y = raw[:, s:e]
        obs = ~np.isnan(y)
        obs_cm = obs.T.reshape(-1)                     # column-major order
        rank = np.cumsum(obs_cm) - 1
        u = np.ones(obs_cm.shape)
        u[obs_cm] = mask_uniform(rng, seed + seq, rank[obs_cm].astype(np.uint64))
        m_cm = obs_cm & (u < cv_rate)
        mask = m_cm.reshape(e - s, n).T
        if not mask.any():
            continue
        masked = y.copy()
        masked[mask] = np.nan
        filled = fill_missing_with_column_means(masked)
        hh = np.maximum(w_pinv @ filled, 0.0)
        pred = w @ hh
        nmf_err += float(np.abs(y[mask] - pred[mask]).sum())
        mean_err += float(np.abs(y[mask] - filled[mask]).sum())
        cnt += int(mask.sum())
    if cnt == 0:
        return 0.0, 0.0, 0
    return nmf_err / cnt, mean_err / cnt, cnt


# ---------------------------------------------------------------------------
# Whole-pipeline oracle  (src/lib.rs:162-263)
# ---------------------------------------------------------------------------

@dataclass
class FitResult:
    u_hat: np.ndarray
    assoc: AssocResults
    nmf: Optional[NmfResult] = None
    gwas_cv: Optional[Tuple[float, float, int]] = None


def fit_oracle64(raw_est: np.ndarray, raw_full: np.ndarray, x: np.ndarray, *, k: int,
                 lam: float = 1e-5, oversampling: int = 10, power_iter: int = 2,
                 seed: int = 42, norm: int = NORM_EIGENSTRAT, scale_cov: bool = False,
                 omega: Optional[np.ndarray] = None, nmf: Optional[dict] = None,
                 chunk: int = 10_000, rng: str = "counter") -> FitResult:
    """fit_lfmm2 (src/lib.rs:162-263) in the thin FP64 formulation.

    ``raw_est``/``raw_full`` are raw (n, p) matrices with NaN for missing.
    ``nmf`` = dict(k=, n_iter=, eps=, cv_rate=) switches on NMF imputation.
    ``rng`` ("counter" or "chacha8") names the stream of the Gaussian
    sketches that are not given (Omega, the NMF probe) and of the CV
    hold-out masks."""
    xs = center_covariates(x, scale_cov)
    n, d = xs.shape
    pre = precompute_thin(xs, lam)
    l = k + oversampling
    if omega is None:
        omega = sketch_normal(rng, seed, n, l)
    nmf_res = None
    gwas_cv = None
    if nmf is not None:
        nmf_res = nmf_impute_estimation(raw_est, nmf["k"], nmf["n_iter"], nmf.get("eps", 1e-16),
                                        nmf["cv_rate"], seed, chunk, rng)
        w = nmf_res.w
        inv_wtw, _ = safe_inv(w.T @ w, "W^T W for NMF pinv")
        w_pinv = inv_wtw @ w.T
        fill_est = w @ nmf_res.h                                     # NmfInRam
        y_est, _, _ = decode_standardized(raw_est, norm, fill_est)
        fill_full = nmf_onthefly_fill(raw_full, w, w_pinv)           # NmfOnTheFly
        y_full, _, _ = decode_standardized(raw_full, norm, fill_full)
        gwas_cv = nmf_gwas_cv(raw_full, w, w_pinv, nmf["cv_rate"], seed, chunk, rng)
    else:
        y_est, _, _ = decode_standardized(raw_est, norm)
        y_full, _, _ = decode_standardized(raw_full, norm)
    u_hat = rsvd_thin(y_est, pre, k, l, power_iter, omega)
    assoc = assoc_oracle64(y_full, xs, u_hat, pre.ridge_inv)
    return FitResult(u_hat, assoc, nmf_res, gwas_cv)


# ---------------------------------------------------------------------------
# The same thin FP64 fit streamed from the packed payload, for shapes whose
# dense (n, p) matrix does not fit in host memory (n = 20 000 and more)
# ---------------------------------------------------------------------------

_DECODE_LIB = []


def _decode_helper():
    """The oracle's C decode helper (oracle/liboracle.so, built by
    oracle/build_oracle.py) when present; the NumPy decode otherwise."""
    if not _DECODE_LIB:
        import ctypes
        path = Path(__file__).resolve().parent / "liboracle.so"
        lib = None
        if path.exists():
            try:
                lib = ctypes.CDLL(str(path))
                lib.oracle_decode_rows.restype = ctypes.c_int
            except OSError:
                lib = None
        _DECODE_LIB.append(lib)
    return _DECODE_LIB[0]


class PackedMatrix:
    """A PLINK payload (p, ceil(n/4)) read as standardised SNP chunks
    (decode_single_snp, src/bed.rs:300-379, mean imputation): per-SNP mean
    and scale come from the integer allele counts (bit-identical to the
    reference's FP64 sums), and each code maps to (g - mean) * scale, a
    missing call to 0."""

    def __init__(self, packed: np.ndarray, n: int, norm: int, snps: Optional[np.ndarray] = None,
                 chunk: int = 4096):
        self.packed = np.asarray(packed, dtype=np.uint8)
        self.n = int(n)
        self.norm = norm
        self.snps = np.arange(self.packed.shape[0]) if snps is None else np.asarray(snps, dtype=np.int64)
        self.chunk = int(chunk)
        self.p = len(self.snps)
        self.mean = np.empty(self.p)
        self.scale = np.empty(self.p)
        self.counts = np.empty((self.p, 4), dtype=np.int64)
        for s, e in self.ranges():
            codes = unpack_codes(self.packed[self.snps[s:e]], self.n)
            cnt = np.stack([(codes == c).sum(axis=1) for c in (0, 2, 3, 1)], axis=1)
            self.counts[s:e] = cnt
        c0, c1, c2 = self.counts[:, 0], self.counts[:, 1], self.counts[:, 2]
        nobs = c0 + c1 + c2
        s1 = c1 + 2 * c2
        self.mean[:] = np.where(nobs > 0, s1.astype(np.float64) / np.maximum(nobs, 1).astype(np.float64), 0.0)
        self.scale[:] = compute_scale(self.mean, norm)
        # ||y||^2 of each standardised column, as snp_stats
        num = nobs * (c1 + 4 * c2) - s1 * s1
        css = np.where(nobs > 0, num.astype(np.float64) / np.maximum(nobs, 1), 0.0)
        self.tss = self.scale * self.scale * css

    def ranges(self):
        return [(s, min(s + self.chunk, self.p)) for s in range(0, self.p, self.chunk)]

    _BYTE_CODES = ((np.arange(256)[:, None] >> (2 * np.arange(4))[None, :]) & 3).astype(np.intp)

    def block(self, s: int, e: int) -> np.ndarray:
        """Standardised SNPs [s, e) as an (n, e - s) FP64 block."""
        lib = _decode_helper()
        if lib is not None:
            import ctypes
            rows = np.ascontiguousarray(self.snps[s:e], dtype=np.int64)
            out = np.empty((e - s, self.n))
            mean = np.ascontiguousarray(self.mean[s:e])
            scale = np.ascontiguousarray(self.scale[s:e])
            vp = ctypes.c_void_p
            rc = lib.oracle_decode_rows(self.packed.ctypes.data_as(vp), ctypes.c_uint64(self.packed.shape[1]),
                                        rows.ctypes.data_as(vp), ctypes.c_uint64(e - s), ctypes.c_uint64(self.n),
                                        mean.ctypes.data_as(vp), scale.ctypes.data_as(vp), out.ctypes.data_as(vp),
                                        ctypes.c_int(os.cpu_count() or 1))
            if rc == 0:
                return out.T
        m, sc = self.mean[s:e, None], self.scale[s:e, None]
        vals = np.concatenate([(0.0 - m) * sc, np.zeros_like(m), (1.0 - m) * sc, (2.0 - m) * sc], axis=1)
        # per SNP: the four values of each possible byte (4 samples per byte)
        lut = vals[:, self._BYTE_CODES]                      # (c, 256, 4)
        rows = self.packed[self.snps[s:e]]                   # (c, bps)
        out = lut[np.arange(e - s)[:, None], rows]           # (c, bps, 4)
        return out.reshape(e - s, -1)[:, :self.n].T

    def t_mul(self, w: np.ndarray) -> np.ndarray:
        """Y^T W (p, w)."""
        out = np.empty((self.p, w.shape[1]))
        for s, e in self.ranges():
            out[s:e] = self.block(s, e).T @ w
        return out

    def mul(self, q: np.ndarray) -> np.ndarray:
        """Y Q (n, w) for Q (p, w)."""
        acc = np.zeros((self.n, q.shape[1]))
        for s, e in self.ranges():
            acc += self.block(s, e) @ q[s:e]
        return acc


def rsvd_thin_packed(y: PackedMatrix, pre: PrecomputedThin, k: int, l: int, q_iter: int,
                     omega: np.ndarray) -> np.ndarray:
    """rsvd_thin on a PackedMatrix: the same passes (src/rsvd.rs:26-177), each
    streamed over SNP chunks."""
    z = y.t_mul(pre.apply_p(omega))
    q_z = _qr_q(z)
    for _ in range(q_iter):
        q_s = _qr_q(pre.apply_p(y.mul(q_z)))
        q_z = _qr_q(y.t_mul(pre.apply_p(q_s)))
    u_b, _, _ = np.linalg.svd(pre.apply_p(y.mul(q_z)), full_matrices=False)
    return pre.apply_pinv(u_b[:, :k])


def assoc_oracle64_packed(y: PackedMatrix, xs: np.ndarray, u_hat: np.ndarray,
                          ridge_inv: np.ndarray) -> AssocResults:
    """assoc_oracle64 with the SNP chunks decoded from a PackedMatrix.  Every
    per-SNP statistic follows from T = C^T y (one FP64 product per chunk):
    coefs = (C^T C)^-1 T; RSS = ||y||^2 - coefs^T T (= ||y - C coefs||^2 for
    the least-squares coefs, src/testing.rs:365-371); SS_cov = (X^T y)^T
    (X^T X)^-1 (X^T y) (:374-377); beta = R (X^T y - X^T U (U^T U)^-1 U^T y)
    (:360-362); ||y||^2 from the SNP's allele counts (exact integers).  At
    n = 20 000 the residual matrix of the dense form would be rebuilt for
    every chunk; the forms are equal in exact arithmetic and agree to FP64
    rounding (RSS keeps > 90 % of TSS in these cohorts)."""
    n, d = xs.shape
    k = u_hat.shape[1]
    df = check_df(n, d, k)
    utu_inv, _ = safe_inv(u_hat.T @ u_hat, "U_hat^T U_hat")
    c = np.hstack([np.ones((n, 1)), xs, u_hat])
    ctc_inv, _ = safe_inv(c.T @ c, "C^T C")
    xtx_inv, _ = safe_inv(xs.T @ xs, "X^T X")
    xtu = xs.T @ u_hat
    ctc_inv_diag = np.array([ctc_inv[1 + j, 1 + j] for j in range(d)])
    hist = TsqHistogram(d)
    beta = np.empty((y.p, d))
    tstat = np.empty((y.p, d))
    r2 = np.empty((y.p, 3))
    for s, e in y.ranges():
        ch = y.block(s, e)
        ct = c.T @ ch
        coefs = ctc_inv @ ct
        tss = y.tss[s:e]
        rss = tss - np.einsum("ij,ij->j", coefs, ct)
        xty = ct[1:1 + d]
        ss_cov = np.einsum("ij,ij->j", xty, xtx_inv @ xty)
        b = ridge_inv @ (xty - xtu @ (utu_inv @ ct[1 + d:]))
        t, r2c = _per_snp_stats(ch, coefs, rss, ss_cov, tss, ctc_inv_diag, df, d)
        hist.add_chunk(t)
        beta[s:e] = b.T
        tstat[s:e] = t
        r2[s:e] = r2c
    gif_per_trait, gif = hist.compute_gif()
    return AssocResults(beta, tstat, calibrate_p(tstat, gif_per_trait), r2, gif_per_trait, gif, hist)


def fit_oracle64_packed(packed: np.ndarray, n: int, x: np.ndarray, *, k: int, lam: float = 1e-5,
                        oversampling: int = 10, power_iter: int = 2, norm: int = NORM_EIGENSTRAT,
                        scale_cov: bool = False, omega: np.ndarray, est_snps: Optional[np.ndarray] = None,
                        chunk: int = 4096) -> FitResult:
    """fit_oracle64 (mean imputation) from a packed payload, streamed in SNP
    chunks so that no (n, p) matrix exists; ``est_snps`` selects the
    estimation rows (SubsetSpec)."""
    xs = center_covariates(x, scale_cov)
    pre = precompute_thin(xs, lam)
    l = k + oversampling
    y_est = PackedMatrix(packed, n, norm, est_snps, chunk)
    u_hat = rsvd_thin_packed(y_est, pre, k, l, power_iter, omega)
    y_full = y_est if est_snps is None else PackedMatrix(packed, n, norm, None, chunk)
    return FitResult(u_hat, assoc_oracle64_packed(y_full, xs, u_hat, pre.ridge_inv))


def principal_angles_sin_max(a: np.ndarray, b: np.ndarray) -> float:
    """sin of the largest principal angle between span(a) and span(b)."""
    qa, _ = np.linalg.qr(a)
    qb, _ = np.linalg.qr(b)
    resid = qb - qa @ (qa.T @ qb)          # ||(I - P_a) Q_b||_2 = sin(theta_max)
    return float(np.linalg.norm(resid, 2))


# ---------------------------------------------------------------------------
# Output formatting  (src/testing.rs:740-801)
# ---------------------------------------------------------------------------

def rust_exp(v: float, prec: int) -> str:
    """Rust ``format!("{:.prec$e}", v)`` of a finite value (the safe_inv
    warning's ``{:.2e}``, src/testing.rs:1006-1009): exponent without '+' or
    zero padding."""
    mant, exp = ("%.*e" % (prec, v)).split("e")
    return f"{mant}e{int(exp)}"


def rust_lower_exp6(v: float) -> str:
    """Rust ``format!("{:.6e}", v)``: 7 significant digits, exponent without
    '+' or zero padding; NaN -> 'NaN', +-inf -> 'inf'/'-inf'."""
    if math.isnan(v):
        return "NaN"
    if math.isinf(v):
        return "inf" if v > 0 else "-inf"
    s = "%.6e" % v
    mant, exp = s.split("e")
    return f"{mant}e{int(exp)}"


def tsv_header(cov_names: Sequence[str]) -> str:
    cols = ["chr", "pos", "snp_id"]
    for c in cov_names:
        cols += [f"p_{c}", f"beta_{c}", f"t_{c}"]
    cols += ["r2_cov", "r2_latent", "r2_resid"]
    return "\t".join(cols)


def tsv_rows(chrom: Sequence[str], pos: Sequence[int], snp_id: Sequence[str], res: AssocResults) -> List[str]:
    d = res.beta.shape[1]
    out = []
    for i in range(res.beta.shape[0]):
        f = [str(chrom[i]), str(pos[i]), str(snp_id[i])]
        for j in range(d):
            f += [rust_lower_exp6(res.pvalue[i, j]), rust_lower_exp6(res.beta[i, j]),
                  rust_lower_exp6(res.tstat[i, j])]
        f += [rust_lower_exp6(v) for v in res.r2[i]]
        out.append("\t".join(f))
    return out
