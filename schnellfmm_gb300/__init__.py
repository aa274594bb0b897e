"""schnellfmm_gb300 -- GB300-native streaming LFMM2 (host mirror of schnelLFMM).

The compute runs in ``libschnelgpu.so`` (sm_103a CUDA kernels behind the C
ABI declared in ``include/schnelgpu.h``).  This module is a thin ctypes host
layer that mirrors the reference crate's library surface:

=============================  ============================================
reference (src/lib.rs, ...)    here
=============================  ============================================
``BedFile::open``              :meth:`BedFile.open`  (src/bed.rs:78-135)
``BedFile::subset_samples``    :meth:`BedFile.subset_samples` (:155-159)
``SubsetSpec``                 :class:`SubsetSpec`   (src/bed.rs:50-57)
``SnpNorm``                    :class:`SnpNorm`      (src/bed.rs:19-26)
``Lfmm2Config`` / ``NmfConfig``:class:`Lfmm2Config` / :class:`NmfConfig`
``load_covariates`` (CLI)      :func:`load_covariates`   (src/main.rs:339-571)
``center_covariates``          :func:`center_covariates` (src/lib.rs:102-117)
``estimate_factors``           :func:`estimate_factors`  (src/lib.rs:127-136)
``test_associations``          :func:`test_associations` (src/lib.rs:144-154)
``fit_lfmm2``                  :func:`fit_lfmm2`         (src/lib.rs:162-263)
``TestResults``                :class:`TestResults`  (src/testing.rs:76-93)
=============================  ============================================

There is no CPU fallback: without the built library or an sm_103a device
every call raises :class:`SchnelGpuError`.
"""
from __future__ import annotations

import ctypes as C
import enum
import weakref
import math
import os
import sys
from dataclasses import dataclass, field
from pathlib import Path
from typing import List, Optional, Sequence, Tuple

import numpy as np

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "libschnelgpu.so"

OK = 0
ERR_BAD_ARG = -1
ERR_BAD_BED = -2
ERR_SINGULAR = -3
ERR_DF_NONPOSITIVE = -4
ERR_CUDA = -5
ERR_DEVICE_TIMEOUT = -6
ERR_IO = -7
ERR_NOMEM = -8


class SchnelGpuError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


class SnpNorm(enum.IntEnum):
    CENTER_ONLY = 0   # library default (src/bed.rs:22-23)
    EIGENSTRAT = 1    # CLI default (src/main.rs:79-80)


class ImputeStrategy(enum.IntEnum):
    MEAN = 0
    NMF = 1


class Precision(enum.IntEnum):
    FP32 = 0
    SPLIT_BF16 = 1
    SPLIT_FP8 = 2


class SketchRng(enum.IntEnum):
    """Streams of the Gaussian sketches (src/rsvd.rs:44-46,
    src/nmf.rs:291-293) and the NMF CV hold-out masks (src/nmf.rs:433-448,
    src/testing.rs:437-452): the device counter streams, or the reference's
    ChaCha8Rng::seed_from_u64 streams (Normal(0, 1) sketches drawn on the
    host threads, Uniform(0, 1) masks drawn on the device), the default."""
    CHACHA8 = 0
    COUNTER = 1


# ---------------------------------------------------------------------------
# ctypes declarations (must match include/schnelgpu.h)
# ---------------------------------------------------------------------------
class _Opts(C.Structure):
    _fields_ = [("precision", C.c_int), ("verbose", C.c_int), ("stream", C.c_void_p), ("autotune", C.c_int),
                ("rng", C.c_int)]


class _Subset(C.Structure):
    _fields_ = [("kind", C.c_int), ("rate", C.c_double), ("indices", C.POINTER(C.c_uint64)),
                ("n_indices", C.c_uint64)]


class _Config(C.Structure):
    _fields_ = [("k", C.c_uint32), ("lambda_", C.c_double), ("chunk_size", C.c_uint32),
                ("oversampling", C.c_uint32), ("n_power_iter", C.c_uint32), ("seed", C.c_uint64),
                ("norm", C.c_int), ("scale_cov", C.c_int), ("impute", C.c_int), ("nmf_k", C.c_uint32),
                ("nmf_iter", C.c_uint32), ("nmf_eps", C.c_double), ("nmf_cv_rate", C.c_double)]


_dp = C.POINTER(C.c_double)


class _Problem(C.Structure):
    _fields_ = [("packed", C.c_void_p), ("n_physical", C.c_uint64), ("n_snps", C.c_uint64), ("x", C.c_void_p),
                ("d", C.c_uint32), ("cfg", C.c_void_p), ("omega", C.c_void_p), ("res", C.c_void_p)]


class _Results(C.Structure):
    _fields_ = [("u_hat", _dp), ("beta", _dp), ("tstat", _dp), ("pvalue", _dp), ("r2", _dp),
                ("gif_per_trait", _dp), ("gif", C.c_double), ("nmf_cv", _dp), ("nmf_cv_mean", C.c_double),
                ("nmf_gwas_cv_mae", C.c_double), ("nmf_gwas_cv_mean_mae", C.c_double),
                ("nmf_gwas_cv_count", C.c_uint64)]


EXPORTED_SYMBOLS = (
    "slfmm_create", "slfmm_destroy", "slfmm_last_error", "slfmm_launch_count", "slfmm_stream",
    "slfmm_bed_validate", "slfmm_geno_upload", "slfmm_geno_free", "slfmm_geno_n_samples",
    "slfmm_geno_n_snps", "slfmm_decode_stats", "slfmm_decode_chunk", "slfmm_center_covariates",
    "slfmm_generate_omega", "slfmm_estimate_factors", "slfmm_test_associations", "slfmm_fit",
    "slfmm_fit_host", "slfmm_write_tsv", "slfmm_format_exp6", "slfmm_simulate", "slfmm_geno_download",
    "slfmm_profile_enable", "slfmm_profile_read", "slfmm_host_alloc", "slfmm_host_free", "slfmm_contract_raw",
    "slfmm_gif_noalloc", "slfmm_fit_traits", "slfmm_fit_many", "slfmm_reference_normal", "slfmm_write_parquet",
    "slfmm_phase_count", "slfmm_phase_read", "slfmm_debug_expire_next_wait", "slfmm_small_eigh",
)

_lib_handle = None


def load_library(path: Optional[os.PathLike] = None) -> C.CDLL:
    """Load the C-ABI library (raises if it was never built)."""
    global _lib_handle
    if _lib_handle is not None and path is None:
        return _lib_handle
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise SchnelGpuError(ERR_CUDA, f"{p} is not built; run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(p))
    vp, u64, i32, u32 = C.c_void_p, C.c_uint64, C.c_int, C.c_uint32
    sig = {
        "slfmm_create": (i32, [i32, C.POINTER(_Opts), C.POINTER(vp)]),
        "slfmm_destroy": (None, [vp]),
        "slfmm_last_error": (C.c_char_p, [vp]),
        "slfmm_launch_count": (u64, [vp]),
        "slfmm_stream": (vp, [vp]),
        "slfmm_bed_validate": (i32, [C.c_char_p, u64, u64, vp, C.c_char_p, C.c_size_t]),
        "slfmm_geno_upload": (i32, [vp, vp, u64, u64, C.POINTER(u64), u64, C.POINTER(_Subset), C.POINTER(vp)]),
        "slfmm_geno_free": (i32, [vp, vp]),
        "slfmm_geno_n_samples": (u64, [vp]),
        "slfmm_geno_n_snps": (u64, [vp]),
        "slfmm_decode_stats": (i32, [vp, vp, i32, vp, vp, vp, vp]),
        "slfmm_decode_chunk": (i32, [vp, vp, u64, u64, i32, vp]),
        "slfmm_center_covariates": (i32, [vp, vp, u64, u32, i32, vp]),
        "slfmm_generate_omega": (i32, [vp, u64, u64, u32, vp]),
        "slfmm_estimate_factors": (i32, [vp, vp, vp, u32, C.POINTER(_Config), vp, vp]),
        "slfmm_test_associations": (i32, [vp, vp, vp, u32, vp, C.POINTER(_Config), C.POINTER(_Results)]),
        "slfmm_fit": (i32, [vp, vp, vp, vp, u32, C.POINTER(_Config), vp, C.POINTER(_Results)]),
        "slfmm_fit_host": (i32, [vp, vp, u64, u64, C.POINTER(u64), u64, C.POINTER(_Subset), vp, u32,
                                 C.POINTER(_Config), vp, C.POINTER(_Results)]),
        "slfmm_write_tsv": (i32, [C.c_char_p, u64, u32, C.POINTER(C.c_char_p), C.POINTER(u64),
                                  C.POINTER(C.c_char_p), C.POINTER(C.c_char_p), C.POINTER(_Results), i32]),
        "slfmm_format_exp6": (i32, [C.c_double, C.c_char_p, C.c_size_t]),
        "slfmm_simulate": (i32, [vp, u64, u64, u32, vp, C.c_double, C.c_double, C.c_double, C.c_double,
                                 C.c_double, u64, C.POINTER(vp)]),
        "slfmm_geno_download": (i32, [vp, vp, vp]),
        "slfmm_profile_enable": (i32, [vp, i32]),
        "slfmm_profile_read": (i32, [vp, C.c_char_p, _dp, C.POINTER(u64), _dp, _dp]),
        "slfmm_phase_count": (i32, [vp]),
        "slfmm_small_eigh": (i32, [vp, vp, u32, vp, vp]),
        "slfmm_debug_expire_next_wait": (i32, [vp, u64]),
        "slfmm_phase_read": (i32, [vp, i32, C.c_char_p, C.c_size_t, _dp, _dp]),
        "slfmm_host_alloc": (i32, [C.c_size_t, C.POINTER(vp)]),
        "slfmm_host_free": (i32, [vp]),
        "slfmm_contract_raw": (i32, [vp, vp, i32, vp, u32, vp]),
        "slfmm_gif_noalloc": (i32, [vp, vp, u64, u32, vp]),
        "slfmm_fit_traits": (i32, [vp, vp, vp, vp, u32, C.POINTER(_Config), C.POINTER(_Results)]),
        "slfmm_fit_many": (i32, [vp, C.POINTER(_Problem), u32, u32, C.POINTER(C.c_int)]),
        "slfmm_reference_normal": (i32, [u64, u64, u32, vp]),
        "slfmm_write_parquet": (i32, [C.c_char_p, u64, u32, C.POINTER(C.c_char_p), C.POINTER(u64),
                                      C.POINTER(C.c_char_p), C.POINTER(C.c_char_p), C.POINTER(_Results), i32, i32]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib_handle = lib
    return lib


def reference_normal(seed: int, rows: int, cols: int) -> np.ndarray:
    """rows x cols Normal(0, 1) draws from ChaCha8Rng::seed_from_u64(seed) in
    row-major order, the reference's sketch Omega (src/rsvd.rs:44-46; the NMF
    probe uses seed + 1 000 000, src/nmf.rs:291-293).  Host only: needs the
    built library, not a GPU.  Pass it as ``omega=`` or create the engine
    with ``rng=SketchRng.CHACHA8`` to draw every sketch this way."""
    out = np.empty((rows, cols))
    rc = load_library().slfmm_reference_normal(seed & 0xFFFFFFFFFFFFFFFF, rows, cols, _ptr(out))
    if rc != OK:
        raise SchnelGpuError(rc, f"slfmm_reference_normal failed ({rc})")
    return out


class PinnedArray:
    """Page-locked host array (cudaMallocHost) exposed as a numpy array."""

    def __init__(self, shape, dtype):
        self.lib = load_library()
        dt = np.dtype(dtype)
        nbytes = int(np.prod(shape)) * dt.itemsize
        self.ptr = C.c_void_p()
        rc = self.lib.slfmm_host_alloc(nbytes, C.byref(self.ptr))
        if rc != OK:
            raise SchnelGpuError(rc, f"pinned allocation of {nbytes} bytes failed")
        buf = (C.c_uint8 * max(nbytes, 1)).from_address(self.ptr.value) if nbytes else bytearray(1)
        self.array = np.frombuffer(buf, dtype=dt, count=int(np.prod(shape))).reshape(shape)

    def free(self):
        if self.ptr:
            self.array = None
            self.lib.slfmm_host_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _dptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(_dp)


def _check_shape(name: str, a: Optional[np.ndarray], rows: int, cols: Optional[int] = None) -> None:
    """The library reads host matrices with the shapes a call implies; a
    mismatch is an argument error here, never a read past the buffer."""
    if a is None:
        return
    if a.ndim != 2 or a.shape[0] != rows or (cols is not None and a.shape[1] != cols):
        want = f"({rows}, {'d' if cols is None else cols})"
        raise SchnelGpuError(ERR_BAD_ARG, f"{name} has shape {a.shape}, expected {want}")


def _payload(packed: np.ndarray, n_physical: int) -> Tuple[np.ndarray, int]:
    """The SNP-major .bed payload as contiguous bytes and its SNP count."""
    packed = np.ascontiguousarray(packed, dtype=np.uint8)
    bps = (n_physical + 3) // 4
    n_snps = packed.size // bps if bps else 0
    if packed.size != n_snps * bps:
        raise SchnelGpuError(ERR_BAD_BED, "payload size is not a multiple of ceil(n/4)")
    return packed, n_snps


# ---------------------------------------------------------------------------
# configuration mirrors
# ---------------------------------------------------------------------------
@dataclass
class NmfConfig:
    """src/nmf.rs:15-50."""
    k: int = 5
    n_iter: int = 10
    eps: float = 1e-16
    cv_rate: float = 0.0005
    chunk_size: int = 10_000
    n_workers: int = 0
    progress: bool = False
    seed: int = 42


@dataclass
class Lfmm2Config:
    """src/lib.rs:47-98 (norm defaults to CenterOnly like the library)."""
    k: int = 5
    lambda_: float = 1e-5
    chunk_size: int = 10_000
    oversampling: int = 10
    n_power_iter: int = 2
    seed: int = 42
    n_workers: int = 0
    progress: bool = False
    norm: SnpNorm = SnpNorm.CENTER_ONLY
    scale_cov: bool = False
    impute: ImputeStrategy = ImputeStrategy.MEAN
    nmf: Optional[NmfConfig] = None

    def _c(self) -> _Config:
        nmf = self.nmf or NmfConfig(k=self.k)
        return _Config(self.k, self.lambda_, self.chunk_size, self.oversampling, self.n_power_iter,
                       self.seed & 0xFFFFFFFFFFFFFFFF, int(self.norm), int(self.scale_cov), int(self.impute),
                       nmf.k, nmf.n_iter, nmf.eps, nmf.cv_rate)


@dataclass
class SubsetSpec:
    """All / Rate(r) / Indices(v) (src/bed.rs:50-57)."""
    kind: str = "all"
    rate: float = 1.0
    indices: Optional[np.ndarray] = None

    @staticmethod
    def all() -> "SubsetSpec":
        return SubsetSpec("all")

    @staticmethod
    def from_rate(rate: float) -> "SubsetSpec":
        if not 0.0 < rate <= 1.0:       # src/main.rs:169-172
            raise SchnelGpuError(ERR_BAD_ARG, f"--est-rate must be in (0.0, 1.0], got {rate}")
        return SubsetSpec("rate", rate=rate)

    @staticmethod
    def from_indices(idx: Sequence[int]) -> "SubsetSpec":
        return SubsetSpec("indices", indices=np.ascontiguousarray(idx, dtype=np.uint64))

    def _c(self) -> _Subset:
        if self.kind == "all":
            return _Subset(0, 1.0, None, 0)
        if self.kind == "rate":
            return _Subset(1, float(self.rate), None, 0)
        idx = self.indices
        return _Subset(2, 1.0, idx.ctypes.data_as(C.POINTER(C.c_uint64)), len(idx))

    def count(self, n_snps: int) -> int:
        """subset_snp_count (src/bed.rs:162-171)."""
        if self.kind == "all":
            return n_snps
        if self.kind == "rate":
            step = math.ceil(1.0 / self.rate)
            return (n_snps + step - 1) // step
        return len(self.indices)


@dataclass
class TestResults:
    """src/testing.rs:76-93 plus the per-SNP columns of <out>.tsv."""
    u_hat: np.ndarray
    gif: float
    gif_per_trait: np.ndarray
    beta: np.ndarray
    tstat: np.ndarray
    pvalue: np.ndarray
    r2: np.ndarray
    nmf_cv: Optional[List[float]] = None
    nmf_cv_mean: Optional[float] = None
    nmf_gwas_cv_mae: Optional[float] = None
    nmf_gwas_cv_mean_mae: Optional[float] = None
    nmf_gwas_cv_count: Optional[int] = None

    __test__ = False  # not a pytest class


# ---------------------------------------------------------------------------
# engine + resident genotypes
# ---------------------------------------------------------------------------
class Engine:
    """One CUDA context + stream on one device (replaces the worker pool)."""

    def __init__(self, device: int = 0, precision: Precision = Precision.SPLIT_FP8, stream: Optional[int] = None,
                 verbose: bool = False, autotune: bool = False, rng: SketchRng = SketchRng.CHACHA8):
        self.lib = load_library()
        opts = _Opts(int(precision), int(verbose), C.c_void_p(stream) if stream else None, int(autotune),
                     int(rng))
        h = C.c_void_p()
        rc = self.lib.slfmm_create(device, C.byref(opts), C.byref(h))
        if rc != OK:
            raise SchnelGpuError(rc, f"slfmm_create failed ({rc})")
        self.h = h
        self.precision = Precision(precision)
        self._genos = weakref.WeakSet()

    def close(self):
        if getattr(self, "h", None):
            for g in list(self._genos):     # device buffers go first, on a live stream
                g.free()
            self.lib.slfmm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def check(self, rc: int):
        if rc != OK:
            msg = self.lib.slfmm_last_error(self.h)
            raise SchnelGpuError(rc, msg.decode() if msg else f"error {rc}")

    @property
    def launches(self) -> int:
        return int(self.lib.slfmm_launch_count(self.h))

    @property
    def stream(self) -> int:
        return int(self.lib.slfmm_stream(self.h) or 0)

    def upload(self, packed: np.ndarray, n_physical: int, sample_keep: Optional[Sequence[int]] = None,
               snps: Optional[SubsetSpec] = None) -> "Genotypes":
        packed, n_snps = _payload(packed, n_physical)
        keep = None if sample_keep is None else np.ascontiguousarray(sample_keep, dtype=np.uint64)
        sub = (snps or SubsetSpec.all())._c()
        h = C.c_void_p()
        self.check(self.lib.slfmm_geno_upload(
            self.h, _ptr(packed), n_physical, n_snps,
            None if keep is None else keep.ctypes.data_as(C.POINTER(C.c_uint64)),
            0 if keep is None else len(keep), C.byref(sub), C.byref(h)))
        return Genotypes(self, h)

    def simulate(self, admix: np.ndarray, p: int, *, fst: float, f_lo: float, f_hi: float, miss: float,
                 inbreeding: float = 0.0, seed: int = 42) -> "Genotypes":
        """Structured synthetic cohort drawn on the device (benchmark inputs)."""
        q = np.ascontiguousarray(admix, dtype=np.float32)
        h = C.c_void_p()
        self.check(self.lib.slfmm_simulate(self.h, q.shape[0], p, q.shape[1], _ptr(q), fst, f_lo, f_hi, miss,
                                           inbreeding, seed & 0xFFFFFFFFFFFFFFFF, C.byref(h)))
        return Genotypes(self, h)

    def profile(self, on: bool) -> None:
        self.check(self.lib.slfmm_profile_enable(self.h, int(on)))

    def profile_read(self, kernel: str) -> dict:
        ms, b, f = C.c_double(), C.c_double(), C.c_double()
        n = C.c_uint64()
        self.check(self.lib.slfmm_profile_read(self.h, kernel.encode(), C.byref(ms), C.byref(n), C.byref(b),
                                               C.byref(f)))
        return {"ms": ms.value, "launches": n.value, "bytes": b.value, "flops": f.value}

    def phases(self) -> List[dict]:
        """Phases of the last fit run with profiling on: name, device time
        (events on the stream) and host wall time, in ms."""
        out = []
        for i in range(self.lib.slfmm_phase_count(self.h)):
            name = C.create_string_buffer(96)
            dev, host = C.c_double(), C.c_double()
            self.check(self.lib.slfmm_phase_read(self.h, i, name, 96, C.byref(dev), C.byref(host)))
            out.append({"phase": name.value.decode(), "device_ms": dev.value, "host_ms": host.value})
        return out

    def small_eigh(self, a: np.ndarray):
        """Eigenvalues (descending) and eigenvectors (columns) of a small
        symmetric PSD matrix by the engine's FP32-sweep / FP64-refined Jacobi
        solve (the parity hook of the Step 0 and RSVD eigen-solves)."""
        a = np.ascontiguousarray(a, dtype=np.float64)
        m = a.shape[0]
        v = np.empty((m, m))
        s = np.empty(m)
        self.check(self.lib.slfmm_small_eigh(self.h, _ptr(a), m, _ptr(v), _ptr(s)))
        return s, v

    def generate_omega(self, seed: int, n: int, l: int) -> np.ndarray:
        out = np.empty((n, l))
        self.check(self.lib.slfmm_generate_omega(self.h, seed & 0xFFFFFFFFFFFFFFFF, n, l, _ptr(out)))
        return out

    def center_covariates(self, x: np.ndarray, scale: bool) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.empty_like(x)
        self.check(self.lib.slfmm_center_covariates(self.h, _ptr(x), x.shape[0], x.shape[1], int(scale), _ptr(out)))
        return out


class Genotypes:
    """Device-resident packed genotype matrix (slfmm_geno)."""

    def __init__(self, eng: Engine, h: C.c_void_p):
        self.eng = eng
        self.h = h
        eng._genos.add(self)

    @property
    def n_samples(self) -> int:
        return int(self.eng.lib.slfmm_geno_n_samples(self.h))

    @property
    def n_snps(self) -> int:
        return int(self.eng.lib.slfmm_geno_n_snps(self.h))

    def free(self):
        if self.h:
            self.eng.lib.slfmm_geno_free(self.eng.h, self.h)   # eng.h may be None: default stream
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def decode_stats(self, norm: SnpNorm):
        p = self.n_snps
        counts = np.empty((p, 4), dtype=np.int32)
        mean, scale, tss = np.empty(p), np.empty(p), np.empty(p)
        self.eng.check(self.eng.lib.slfmm_decode_stats(self.eng.h, self.h, int(norm), _ptr(counts), _ptr(mean),
                                                       _ptr(scale), _ptr(tss)))
        return counts, mean, scale, tss

    def download(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        """PLINK payload (p x ceil(n/4) bytes) of the resident matrix."""
        bps = (self.n_samples + 3) // 4
        if out is None:
            out = np.empty((self.n_snps, bps), dtype=np.uint8)
        self.eng.check(self.eng.lib.slfmm_geno_download(self.eng.h, self.h, _ptr(out)))
        return out

    def contract_raw(self, w: np.ndarray, transposed: bool = False, missing_as_one: bool = False) -> np.ndarray:
        """Tensor-core product of the exact genotypes (missing = 0, or 1 with
        ``missing_as_one``) with the engine's split of ``w``: G~^T w (w is
        n x c) or G~ w (w is p x c)."""
        w = np.ascontiguousarray(w, dtype=np.float64)
        rows = self.n_samples if transposed else self.n_snps
        out = np.empty((rows, w.shape[1]), dtype=np.float32)
        flags = int(transposed) | (2 if missing_as_one else 0)
        self.eng.check(self.eng.lib.slfmm_contract_raw(self.eng.h, self.h, flags, _ptr(w), w.shape[1], _ptr(out)))
        return out

    def decode_chunk(self, snp0: int, ncols: int, norm: SnpNorm) -> np.ndarray:
        out = np.empty((self.n_samples, ncols))
        self.eng.check(self.eng.lib.slfmm_decode_chunk(self.eng.h, self.h, snp0, ncols, int(norm), _ptr(out)))
        return out


# ---------------------------------------------------------------------------
# PLINK triplet (src/bed.rs)
# ---------------------------------------------------------------------------
@dataclass
class BimRecord:
    chrom: str
    snp_id: str
    cm: float
    pos: int
    allele1: str
    allele2: str


@dataclass
class FamRecord:
    fid: str
    iid: str
    father: str
    mother: str
    sex: int
    pheno: str


def _parse_fam(path: Path) -> List[FamRecord]:
    out = []
    with open(path) as f:
        for i, line in enumerate(f):
            fs = line.split()
            if len(fs) < 6:
                raise SchnelGpuError(ERR_BAD_BED, f"FAM line {i + 1} has {len(fs)} fields, expected 6")
            try:
                sex = int(fs[4])
            except ValueError:
                raise SchnelGpuError(ERR_BAD_BED, f"FAM line {i + 1}: invalid sex '{fs[4]}'")
            out.append(FamRecord(fs[0], fs[1], fs[2], fs[3], sex, fs[5]))
    return out


def _parse_bim(path: Path) -> List[BimRecord]:
    out = []
    with open(path) as f:
        for i, line in enumerate(f):
            fs = line.split()
            if len(fs) < 6:
                raise SchnelGpuError(ERR_BAD_BED, f"BIM line {i + 1} has {len(fs)} fields, expected 6")
            try:
                cm = float(fs[2])
            except ValueError:
                raise SchnelGpuError(ERR_BAD_BED, f"BIM line {i + 1}: invalid cM '{fs[2]}'")
            try:
                pos = int(fs[3])
            except ValueError:
                raise SchnelGpuError(ERR_BAD_BED, f"BIM line {i + 1}: invalid position '{fs[3]}'")
            out.append(BimRecord(fs[0], fs[1], cm, pos, fs[4], fs[5]))
    return out


class BedFile:
    """PLINK .bed/.bim/.fam triplet (src/bed.rs:60-171)."""

    def __init__(self, bed_path: Path, fam: List[FamRecord], bim: List[BimRecord], payload: np.ndarray):
        self.bed_path = bed_path
        self.fam_records = fam
        self.bim_records = bim
        self.n_physical_samples = len(fam)
        self.n_samples = len(fam)
        self.n_snps = len(bim)
        self.payload = payload          # bytes after the magic, SNP-major
        self.sample_keep: Optional[np.ndarray] = None

    @staticmethod
    def open(bed_path: os.PathLike) -> "BedFile":
        bed_path = Path(bed_path)
        stem = bed_path.with_suffix("")
        fam_path, bim_path = stem.with_suffix(".fam"), stem.with_suffix(".bim")
        try:
            fam = _parse_fam(fam_path)
        except FileNotFoundError:
            raise SchnelGpuError(ERR_IO, f"Failed to parse {fam_path}")
        try:
            bim = _parse_bim(bim_path)
        except FileNotFoundError:
            raise SchnelGpuError(ERR_IO, f"Failed to parse {bim_path}")
        lib = load_library()
        err = C.create_string_buffer(512)
        rc = lib.slfmm_bed_validate(str(bed_path).encode(), len(fam), len(bim), None, err, 512)
        if rc != OK:
            raise SchnelGpuError(rc, err.value.decode())
        payload = np.memmap(bed_path, dtype=np.uint8, mode="r", offset=3) if len(bim) else np.zeros(0, np.uint8)
        return BedFile(bed_path, fam, bim, payload)

    def bytes_per_snp(self) -> int:
        return (self.n_physical_samples + 3) // 4

    def subset_samples(self, indices: Sequence[int]) -> None:
        """src/bed.rs:155-159."""
        idx = np.asarray(indices, dtype=np.uint64)
        self.fam_records = [self.fam_records[int(i)] for i in idx]
        self.n_samples = len(idx)
        self.sample_keep = idx

    def subset_snp_count(self, subset: SubsetSpec) -> int:
        return subset.count(self.n_snps)

    def upload(self, eng: Engine, snps: Optional[SubsetSpec] = None) -> Genotypes:
        return eng.upload(np.asarray(self.payload), self.n_physical_samples, self.sample_keep, snps)


def align_est_bed_samples(est_bed: BedFile, main_bed: BedFile) -> None:
    """--est-bed alignment (align_est_bed_samples, src/main.rs:282-331): the
    estimation .bed takes the main .bed's samples in the main .bed's order
    (matched by IID; a repeated IID in the estimation .fam resolves to its
    last row), via subset_samples when the order or the count differs; an
    estimation .bed without some main-.bed sample is an error."""
    index = {r.iid: i for i, r in enumerate(est_bed.fam_records)}
    idx, missing = [], []
    for r in main_bed.fam_records:
        if r.iid in index:
            idx.append(index[r.iid])
        else:
            missing.append(r.iid)
    if missing:
        raise SchnelGpuError(ERR_BAD_ARG, f"est-bed is missing {len(missing)} sample(s) that are in the main BED "
                                          f"file: [{', '.join(missing[:5])}]{', ...' if len(missing) > 5 else ''}")
    if len(idx) != est_bed.n_samples or any(i != j for i, j in enumerate(idx)):
        sys.stderr.write(f"  Reordering/subsetting est-bed samples to match main BED ({est_bed.n_samples} → "
                         f"{len(idx)} samples)\n")
        est_bed.subset_samples(idx)


_MISSING_COV = (".",)


def _cov_value(text: str, name: str, line: int, sample: str) -> float:
    """One covariate cell: empty, '.' and NA (any case) are missing; anything
    else must parse as a finite number (src/main.rs:413-440)."""
    t = text.strip()
    if not t or t in _MISSING_COV or t.lower() == "na":
        return math.nan
    try:
        if "_" in t:               # digit separators: not a number to the reference's parser
            raise ValueError
        v = float(t)
    except ValueError:
        raise SchnelGpuError(ERR_BAD_ARG, f"Failed to parse value '{t}' for covariate '{name}' on line {line} "
                                          f"(sample '{sample}')")
    if math.isinf(v):
        # the parsed value as Rust displays it ("inf" / "-inf"), not the input text
        shown = "inf" if v > 0 else "-inf"
        raise SchnelGpuError(ERR_BAD_ARG, f"Infinite value ({shown}) for covariate '{name}' on line {line} "
                                          f"(sample '{sample}'): Inf values will propagate through all matrix "
                                          f"operations")
    return v


def load_covariates(path: os.PathLike, fam: Sequence[FamRecord], intersect: bool = False,
                    verbose: bool = False) -> Tuple[List[str], np.ndarray, List[int]]:
    """Covariate / phenotype table matched to .fam order (load_covariates,
    src/main.rs:339-571).

    Comma-delimited for a ``.csv`` extension, tab-delimited otherwise.  The
    header's first cell names the sample-ID column (may be blank), the rest
    name the covariates; each row is a sample ID (matched against the .fam
    IIDs) and one value per covariate.  Blank lines are skipped; duplicate IDs,
    ragged rows, unparsable or infinite values are errors.  Samples of the
    .fam absent from the table are an error unless ``intersect`` (then they
    are dropped).  Missing values are imputed per column with the mean of
    the observed ones (0 if none).  Returns (names, x kept x d, kept .fam
    row indices)."""
    path = Path(path)
    delim = "," if path.suffix == ".csv" else "\t"
    if verbose:
        sys.stderr.write(f"  Detected {'CSV' if delim == ',' else 'TSV'} format (delimiter: {delim!r})\n")
    try:
        with open(path, newline="") as f:
            lines = f.read().split("\n")
    except OSError:
        raise SchnelGpuError(ERR_IO, f"Failed to open covariate file: {path}")
    if lines and lines[-1] == "":
        lines.pop()                                   # the final newline ends the last line
    lines = [ln[:-1] if ln.endswith("\r") else ln for ln in lines]
    if not lines:
        raise SchnelGpuError(ERR_BAD_ARG, "Covariate file is empty")
    header = lines[0].split(delim)
    if len(header) < 2:
        raise SchnelGpuError(ERR_BAD_ARG, f"Covariate file header has only {len(header)} field(s) - expected at "
                                          f"least a sample ID column and one covariate column (delimiter: "
                                          f"{delim!r})")
    names = [h.strip() for h in header[1:]]
    d = len(names)
    data, order = {}, []
    for i, line in enumerate(lines[1:]):
        if not line.strip():
            continue
        fields = line.split(delim)
        if len(fields) != d + 1:
            raise SchnelGpuError(ERR_BAD_ARG, f"Line {i + 2} has {len(fields)} fields, expected {d + 1} "
                                              f"(1 sample ID + {d} covariates)")
        sid = fields[0].strip()
        vals = [_cov_value(s, names[j], i + 2, sid) for j, s in enumerate(fields[1:])]
        if sid in data:
            raise SchnelGpuError(ERR_BAD_ARG, f"Duplicate sample ID '{sid}' in covariate file (line {i + 2})")
        data[sid] = vals
        order.append(sid)
    if not data:
        raise SchnelGpuError(ERR_BAD_ARG, "Covariate file has no data rows")
    sys.stderr.write(f"  Read {len(data)} samples from covariate file\n")
    kept, rows = [], []
    for r, rec in enumerate(fam):
        vals = data.get(rec.iid)
        if vals is not None:
            kept.append(r)
            rows.append(vals)
        elif not intersect:
            raise SchnelGpuError(ERR_BAD_ARG, f"Sample '{rec.iid}' (FID='{rec.fid}') from .fam file not found in "
                                              f"covariate file.\n.fam has {len(fam)} samples, covariate file has "
                                              f"{len(data)}.\nFirst few covariate sample IDs: "
                                              f"[{', '.join(order[:5])}]\nHint: use --intersect-samples to use "
                                              f"only samples present in both files.")
    if not kept:
        raise SchnelGpuError(ERR_BAD_ARG, f"No samples in common between .fam file ({len(fam)} samples) and "
                                          f"covariate file ({len(data)} samples).\nFirst few .fam IIDs: "
                                          f"[{', '.join(r.iid for r in fam[:5])}]\nFirst few covariate IDs: "
                                          f"[{', '.join(order[:5])}]")
    if len(data) > len(kept):
        sys.stderr.write(f"  Warning: {len(data) - len(kept)} sample(s) in covariate file not present in .fam "
                         f"file (ignored)\n")
    if len(fam) > len(kept):
        sys.stderr.write(f"  Warning: {len(fam) - len(kept)} sample(s) in .fam file not present in covariate "
                         f"file (dropped with --intersect-samples)\n")
    sys.stderr.write(f"  Matched {len(kept)} samples to .fam order\n")
    x = np.array(rows, dtype=np.float64).reshape(len(kept), d)
    for j in range(d):
        col = x[:, j]
        miss = np.isnan(col)
        if not miss.any():
            continue
        total, n_obs = 0.0, 0
        for v in col[~miss]:                      # in row order, like the reference's running sum
            total += float(v)
            n_obs += 1
        mean = total / n_obs if n_obs else 0.0
        col[miss] = mean
        sys.stderr.write(f"  Warning: covariate '{names[j]}' has {int(miss.sum())} missing value(s) ('.', 'NA', "
                         f"or empty), imputed to column mean ({mean:.6f})\n")
    return names, x, kept


# ---------------------------------------------------------------------------
# library API (src/lib.rs)
# ---------------------------------------------------------------------------
_default_engine: Optional[Engine] = None


def default_engine() -> Engine:
    global _default_engine
    if _default_engine is None:
        _default_engine = Engine()
    return _default_engine


def center_covariates(x: np.ndarray, scale: bool, engine: Optional[Engine] = None) -> np.ndarray:
    return (engine or default_engine()).center_covariates(x, scale)


def _as_geno(y, eng: Engine, subset: Optional[SubsetSpec] = None) -> Genotypes:
    if isinstance(y, Genotypes):
        if subset is not None and subset.kind != "all":
            raise SchnelGpuError(ERR_BAD_ARG, "apply SNP subsets at upload time for resident genotypes")
        return y
    return y.upload(eng, subset)


def estimate_factors(y_est, subset: SubsetSpec, x: np.ndarray, config: Lfmm2Config,
                     omega: Optional[np.ndarray] = None, engine: Optional[Engine] = None) -> np.ndarray:
    eng = engine or default_engine()
    g = _as_geno(y_est, eng, subset)
    x = np.ascontiguousarray(x, dtype=np.float64)
    u = np.empty((g.n_samples, config.k))
    om = None if omega is None else np.ascontiguousarray(omega, dtype=np.float64)
    _check_shape("x", x, g.n_samples)
    _check_shape("omega", om, g.n_samples, config.k + config.oversampling)
    cfg = config._c()
    eng.check(eng.lib.slfmm_estimate_factors(eng.h, g.h, _ptr(x), x.shape[1], C.byref(cfg), _ptr(om), _ptr(u)))
    return u


def _alloc_results(n: int, p: int, d: int, k: int, nmf_iter: int):
    arr = dict(u_hat=np.empty((n, k)), beta=np.empty((p, d)), tstat=np.empty((p, d)), pvalue=np.empty((p, d)),
               r2=np.empty((p, 3)), gif_per_trait=np.empty(d), nmf_cv=np.empty(max(nmf_iter, 1)))
    r = _Results(_dptr(arr["u_hat"]), _dptr(arr["beta"]), _dptr(arr["tstat"]), _dptr(arr["pvalue"]),
                 _dptr(arr["r2"]), _dptr(arr["gif_per_trait"]), 0.0, _dptr(arr["nmf_cv"]), 0.0, 0.0, 0.0, 0)
    return r, arr


def _to_results(r: _Results, arr, config: Lfmm2Config) -> TestResults:
    out = TestResults(arr["u_hat"], r.gif, arr["gif_per_trait"], arr["beta"], arr["tstat"], arr["pvalue"], arr["r2"])
    if config.impute == ImputeStrategy.NMF:
        nmf = config.nmf or NmfConfig(k=config.k)
        cv = arr.get("nmf_cv")
        out.nmf_cv = [] if cv is None else list(cv[:nmf.n_iter])
        out.nmf_cv_mean = r.nmf_cv_mean
        out.nmf_gwas_cv_mae = r.nmf_gwas_cv_mae
        out.nmf_gwas_cv_mean_mae = r.nmf_gwas_cv_mean_mae
        out.nmf_gwas_cv_count = int(r.nmf_gwas_cv_count)
    return out


def test_associations(y_full, x: np.ndarray, u_hat: np.ndarray, config: Lfmm2Config,
                      engine: Optional[Engine] = None) -> TestResults:
    eng = engine or default_engine()
    g = _as_geno(y_full, eng)
    x = np.ascontiguousarray(x, dtype=np.float64)
    u_hat = np.ascontiguousarray(u_hat, dtype=np.float64)
    _check_shape("x", x, g.n_samples)
    _check_shape("u_hat", u_hat, g.n_samples, config.k)
    r, arr = _alloc_results(g.n_samples, g.n_snps, x.shape[1], config.k, 0)
    cfg = config._c()
    eng.check(eng.lib.slfmm_test_associations(eng.h, g.h, _ptr(x), x.shape[1], _ptr(u_hat), C.byref(cfg),
                                              C.byref(r)))
    return _to_results(r, arr, config)


test_associations.__test__ = False  # keep pytest from collecting the API function


class OutputFormat(enum.Enum):
    """src/testing.rs:35-48."""
    TSV = "tsv"
    PARQUET = "parquet"


@dataclass
class OutputConfig:
    """src/testing.rs:68-73."""
    path: Path
    bim: Sequence[BimRecord]
    cov_names: Sequence[str]
    format: OutputFormat = OutputFormat.TSV


class _CStrings:
    """Strings as one NUL-separated UTF-8 buffer and a char* per string (the
    buffer lives as long as this object)."""

    def __init__(self, strs: Sequence[str]):
        strs = list(strs)
        self.blob = np.frombuffer(("\0".join(strs) + "\0").encode(), dtype=np.uint8)
        ends = np.flatnonzero(self.blob == 0)
        if strs and ends.size != len(strs):
            raise SchnelGpuError(ERR_BAD_ARG, "a name contains a NUL character")
        self.ptrs = np.zeros(max(len(strs), 1), dtype=np.uint64)
        if strs:
            self.ptrs[1:] = ends[:-1] + 1
            self.ptrs += np.uint64(self.blob.ctypes.data)

    def arg(self):
        return self.ptrs.ctypes.data_as(C.POINTER(C.c_char_p))


def _output_args(bim: Sequence[BimRecord], cov_names: Sequence[str], res: TestResults):
    """The writers' arguments: per-SNP names, positions, covariate names and
    the result columns as contiguous FP64, checked against each other."""
    p, d = res.beta.shape
    if len(bim) != p or len(cov_names) != d:
        raise SchnelGpuError(ERR_BAD_ARG, "bim must have one record per SNP and cov_names one name per trait")
    cols = {k: np.ascontiguousarray(getattr(res, k), dtype=np.float64) for k in ("beta", "tstat", "pvalue", "r2")}
    for k, shape in (("beta", (p, d)), ("tstat", (p, d)), ("pvalue", (p, d)), ("r2", (p, 3))):
        if cols[k].shape != shape:
            raise SchnelGpuError(ERR_BAD_ARG, f"{k} has shape {cols[k].shape}, expected {shape}")
    chrom = _CStrings(b.chrom for b in bim)
    sid = _CStrings(b.snp_id for b in bim)
    names = _CStrings(cov_names)
    pos = np.ascontiguousarray([b.pos for b in bim] or [0], dtype=np.uint64)
    r = _Results(None, _dptr(cols["beta"]), _dptr(cols["tstat"]), _dptr(cols["pvalue"]), _dptr(cols["r2"]), None,
                 res.gif, None, 0.0, 0.0, 0.0, 0)
    keep = (cols, chrom, sid, names, pos)
    return p, d, chrom.arg(), pos.ctypes.data_as(C.POINTER(C.c_uint64)), sid.arg(), names.arg(), r, keep


def write_tsv(path: os.PathLike, bim: Sequence[BimRecord], cov_names: Sequence[str], res: TestResults,
              n_threads: int = 0) -> None:
    """<out>.tsv as coalesce_output_tsv (src/testing.rs:740-801)."""
    lib = load_library()
    p, d, chrom, pos, sid, names, r, keep = _output_args(bim, cov_names, res)
    rc = lib.slfmm_write_tsv(str(path).encode(), p, d, chrom, pos, sid, names, C.byref(r), n_threads)
    del keep
    if rc != OK:
        raise SchnelGpuError(rc, f"Failed to create {path}")


PARQUET_UNCOMPRESSED = 0
PARQUET_ZSTD = 6


def write_parquet(path: os.PathLike, bim: Sequence[BimRecord], cov_names: Sequence[str], res: TestResults,
                  compression: int = PARQUET_ZSTD, n_threads: int = 0) -> None:
    """<out>.parquet as coalesce_output_parquet (src/testing.rs:818-983):
    chr, pos, snp_id, p_*, beta_*, t_*, r2_cov, r2_latent, r2_resid; rows in
    SNP order; ZSTD (the reference's codec) or uncompressed."""
    lib = load_library()
    p, d, chrom, pos, sid, names, r, keep = _output_args(bim, cov_names, res)
    rc = lib.slfmm_write_parquet(str(path).encode(), p, d, chrom, pos, sid, names, C.byref(r), compression, n_threads)
    del keep
    if rc != OK:
        raise SchnelGpuError(rc, f"Failed to create {path}")


def fit_lfmm2(y_est, est_subset: SubsetSpec, y_full, x: np.ndarray, config: Lfmm2Config,
              output: Optional[OutputConfig] = None, omega: Optional[np.ndarray] = None,
              engine: Optional[Engine] = None) -> TestResults:
    """fit_lfmm2 (src/lib.rs:162-263): estimate U_hat on y_est (subset), test
    every SNP of y_full, calibrate, optionally write <out>.tsv."""
    eng = engine or default_engine()
    gf = _as_geno(y_full, eng)
    if y_est is y_full and (est_subset is None or est_subset.kind == "all"):
        ge = gf
    else:
        ge = _as_geno(y_est, eng, est_subset)
    x = np.ascontiguousarray(x, dtype=np.float64)
    om = None if omega is None else np.ascontiguousarray(omega, dtype=np.float64)
    _check_shape("x", x, gf.n_samples)
    _check_shape("omega", om, gf.n_samples, config.k + config.oversampling)
    nmf_iter = (config.nmf.n_iter if config.nmf else 0) if config.impute == ImputeStrategy.NMF else 0
    r, arr = _alloc_results(gf.n_samples, gf.n_snps, x.shape[1], config.k, nmf_iter)
    cfg = config._c()
    eng.check(eng.lib.slfmm_fit(eng.h, ge.h, gf.h, _ptr(x), x.shape[1], C.byref(cfg), _ptr(om), C.byref(r)))
    res = _to_results(r, arr, config)
    if output is not None:
        (write_parquet if output.format == OutputFormat.PARQUET else write_tsv)(output.path, output.bim,
                                                                                 output.cov_names, res)
    return res


def fit_lfmm2_traits(y_full: "Genotypes", y: np.ndarray, masks: np.ndarray, config: Lfmm2Config,
                     engine: Optional[Engine] = None) -> List[TestResults]:
    """One d = 1 model per trait (column of y, n x T) on the samples where
    masks[:, t] is nonzero -- the reference run once per trait with that
    trait's samples and --intersect-samples.  Genotypes stay resident."""
    eng = engine or default_engine()
    y = np.ascontiguousarray(y, dtype=np.float64)
    masks = np.ascontiguousarray(masks, dtype=np.uint8)
    n, t_count = y.shape
    if masks.shape != y.shape or n != y_full.n_samples:
        raise SchnelGpuError(ERR_BAD_ARG, "y and masks must be n_samples x n_traits")
    p = y_full.n_snps
    nmf_iter = config.nmf.n_iter if (config.impute == ImputeStrategy.NMF and config.nmf) else 0
    rs = (_Results * t_count)()
    arrs = []
    for t in range(t_count):
        r, arr = _alloc_results(int(np.count_nonzero(masks[:, t])), p, 1, config.k, nmf_iter)
        rs[t] = r
        arrs.append(arr)
    cfg = config._c()
    eng.check(eng.lib.slfmm_fit_traits(eng.h, y_full.h, _ptr(y), _ptr(masks), t_count, C.byref(cfg), rs))
    return [_to_results(rs[t], arrs[t], config) for t in range(t_count)]


def fit_lfmm2_many(problems: Sequence[Tuple[np.ndarray, int, np.ndarray, Lfmm2Config]],
                   engine: Optional[Engine] = None, n_streams: int = 0,
                   outs: Optional[Sequence[dict]] = None) -> List[TestResults]:
    """Independent problems (packed payload, n_physical, x, config), run
    concurrently on n_streams streams of the engine's device (0: 8).
    ``outs`` may hold preallocated (e.g. pinned) result arrays per problem."""
    eng = engine or default_engine()
    keep = []
    probs = (_Problem * len(problems))()
    rs = (_Results * len(problems))()
    arrs = []
    for i, (packed, n_physical, x, config) in enumerate(problems):
        x = np.ascontiguousarray(x, dtype=np.float64)
        packed, n_snps = _payload(packed, n_physical)
        _check_shape(f"problem {i}: x", x, n_physical)
        if outs is None:
            nmf_iter = config.nmf.n_iter if (config.impute == ImputeStrategy.NMF and config.nmf) else 0
            r, arr = _alloc_results(n_physical, n_snps, x.shape[1], config.k, nmf_iter)
        else:
            arr = outs[i]
            r = _Results(_dptr(arr["u_hat"]), _dptr(arr["beta"]), _dptr(arr["tstat"]), _dptr(arr["pvalue"]),
                         _dptr(arr["r2"]), _dptr(arr["gif_per_trait"]), 0.0, _dptr(arr.get("nmf_cv")), 0.0, 0.0,
                         0.0, 0)
        rs[i] = r
        arrs.append(arr)
        cfg = config._c()
        keep += [x, cfg, packed]
        probs[i] = _Problem(packed.ctypes.data, n_physical, n_snps, x.ctypes.data, x.shape[1],
                            C.addressof(cfg), None, C.addressof(rs[i]))
    status = (C.c_int * max(len(problems), 1))()
    eng.check(eng.lib.slfmm_fit_many(eng.h, probs, len(problems), n_streams, status))
    return [_to_results(rs[i], arrs[i], problems[i][3]) for i in range(len(problems))]


def fit_lfmm2_host(packed: np.ndarray, n_physical: int, x: np.ndarray, config: Lfmm2Config,
                   est_subset: Optional[SubsetSpec] = None, sample_keep: Optional[Sequence[int]] = None,
                   omega: Optional[np.ndarray] = None, engine: Optional[Engine] = None,
                   out: Optional[dict] = None) -> TestResults:
    """fit_lfmm2 from a HOST payload (upload, fit, copy back) in one C-ABI call.
    ``out`` may hold preallocated (e.g. pinned) result arrays."""
    eng = engine or default_engine()
    packed, n_snps = _payload(packed, n_physical)
    n = n_physical if sample_keep is None else len(sample_keep)
    x = np.ascontiguousarray(x, dtype=np.float64)
    _check_shape("x", x, n)
    if omega is not None:
        _check_shape("omega", np.asarray(omega), n, config.k + config.oversampling)
    d = x.shape[1]
    if out is None:
        r, arr = _alloc_results(n, n_snps, d, config.k, config.nmf.n_iter if config.nmf else 0)
    else:
        arr = out
        r = _Results(_dptr(arr["u_hat"]), _dptr(arr["beta"]), _dptr(arr["tstat"]), _dptr(arr["pvalue"]),
                     _dptr(arr["r2"]), _dptr(arr["gif_per_trait"]), 0.0, _dptr(arr.get("nmf_cv")), 0.0, 0.0, 0.0, 0)
    keep = None if sample_keep is None else np.ascontiguousarray(sample_keep, dtype=np.uint64)
    sub = (est_subset or SubsetSpec.all())._c()
    om = None if omega is None else np.ascontiguousarray(omega, dtype=np.float64)
    cfg = config._c()
    eng.check(eng.lib.slfmm_fit_host(eng.h, _ptr(packed), n_physical, n_snps,
                                     None if keep is None else keep.ctypes.data_as(C.POINTER(C.c_uint64)),
                                     0 if keep is None else len(keep), C.byref(sub), _ptr(x), d, C.byref(cfg),
                                     _ptr(om), C.byref(r)))
    return _to_results(r, arr, config)


def format_exp6(v: float) -> str:
    """Rust ``{:.6e}`` as produced by the C ABI."""
    lib = load_library()
    buf = C.create_string_buffer(64)
    n = lib.slfmm_format_exp6(float(v), buf, 64)
    return buf.value[:n].decode()
