/*
 * schnelgpu.h -- C ABI of the GB300 (sm_103a) streaming LFMM2 engine.
 *
 * Drop-in boundary for the hot path of schnelLFMM v0.3.2.  Every entry point
 * takes plain pointers and sizes, returns an int status (0 = OK, negative =
 * error) and leaves a human-readable message in slfmm_last_error().  There is
 * no CPU fallback: when no sm_103a device is present the calls fail with
 * SLFMM_ERR_CUDA.
 *
 * Layout conventions (all host arrays):
 *   - packed genotypes: the .bed payload AFTER the 3-byte magic, SNP-major,
 *     ceil(n_physical/4) bytes per SNP (src/bed.rs:137-145);
 *   - dense matrices are row-major: X is n x d, U_hat is n x K, per-SNP
 *     outputs are p x d (SNP-major rows);
 *   - index arrays are uint64_t.
 *
 * Threading: a context is bound to one device and one CUDA stream and is not
 * thread-safe; use one context per host thread.  Calls are blocking (results
 * are in host memory when the call returns) unless documented otherwise.
 */
#ifndef SCHNELGPU_H
#define SCHNELGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define SLFMM_OK                  0
#define SLFMM_ERR_BAD_ARG        -1   /* invalid argument / shape            */
#define SLFMM_ERR_BAD_BED        -2   /* magic or size mismatch, parse error */
#define SLFMM_ERR_SINGULAR       -3   /* inversion failed even regularised   */
#define SLFMM_ERR_DF_NONPOSITIVE -4   /* n <= 1 + d + K                      */
#define SLFMM_ERR_CUDA           -5   /* CUDA runtime / launch failure       */
#define SLFMM_ERR_DEVICE_TIMEOUT -6   /* a bounded device wait expired       */
#define SLFMM_ERR_IO             -7   /* file open/read/write failure        */
#define SLFMM_ERR_NOMEM          -8   /* device or host allocation failed    */

/* ---- enums ------------------------------------------------------------- */
#define SLFMM_NORM_CENTER_ONLY 0      /* SnpNorm::CenterOnly (src/bed.rs:19-26) */
#define SLFMM_NORM_EIGENSTRAT  1      /* SnpNorm::Eigenstrat                     */

#define SLFMM_PREC_FP32        0      /* plain FP32 SIMT contractions            */
#define SLFMM_PREC_SPLIT_BF16  1      /* tcgen05 tensor cores, exact BF16
                                         genotypes x hi+lo BF16 operand          */
#define SLFMM_PREC_SPLIT_FP8   2      /* tcgen05 kind::f8f6f4, exact E4M3
                                         genotypes x 4 scaled E4M3 terms, exact
                                         missing-call operand (default)          */

#define SLFMM_IMPUTE_MEAN      0      /* ImputeStrategy::Mean (src/lib.rs:39-44) */
#define SLFMM_IMPUTE_NMF       1      /* ImputeStrategy::Nmf                     */

/* Stream the Gaussian sketches (Omega of src/rsvd.rs:44-46, the NMF probe of
 * src/nmf.rs:291-293) and the NMF CV hold-out masks (src/nmf.rs:433-448,
 * src/testing.rs:437-452) are drawn from. */
#define SLFMM_RNG_CHACHA8      0      /* the reference's streams (default):
                                         ChaCha8Rng::seed_from_u64(seed) sampled
                                         by Normal(0, 1) in row-major order for
                                         the sketches (on the host threads) and by
                                         Uniform(0, 1) for the masks (on the
                                         device)                                 */
#define SLFMM_RNG_COUNTER      1      /* SplitMix64 counter streams, drawn on the
                                         device                                  */

#define SLFMM_SUBSET_ALL       0      /* SubsetSpec::All     (src/bed.rs:50-57)  */
#define SLFMM_SUBSET_RATE      1      /* SubsetSpec::Rate(r)                     */
#define SLFMM_SUBSET_INDICES   2      /* SubsetSpec::Indices(v)                  */

typedef struct slfmm_ctx  slfmm_ctx;   /* one per device+stream              */
typedef struct slfmm_geno slfmm_geno;  /* device-resident packed genotypes   */

typedef struct {
    int   precision;   /* SLFMM_PREC_*                                     */
    int   verbose;     /* progress/diagnostics on stderr                   */
    void* stream;      /* optional cudaStream_t to run on (NULL = own)     */
    int   autotune;    /* time the tensor-core ring depths once per shape
                          and keep the fastest (results are unchanged);
                          also switched on by SLFMM_AUTOTUNE=1             */
    int   rng;         /* SLFMM_RNG_* stream of the sketch matrices        */
} slfmm_opts;

typedef struct {
    int             kind;      /* SLFMM_SUBSET_*                      */
    double          rate;      /* for RATE: step = ceil(1/rate)       */
    const uint64_t* indices;   /* for INDICES                         */
    uint64_t        n_indices;
} slfmm_subset;

/* Mirrors Lfmm2Config (src/lib.rs:47-98) and NmfConfig (src/nmf.rs:15-50). */
typedef struct {
    uint32_t k;             /* latent factors K                           */
    double   lambda;        /* ridge penalty, must be > 0                 */
    uint32_t chunk_size;    /* SNPs per streaming chunk (CV streams)      */
    uint32_t oversampling;  /* RSVD oversampling (l = K + oversampling)   */
    uint32_t n_power_iter;  /* RSVD power iterations q                    */
    uint64_t seed;          /* RNG seed                                   */
    int      norm;          /* SLFMM_NORM_*                               */
    int      scale_cov;     /* divide covariates by sd after centring     */
    int      impute;        /* SLFMM_IMPUTE_*                             */
    uint32_t nmf_k;         /* NMF rank (0 = K)                           */
    uint32_t nmf_iter;      /* multiplicative-update iterations           */
    double   nmf_eps;       /* denominator/clamp epsilon (1e-16)          */
    double   nmf_cv_rate;   /* CV hold-out rate                           */
} slfmm_config;

/* Mirrors TestResults (src/testing.rs:76-93) plus the per-SNP columns the
 * reference writes to <out>.tsv.  All arrays are CALLER-allocated; a NULL
 * pointer skips that output. */
typedef struct {
    double*  u_hat;          /* n x K                                       */
    double*  beta;           /* p x d  ridge effect sizes                   */
    double*  tstat;          /* p x d                                       */
    double*  pvalue;         /* p x d  GIF-calibrated                       */
    double*  r2;             /* p x 3  r2_cov, r2_latent, r2_resid          */
    double*  gif_per_trait;  /* d      clamped >= 1, used for calibration   */
    double   gif;            /* mean of the unclamped per-trait GIFs        */
    double*  nmf_cv;         /* nmf_iter per-iteration CV MAE (NMF only)    */
    double   nmf_cv_mean;    /* mean-imputation CV MAE on the last mask     */
    double   nmf_gwas_cv_mae;
    double   nmf_gwas_cv_mean_mae;
    uint64_t nmf_gwas_cv_count;
} slfmm_results;

/* ---- context ------------------------------------------------------------ */
/* Replaces the thread pool set-up of parallel_stream (src/parallel.rs:156-199)
 * and openblas_set_num_threads (src/lib.rs:23-35). */
int         slfmm_create(int device, const slfmm_opts* opts, slfmm_ctx** out);
void        slfmm_destroy(slfmm_ctx* ctx);
const char* slfmm_last_error(const slfmm_ctx* ctx);
/* Number of kernels this context launched since creation. */
uint64_t    slfmm_launch_count(const slfmm_ctx* ctx);
/* Opaque cudaStream_t the context runs on. */
void*       slfmm_stream(const slfmm_ctx* ctx);

/* ---- .bed ingest --------------------------------------------------------- */
/* BedFile::open validation (src/bed.rs:78-135): magic 6C 1B 01 and size
 * 3 + ceil(n/4)*p.  Reads the payload into a caller buffer of
 * ceil(n/4)*p bytes (pass NULL to only validate). */
int slfmm_bed_validate(const char* bed_path, uint64_t n_samples, uint64_t n_snps,
                       uint8_t* payload_out, char* err, size_t err_len);

/* Upload a packed payload to the device (pinned ring, double-buffered H2D),
 * applying the sample subset (BedFile::subset_samples, src/bed.rs:155-159)
 * and the SNP subset (subset_indices, src/parallel.rs:113-122; copy_raw_chunk
 * :129-146).  Builds the per-SNP allele counts and missing-call lists once;
 * every later pass reads the resident copy. */
int slfmm_geno_upload(slfmm_ctx* ctx, const uint8_t* packed, uint64_t n_physical,
                      uint64_t n_snps, const uint64_t* sample_keep, uint64_t n_keep,
                      const slfmm_subset* snps, slfmm_geno** out);
int slfmm_geno_free(slfmm_ctx* ctx, slfmm_geno* g);
uint64_t slfmm_geno_n_samples(const slfmm_geno* g);
uint64_t slfmm_geno_n_snps(const slfmm_geno* g);

/* ---- parity hooks for stage (a) ----------------------------------------- */
/* Per-SNP allele counts c0,c1,c2,cmiss (int32, p x 4), mean over observed
 * calls, scale (src/bed.rs:382-395) and TSS of the standardised column.
 * counts/mean/scale are bit-exact with decode_single_snp
 * (src/bed.rs:300-379).  Any output may be NULL. */
int slfmm_decode_stats(slfmm_ctx* ctx, const slfmm_geno* g, int norm,
                       int32_t* counts4, double* mean, double* scale, double* tss);
/* Standardised decode of SNPs [snp0, snp0+ncols) into out (n x ncols,
 * row-major), mean imputation: decode_bed_chunk_into (src/bed.rs:211-235). */
int slfmm_decode_chunk(slfmm_ctx* ctx, const slfmm_geno* g, uint64_t snp0,
                       uint64_t ncols, int norm, double* out);

/* Raw tensor-core contraction of the exact genotypes (missing calls = 0)
 * with the split operand of the context's precision.  flags bit 0: 0 gives
 * out (p x w) = G~^T W for W n x w, 1 gives out (n x w) = G~ W for W p x w
 * (transposed copy); bit 1 (split-FP8 only): add the missing-call indicator
 * product, i.e. missing calls count as 1.  Parity hook for the per-chunk
 * dgemms of src/rsvd.rs:61-153. */
int slfmm_contract_raw(slfmm_ctx* ctx, const slfmm_geno* g, int flags, const double* w,
                       uint32_t w_cols, float* out);

/* ---- library API (src/lib.rs) ------------------------------------------- */
/* center_covariates (src/lib.rs:102-117). x, out: n x d row-major. */
int slfmm_center_covariates(slfmm_ctx* ctx, const double* x, uint64_t n, uint32_t d,
                            int scale, double* out);
/* Parity hook for the small symmetric eigen-solves (the X^T X of Step 0,
 * src/precompute.rs:47, and the l x l Gram of the randomized SVD's final
 * small SVD, src/rsvd.rs:162, both LAPACK in the reference): a (a x a,
 * row-major, symmetric positive semi-definite, a <= 256) -> eigenvectors
 * v_out (a x a, column j = vector j) and eigenvalues sig_out, descending. */
int slfmm_small_eigh(slfmm_ctx* ctx, const double* a, uint32_t dim, double* v_out, double* sig_out);
/* Random sketch Omega (n x l) the engine uses for a given seed. */
int slfmm_generate_omega(slfmm_ctx* ctx, uint64_t seed, uint64_t n, uint32_t l,
                         double* out);
/* Host-only (no context, no device): the rows x cols row-major matrix of
 * Normal(0, 1) draws from ChaCha8Rng::seed_from_u64(seed), i.e.
 * Array2::from_shape_fn((rows, cols), |_| normal.sample(&mut rng)) of
 * src/rsvd.rs:44-46 (seed = config.seed) and src/nmf.rs:291-293
 * (seed = config.seed + 1 000 000).  The SLFMM_RNG_CHACHA8 stream. */
int slfmm_reference_normal(uint64_t seed, uint64_t rows, uint32_t cols, double* out);
/* estimate_factors (src/lib.rs:127-136): Step 0 + RSVD of M Y_est.
 * omega: n x (K+oversampling) or NULL (engine RNG).  u_hat: n x K. */
int slfmm_estimate_factors(slfmm_ctx* ctx, const slfmm_geno* y_est, const double* x,
                           uint32_t d, const slfmm_config* cfg, const double* omega,
                           double* u_hat);
/* test_associations (src/lib.rs:144-154) with a given U_hat (n x K). */
int slfmm_test_associations(slfmm_ctx* ctx, const slfmm_geno* y_full, const double* x,
                            uint32_t d, const double* u_hat, const slfmm_config* cfg,
                            slfmm_results* res);
/* fit_lfmm2 (src/lib.rs:162-263) on resident genotypes. */
int slfmm_fit(slfmm_ctx* ctx, const slfmm_geno* y_est, const slfmm_geno* y_full,
              const double* x, uint32_t d, const slfmm_config* cfg, const double* omega,
              slfmm_results* res);
/* fit_lfmm2 from HOST buffers: uploads (H2D inside), fits, copies results
 * back, frees the device copy.  est == NULL or kind ALL uses y_full. */
int slfmm_fit_host(slfmm_ctx* ctx, const uint8_t* packed, uint64_t n_physical,
                   uint64_t n_snps, const uint64_t* sample_keep, uint64_t n_keep,
                   const slfmm_subset* est, const double* x, uint32_t d,
                   const slfmm_config* cfg, const double* omega, slfmm_results* res);

/* ---- batched fits --------------------------------------------------------- */
/* Per-trait models on their own sample sets.  Trait t (of n_traits) uses the
 * samples i of the resident matrix g with masks[i * n_traits + t] != 0, in
 * sample order, and is a d = 1 model with x = y[i * n_traits + t] (y is
 * n x n_traits row-major; values at masked samples are ignored).  This is the
 * reference's one run per trait with its covariate file holding the trait's
 * samples and --intersect-samples (src/main.rs:128-138: load_covariates keeps
 * the matched samples, BedFile::subset_samples (src/bed.rs:155-159)
 * restricts the genotypes).
 * res[t] receives trait t's results with u_hat n_t x K (n_t = its sample
 * count), beta / tstat / pvalue p x 1, r2 p x 3, gif_per_trait 1.  Each
 * trait's sample subset is extracted on the device from the resident matrix;
 * nothing is uploaded again. */
int slfmm_fit_traits(slfmm_ctx* ctx, const slfmm_geno* g, const double* y, const uint8_t* masks,
                     uint32_t n_traits, const slfmm_config* cfg, slfmm_results* res);

/* One independent problem of slfmm_fit_many: the arguments of slfmm_fit_host
 * with every SNP in the estimation. */
typedef struct slfmm_problem {
    const uint8_t* packed; /* p x ceil(n_physical / 4) PLINK payload (host) */
    uint64_t n_physical;
    uint64_t n_snps;
    const double* x;       /* n_physical x d row-major */
    uint32_t d;
    const slfmm_config* cfg;
    const double* omega;   /* n x (K + oversampling) or NULL */
    slfmm_results* res;
} slfmm_problem;

/* Many independent problems of uneven n, p, K and d (the reference runs them
 * one CLI invocation at a time): they run concurrently on n_streams internal
 * streams of the context's device (0: 8), each problem's kernels in order on
 * one stream.  status[i] (may be NULL) receives problem i's status; returns
 * the first nonzero status, or SLFMM_OK. */
int slfmm_fit_many(slfmm_ctx* ctx, const slfmm_problem* problems, uint32_t n_problems,
                   uint32_t n_streams, int* status);

/* ---- synthetic cohorts (plays the role of src/simulate.rs:49-142) ------- */
/* Draw a structured cohort directly into a device-resident matrix: n
 * samples with admixture proportions admix (n x n_pop, host, rows sum to 1),
 * p SNPs with ancestral frequency U(f_lo, f_hi), population drift Fst,
 * inbreeding (probability a genotype is homozygous by descent) and MCAR
 * missing rate. */
int slfmm_simulate(slfmm_ctx* ctx, uint64_t n, uint64_t p, uint32_t n_pop, const float* admix,
                   double fst, double f_lo, double f_hi, double miss_rate, double inbreeding,
                   uint64_t seed, slfmm_geno** out);
/* Copy a resident matrix back as a PLINK payload (p x ceil(n/4) bytes). */
int slfmm_geno_download(slfmm_ctx* ctx, const slfmm_geno* g, uint8_t* packed_out);

/* Page-locked host buffers (cudaMallocHost) for payloads and results, so
 * that slfmm_fit_host copies by DMA without a staging memcpy. */
int slfmm_host_alloc(size_t bytes, void** out);
int slfmm_host_free(void* p);

/* ---- instrumentation ----------------------------------------------------- */
/* Record CUDA events around the streaming contraction kernels (resets the
 * counters).  slfmm_profile_read returns, for a kernel class
 * ("row_contract", "col_contract", "assoc_epilogue"), the summed device time,
 * the number of launches and the algorithmic bytes / flops they moved. */
int slfmm_profile_enable(slfmm_ctx* ctx, int on);
int slfmm_profile_read(slfmm_ctx* ctx, const char* kernel, double* total_ms, uint64_t* launches,
                       double* algo_bytes, double* algo_flops);
/* Phases of the last fit run while profiling is on (slfmm_fit_host: upload
 * with the sketch pass, randomized SVD, association design, row pass and
 * statistics, GIF, results to host).  Each phase has its device time
 * (events on the context's stream, recorded without synchronising) and
 * the host wall time between its marks.  slfmm_phase_count returns the
 * number of phases; slfmm_phase_read fills phase i (0-based). */
int slfmm_phase_count(const slfmm_ctx* ctx);
int slfmm_phase_read(slfmm_ctx* ctx, int i, char* name, size_t name_len, double* device_ms, double* host_ms);

/* ---- failure-detection test hook ---------------------------------------- */
/* The next split-FP8 contraction this context launches starts with a wait
 * on a barrier that nothing completes, bounded by `cycles` SM cycles
 * (1 .. 8e9), before it issues any copy or MMA: the wait expires, the kernel
 * frees its tensor memory and returns, and the call that launched it fails
 * with SLFMM_ERR_DEVICE_TIMEOUT.  Later calls run normally.  Exercises the
 * bounded-wait path of the device pipeline (no counterpart in the
 * reference, whose CPU workers cannot stall on a device). */
int slfmm_debug_expire_next_wait(slfmm_ctx* ctx, uint64_t cycles);

/* ---- allocation-free entry point ----------------------------------------- */
/* Raw genomic inflation factor of each trait from device-resident t
 * statistics, allocating no device memory.  No counterpart in the reference:
 * there the GIF is computed inside the test pass (src/testing.rs:179-224).
 *
 * t_dev: p x d FP32 t statistics on the context's device (row-major, as the
 * fit returns them); gif_dev: d doubles on that device receive median(t^2) /
 * 0.4549 per trait (1 when the median is below 1e-10) -- the fit clamps this
 * at 1 before calibrating p-values.  The work is queued on the context's
 * stream; the call does not wait for it.
 *
 * For callers that must not allocate device memory while they run: a host
 * application whose own allocator owns the device memory, or code that calls
 * in at a point where an allocation would block or fail.  The t^2 histogram
 * lives in one static device array of 8 x 100000 counters (3.2 MB) per
 * device, so at most 8 traits per call (more returns SLFMM_ERR_BAD_ARG).
 * Every call on a device shares that array and zeroes the rows it uses at its
 * start: calls that overlap in time on one device (other streams, other
 * threads) race on it and must be serialised by the caller.  slfmm_create
 * does the set-up on its device: it looks up the array's address
 * (cudaGetSymbolAddress) and loads the module of the two kernels (CUDA loads
 * modules lazily, and a load allocates device memory for the code and the
 * array).  So only context creation may load or allocate; a call does
 * neither. */
int slfmm_gif_noalloc(slfmm_ctx* ctx, const float* t_dev, uint64_t p, uint32_t d, double* gif_dev);

/* ---- output (src/testing.rs:740-801, 818-983) --------------------------- */
/* Write <out>.tsv: header chr pos snp_id {p_,beta_,t_}xcov r2_cov r2_latent
 * r2_resid, numbers in Rust "{:.6e}" form.  chrom/snp_id are arrays of p
 * C strings, cov_names d C strings.  Formatting runs on n_threads host
 * threads (0 = all). */
int slfmm_write_tsv(const char* path, uint64_t p, uint32_t d, const char* const* chrom,
                    const uint64_t* pos, const char* const* snp_id,
                    const char* const* cov_names, const slfmm_results* res, int n_threads);

#define SLFMM_PARQUET_UNCOMPRESSED 0  /* CompressionCodec::UNCOMPRESSED          */
#define SLFMM_PARQUET_ZSTD         6  /* CompressionCodec::ZSTD (the reference's);
                                         libzstd.so.1 is loaded at run time      */
/* Write <out>.parquet, the --format parquet output (coalesce_output_parquet,
 * src/testing.rs:818-983): columns chr, pos, snp_id, p_<cov>...,
 * beta_<cov>..., t_<cov>..., r2_cov, r2_latent, r2_resid, all required
 * (build_calibrated_schema, src/testing.rs:620-640), rows in SNP order, row
 * groups of 2^18 rows encoded on n_threads host threads (0 = all).
 * SLFMM_ERR_IO if the file cannot be written or ZSTD is asked for and libzstd
 * cannot be loaded. */
int slfmm_write_parquet(const char* path, uint64_t p, uint32_t d, const char* const* chrom,
                        const uint64_t* pos, const char* const* snp_id,
                        const char* const* cov_names, const slfmm_results* res,
                        int compression, int n_threads);
/* Format one value like Rust "{:.6e}"; returns the length written. */
int slfmm_format_exp6(double v, char* buf, size_t buf_len);

#ifdef __cplusplus
}
#endif
#endif /* SCHNELGPU_H */
