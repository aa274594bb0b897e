// Internal declarations of the schnelgpu runtime (host C++ + sm_103a kernels).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/schnelgpu.h"

namespace slfmm {

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define SLFMM_CUDA(call)                                                          \
    do {                                                                          \
        cudaError_t e_ = (call);                                                  \
        if (e_ != cudaSuccess)                                                    \
            throw ::slfmm::Error(SLFMM_ERR_CUDA, std::string(#call) + ": " +     \
                                 cudaGetErrorString(e_));                        \
    } while (0)

#define SLFMM_REQUIRE(cond, code, msg)                                            \
    do {                                                                          \
        if (!(cond)) throw ::slfmm::Error((code), (msg));                         \
    } while (0)

// ---------------------------------------------------------------------------
// constants shared by host and device
// ---------------------------------------------------------------------------
constexpr int kHistBins = 100000;      // src/testing.rs:124
constexpr long long kWaitCyclesMax = 8000000000ll;  // the device waits' own limit (~4 s at 2 GHz)
constexpr int kGifNoAllocMaxTraits = 8; // traits the static histogram of slfmm_gif_noalloc holds
constexpr int kMaxNmfK = 32;            // NMF rank limit of the imputation kernels
constexpr double kHistWidth = 0.001;   // src/testing.rs:125
constexpr double kGifDivisor = 0.4549; // src/testing.rs:169
constexpr int kMaxW = 128;             // widest GEMM operand (columns)
constexpr int kMaxSmall = 128;         // largest small dense matrix (w x w) in shared memory
constexpr int kMaxDesign = 256;        // widest association design C = [1 | X | U_hat] (1 + d + K)

inline uint64_t round_up(uint64_t x, uint64_t m) { return (x + m - 1) / m * m; }
inline uint64_t ceil_div(uint64_t x, uint64_t m) { return (x + m - 1) / m; }

// ---------------------------------------------------------------------------
// device buffers (stream-ordered pool allocator)
// ---------------------------------------------------------------------------
struct Ctx;

template <typename T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaStream_t s = nullptr;
    DBuf() = default;
    DBuf(size_t count, cudaStream_t st) { alloc(count, st); }
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    DBuf(DBuf&& o) noexcept : p(o.p), n(o.n), s(o.s) { o.p = nullptr; o.n = 0; }
    DBuf& operator=(DBuf&& o) noexcept {
        if (this != &o) { release(); p = o.p; n = o.n; s = o.s; o.p = nullptr; o.n = 0; }
        return *this;
    }
    void alloc(size_t count, cudaStream_t st) {
        release();
        s = st;
        n = count;
        if (count == 0) return;
        cudaError_t e = cudaMallocAsync((void**)&p, count * sizeof(T), st);
        if (e != cudaSuccess) {
            p = nullptr;
            throw Error(e == cudaErrorMemoryAllocation ? SLFMM_ERR_NOMEM : SLFMM_ERR_CUDA,
                        std::string("device allocation of ") + std::to_string(count * sizeof(T)) +
                            " bytes failed: " + cudaGetErrorString(e));
        }
    }
    void zero() {
        if (n) SLFMM_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s));
    }
    void release() {
        if (p) cudaFreeAsync(p, s);
        p = nullptr;
        n = 0;
    }
    // free later on another (live) stream than the one it was allocated on
    void rebind(cudaStream_t st) { s = st; }
    ~DBuf() { release(); }
    T* get() const { return p; }
    size_t bytes() const { return n * sizeof(T); }
};

// ---------------------------------------------------------------------------
// resident genotype matrix
// ---------------------------------------------------------------------------
struct Geno {
    uint64_t n = 0;        // samples (after sample_keep)
    uint64_t p = 0;        // SNPs (after SNP subset)
    uint64_t stride = 0;   // bytes per SNP row on device (multiple of 128)
    DBuf<uint8_t> packed;  // p x stride, codes of samples >= n are 00
    DBuf<int32_t> counts;  // p x 4: c0, c1(het), c2(hom alt), cmiss
    // missing-call lists, built on first use (caches of the packed matrix)
    mutable bool have_csr = false;
    mutable uint64_t nnz = 0;
    mutable DBuf<uint64_t> miss_ptr;   // p+1, CSR by SNP
    mutable DBuf<uint32_t> miss_idx;   // nnz sample indices (ascending)
    mutable bool have_csc = false;
    mutable DBuf<uint64_t> missT_ptr;  // n+1, CSC by sample
    mutable DBuf<uint32_t> missT_idx;  // nnz SNP indices (ascending)
    mutable uint64_t missT_max = 0;    // longest per-sample list
    // transposed copy (rows = samples, codes of every SNP), built on first use
    mutable bool have_T = false;
    mutable uint64_t strideT = 0;
    mutable DBuf<uint8_t> packedT;     // n x strideT
    // tile-major copies for the tensor-core passes, built on first use:
    // [tile of 128 rows][K block of 128 codes][128 rows][32 B], so every
    // (tile, K block) operand is one contiguous 4 KiB run of HBM; the tile
    // count is padded to a multiple of 8 with zero tiles
    mutable bool have_tiles = false, have_tilesT = false;
    mutable uint64_t kbt = 0, kbtT = 0;      // K blocks per tile
    mutable uint64_t ntiles = 0, ntilesT = 0;
    mutable DBuf<uint8_t> tiles, tilesT;
    // make every buffer free on `st` (the owning context may be gone)
    void rebind(cudaStream_t st) {
        packed.rebind(st); counts.rebind(st); miss_ptr.rebind(st); miss_idx.rebind(st);
        missT_ptr.rebind(st); missT_idx.rebind(st); packedT.rebind(st);
        tiles.rebind(st); tilesT.rebind(st);
    }
};

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
// CUDA-event timing of named kernels (enabled by slfmm_profile_enable)
struct ProfRec {
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending;
    uint64_t launches = 0;
    double ms = 0.0, bytes = 0.0, flops = 0.0;
};

struct Ctx {
    int device = 0;
    int precision = SLFMM_PREC_SPLIT_FP8;
    int verbose = 0;
    bool own_stream = false;
    cudaStream_t stream = nullptr;
    cudaStream_t copy_stream = nullptr;
    std::string last_error;
    uint64_t launches = 0;
    int sm_count = 0;
    DBuf<int> dev_flags;   // [0] device timeout flag, [1] error info
    bool profiling = false;
    std::map<std::string, ProfRec> prof;
    double phase_t0 = 0.0;  // verbose phase log: start of the current phase (ms)
    // with profiling on: an event on the stream and the host clock at every
    // phase mark of the last fit (no synchronisation)
    struct PhaseMark {
        std::string name;
        cudaEvent_t ev;
        double host_ms;
    };
    std::vector<PhaseMark> phase_marks;
    int rng = SLFMM_RNG_CHACHA8;  // stream of the Gaussian sketches
    long long expire_next_wait = 0;  // test hook: next split-FP8 launch's wait limit (SM cycles)
    // a host draw of the reference's sketch stream started ahead of its use
    struct PendingNormal;
    std::shared_ptr<PendingNormal> pending_normal;
    bool autotune = false;   // time the tensor-core ring depths per shape once
    std::map<std::string, std::pair<int, int>> tuned;  // shape -> (packed ring cap, W ring cap)
};

// bracket a launch with CUDA events when profiling is on
struct ProfScope {
    Ctx& c;
    const char* name;
    double bytes, flops;
    cudaEvent_t a = nullptr, b = nullptr;
    ProfScope(Ctx& ctx, const char* nm, double by, double fl) : c(ctx), name(nm), bytes(by), flops(fl) {
        if (c.profiling) {
            cudaEventCreate(&a);
            cudaEventCreate(&b);
            cudaEventRecord(a, c.stream);
        }
    }
    ~ProfScope() {
        if (a) {
            cudaEventRecord(b, c.stream);
            ProfRec& r = c.prof[name];
            r.pending.emplace_back(a, b);
            r.launches += 1;
            r.bytes += bytes;
            r.flops += flops;
        }
    }
};
void profile_collect(Ctx& c);

// grid size for a grid-stride loop over `work` items
inline int grid_for(const Ctx& c, uint64_t work, int block) {
    const uint64_t want = ceil_div(work, (uint64_t)block);
    const uint64_t cap = (uint64_t)(c.sm_count > 0 ? c.sm_count : 1) * 32;
    const uint64_t g = want < cap ? want : cap;
    return (int)(g > 0 ? g : 1);
}

// Raise a kernel's dynamic shared-memory limit to at least `bytes` (no-op up
// to 48 KiB).  The limit is a process-wide attribute of the function, and
// contexts may launch from several host threads, so it only ever grows:
// every launch finds it at least as large as it set it.
void raise_dynamic_smem(const void* fn, size_t bytes);

// count + check a kernel launch
void after_launch(Ctx& c, const char* name);
#define SLFMM_LAUNCHED(ctx, name) ::slfmm::after_launch((ctx), (name))

// ---------------------------------------------------------------------------
// kernel entry points (host wrappers, defined in the .cu files)
// ---------------------------------------------------------------------------
// k_decode.cu
void launch_repack(Ctx& c, const uint8_t* in, uint64_t rows, uint64_t in_bps, uint64_t n_phys,
                   const uint32_t* keep, uint64_t n_out, uint8_t* out, uint64_t stride);
void launch_snp_counts(Ctx& c, const Geno& g, uint64_t* miss_count_out);
// counts of rows [r0, r0 + rows) only
void launch_snp_counts_range(Ctx& c, const Geno& g, uint64_t r0, uint64_t rows);
void build_missing_lists(Ctx& c, const Geno& g);
void build_missing_csc(Ctx& c, const Geno& g);
// missing counts p (from g.counts) and the CSR fill from the SNP-major tiles,
// for matrices without a row-major copy
void launch_miss_counts_of(Ctx& c, const Geno& g, uint64_t* mc);
void launch_miss_fill_tiles(Ctx& c, const Geno& g);
// missing-call lists of an upload chunk [r0, r0 + rows): offsets continue
// g.miss_ptr[r0] (needs the chunk's counts); the fill writes below cap only
void csr_chunk_offsets(Ctx& c, const Geno& g, uint64_t r0, uint64_t rows);
void csr_chunk_fill(Ctx& c, const Geno& g, uint64_t r0, uint64_t rows, uint64_t cap);
void launch_stats_mean_range(Ctx& c, const Geno& g, uint64_t r0, uint64_t rows, int norm, double* mean,
                             double* scale, double* tss, uint8_t* zero_var);
void launch_stats_mean(Ctx& c, const Geno& g, int norm, double* mean, double* scale,
                       double* tss, uint8_t* zero_var);
void launch_decode_chunk(Ctx& c, const Geno& g, uint64_t snp0, uint64_t ncols,
                         const double* mean, const double* scale, double* out);
// per-SNP 4-entry lookup tables (value of code 0,1,2,3)
void launch_lut_std(Ctx& c, uint64_t p, const double* mean, const double* scale, float* lut);

// k_sim.cu : synthetic structured cohort written into a device packed matrix
void launch_simulate(Ctx& c, uint64_t n, uint64_t p, int n_pop, const float* admix_dev, double fst,
                     double f_lo, double f_hi, double miss, double inbreeding, uint64_t seed, uint8_t* out,
                     uint64_t stride);

// k_simt.cu : plain FP32 contractions over the packed matrix
// out[j, c] = sum_i lut_j[code_ij] * W[i, c]      (j in [0,p), ldw = wp)
void launch_row_lut(Ctx& c, const Geno& g, const float* lut, const float* W, int wp, float* out);
// S[i, c] = sum_j lut_j[code_ij] * Q[j, c]        (FP64 result, n x wp)
void launch_col_lut(Ctx& c, const Geno& g, const float* lut, const float* Q, int wp, double* S);

void launch_reduce_splits(Ctx& c, const float* part, int splits, uint64_t n, int wp, uint64_t n_pad,
                          double* S);

// k_tc.cu : tcgen05 split-BF16 contractions
bool tc_available(Ctx& c);
// W (K x w, ld) -> [2 wpad][K_pad] BF16 hi/lo (optional per-K-row scale)
void launch_split_bf16_f64(Ctx& c, const double* src, int ld, uint64_t K, int w, int wpad, uint64_t K_pad,
                           const double* kscale, __nv_bfloat16* dst);
void launch_split_bf16_f32(Ctx& c, const float* src, int ld, uint64_t K, int w, int wpad, uint64_t K_pad,
                           const double* kscale, __nv_bfloat16* dst);
void build_transposed(Ctx& c, const Geno& g);
// out[r, c] = sum_k g(r, k) * (hi + lo)[c, k] over packed rows; split-K over
// grid.y writes splits x rows x ldo partials (split_stride apart)
int launch_tc_rows(Ctx& c, const uint8_t* packed, uint64_t stride, uint64_t rows, uint64_t K,
                    const __nv_bfloat16* bsplit, uint64_t K_pad, int wpad, float* out, int ldo, int splits,
                    uint64_t split_stride);
int tc_split_count(Ctx& c, uint64_t rows, uint64_t K);
// (W has n rows of ldw floats)
void launch_rowfix_mean(Ctx& c, float* P, int ldp, uint64_t rows, int w, const uint64_t* ptr, const uint32_t* idx,
                        const float* W, int ldw, uint64_t n, const double* cs, const double* mean,
                        const double* scale);
void launch_colfix_mean(Ctx& c, double* S, int lds, uint64_t n, int w, const uint64_t* ptr, const uint32_t* idx,
                        const float* Q, int ldq, const double* coef, const double* colterm);
void launch_weighted_colsum(Ctx& c, const float* Q, int ldq, uint64_t p, int w, const double* coef, double* out);
void launch_scale_product(Ctx& c, const double* a, const double* b, uint64_t n, double* out);

// k_tc8.cu : split-FP8 tcgen05 contractions with optional missing-call
// indicator operand
struct Fp8Plan {
    uint32_t wpad, n_main, n_ind, n_total, d_cols, a_cols, stages, wstages, pstages, group, tmem_cols, b_stage_bytes;
    uint32_t kcopies, nsplit, a_base;
    uint32_t ind_shared;  // indicator MMAs read the leading main terms (B holds n_main rows)
    size_t smem;
    bool ok;
};
// ind_shared: the indicator operand's terms are the first kIndTerms terms of
// the main operand's split (a row pass: both multiply the same W), so B holds
// only the main terms and the indicator MMAs read their leading rows
Fp8Plan fp8_plan(int wpad, bool ind, uint64_t tiles, bool ind_shared = false);
Fp8Plan fp8_plan_knobs(int wpad, bool ind, uint64_t tiles, int pmax, int smax, int gmax, int wmax,
                       bool ind_shared = false);
// the row-major packed copy of a matrix (a sample subset built from the
// tile-major copies has none: the passes that need it must not run on it)
inline const uint8_t* packed_rows(const Geno& g) {
    SLFMM_REQUIRE(g.packed.get() != nullptr, SLFMM_ERR_BAD_ARG, "this matrix has no row-major packed copy");
    return g.packed.get();
}

// tile-major packed operand (rows = SNPs, or samples when transposed)
struct TileView {
    const uint8_t* base;
    uint64_t kbt, ntiles;
    uint64_t tile0 = 0;  // index of the first tile in the whole matrix
};
TileView build_tiles(Ctx& c, const Geno& g, bool transposed);
// The samples keep_dev[0 .. n_keep) of a matrix as a new matrix holding only
// the tile-major copies and the counts (no row-major copy): the kept rows of
// the sample-major tiles, their 2-bit transpose, counts from the tiles.
void tiles_subset_samples(Ctx& c, const Geno& full, const uint32_t* keep_dev, uint64_t n_keep, Geno& sub);
void tile_chunk(Ctx& c, const Geno& g, uint64_t r0, uint64_t r1, bool last);
// `terms` E4M3 terms of diag(kscale) src at rows row_off + t * wpad + c of a
// stage-major W operand of n_rows rows (every 256-sample stage one contiguous,
// pre-swizzled blob: one bulk copy per stage in k_tc8_rows)
void launch_fp8_terms_f64(Ctx& c, const double* src, int ld, uint64_t K, int w, int wpad, uint64_t K_pad,
                          const double* kscale, int terms, int row_off, int n_rows, uint8_t* B, float* inv_scale);
// both operands of a transposed pass in one pass over src: 4 terms of
// diag(ks_main) src at B rows 0.., and (ks_ind non-null) 3 terms of
// diag(ks_ind) src at B rows ind_row_off..; the same terms as two separate
// term launches
void launch_fp8_terms_f32_pair(Ctx& c, const float* src, int ld, uint64_t K, int w, int wpad, uint64_t K_pad,
                               const double* ks_main, const double* ks_ind, int ind_row_off, int n_rows, uint8_t* B,
                               float* inv_scale);
// mode 0: out = P (+ M); mode 1: out = s_r (P - mu_r (cs_c - M)) (needs the indicator).
// err_dev null: the launch waits and throws when a bounded device wait expired;
// non-null: the kernel records the site there and the caller checks it later.
int launch_tc8_rows(Ctx& c, const Fp8Plan& pl, const TileView& tv, uint64_t rows, uint64_t K,
                     const uint8_t* B, const float* inv_scale, uint64_t K_pad, int mode, const double* row_mean,
                     const double* row_scale, const double* cs, float* out, int ldo, int splits,
                     uint64_t split_stride, int* err_dev = nullptr);
void throw_tc8_timeout(int site);
void launch_sub_colterm(Ctx& c, double* S, int lds, uint64_t n, int w, const double* colterm);

// k_nmf.cu : NMF imputation -- fill-aware statistics, sparse corrections of
// the contractions at the missing calls, multiplicative updates, CV
void launch_fill_stats(Ctx& c, const Geno& g, int norm, const float* W, const float* H, int k, double* mean,
                       double* scale, double* tss, uint8_t* zero_var);
void launch_fill_row_correct(Ctx& c, const Geno& g, float* out, int ldo, int w, const float* Wop, int ldw,
                             const float* Wn, const float* H, int k, const double* mean, const double* scale);
void launch_fill_col_correct(Ctx& c, const Geno& g, double* S, int lds, int w, const float* Qop, int ldq,
                             const float* Wn, const float* H, int k, const double* mean, const double* scale);
void launch_add_mean_colsum(Ctx& c, float* out, int ldo, uint64_t p, int w, const double* mean, const double* cs);
void launch_nmf_update_f64(Ctx& c, double* X, uint64_t m, int k, const double* num, int ldn, const double* denom,
                           double eps);
void launch_nmf_update_f32(Ctx& c, double* X, uint64_t m, int k, const float* num, int ldn, const double* denom,
                           double eps);
void launch_nmf_normalize(Ctx& c, double* W, uint64_t n, double* H, uint64_t p, int k, const double* colsum,
                          double eps);
void launch_nmf_abs_f64(Ctx& c, const double* src, int ld, double* X, uint64_t m, int k);
void launch_nmf_clamp0_f32(Ctx& c, const float* src, int ld, double* X, uint64_t m, int k);
void launch_nmf_cv(Ctx& c, const Geno& g, uint64_t chunk, uint64_t mask_seed, double rate, const float* W,
                   const float* H, int k, double* part);
void launch_nmf_gwas_cv(Ctx& c, const Geno& g, uint64_t chunk, uint64_t seed, double rate, const float* W,
                        const float* Wpt, int k, double* part);

// k_small.cu : FP64 dense helpers (row-major)
void launch_colmeans(Ctx& c, const double* A, uint64_t m, int a, int lda, double* out);
void launch_colsums(Ctx& c, const double* A, uint64_t m, int a, int lda, double* out);
void launch_sum_partials(Ctx& c, const double* part, int splits, uint64_t count, double* out);
void launch_center_cols(Ctx& c, double* A, uint64_t m, int a, int lda, const double* means);
void launch_scale_cols_sd(Ctx& c, double* A, uint64_t m, int a, int lda);
void launch_atb(Ctx& c, const double* A, int lda, const double* B, int ldb, uint64_t m, int a,
                int b, double* out);  // out (a x b) = A^T B
void launch_gram_f32(Ctx& c, const float* A, int lda, uint64_t m, int a, double* out);
void launch_gemm_small(Ctx& c, const double* A, int lda, uint64_t m, int a, const double* B,
                       int ldb, int b, double alpha, double beta, double* C, int ldc);
// A <- A * Linv^T (Linv lower-triangular a x a, a <= 64)
void launch_trmul_f32(Ctx& c, float* A, int lda, uint64_t m, int a, const double* Linv);
// in place lower Cholesky; drop_tol < 0: replace non-positive pivots by a
// tiny value; drop_tol >= 0: drop (L_kk = 1, column zero) dependent columns
void launch_cholesky(Ctx& c, double* A, int a, int* status, double drop_tol = -1.0,
                     int* dropped = nullptr);
void launch_transpose(Ctx& c, const double* A, int rows, int cols, double* At);
void launch_scale_cols(Ctx& c, double* A, uint64_t m, int a, int lda, const double* f);
void launch_build_design(Ctx& c, const double* X, int d, const double* U, int K, uint64_t n,
                         double* C);
void launch_tri_inv_lower(Ctx& c, const double* L, int a, double* Linv);
void launch_inverse(Ctx& c, const double* A, int a, double* Ainv, int* status, double* eps_used);
// one-sided Jacobi SVD (a <= 64): A is overwritten with U, V and sig
// (descending) written
void launch_jacobi_svd(Ctx& c, const double* A, int a, double* V, double* sig);
void launch_normal(Ctx& c, uint64_t seed, uint64_t rows, int cols, double* out);
// rows x cols Normal(0, 1) sketch into device memory from the context's
// stream: the device counter stream (launch_normal) or the reference's ChaCha8
// stream drawn on the host (reference_normal) and copied
void draw_normal(Ctx& c, uint64_t seed, uint64_t rows, int cols, double* out);
// start the host draw of draw_normal(c, seed, rows, cols, .) on host threads
// now (no-op for the device counter stream); draw_normal then waits for it
void prefetch_normal(Ctx& c, uint64_t seed, uint64_t rows, int cols);
void reference_normal(uint64_t seed, uint64_t rows, uint64_t cols, double* out);
void launch_f64_to_f32_pad(Ctx& c, const double* A, uint64_t m, int a, int lda, float* out,
                           uint64_t m_pad, int ldo);
void launch_f32_to_f64(Ctx& c, const float* A, uint64_t m, int a, int lda, double* out, int ldo);

// k_assoc.cu
struct AssocConsts {
    int d, w;           // covariates, latent-augmented width (cols of u = w)
    double df;
    const float* theta_rows;  // d x w (rows of L^-T restricted to X coefficients)
    const float* beta_rows;   // d x w
    const double* cjj;        // d
    const uint8_t* dropped;   // d
    const uint8_t* zero_var;  // p (may be null): SNP with no variance
};
void launch_assoc_epilogue(Ctx& c, uint64_t p, const float* u, int ldu, const double* tss,
                           const AssocConsts& k, double* beta, float* t32, double* r2,
                           uint32_t* hist);
void launch_gif(Ctx& c, const uint32_t* hist, int d, double* gif_raw);
// raw GIF per trait from p x d FP32 t statistics using the static per-device
// histogram (allocates nothing)
void launch_gif_noalloc(Ctx& c, const float* t, uint64_t p, int d, double* gif_raw);
void gif_noalloc_prepare(int device);
void launch_calibrate(Ctx& c, uint64_t p, int d, const float* t32, const double* gif_per_trait,
                      double* t64, double* pval);

}  // namespace slfmm
