// Stage (c): per-SNP association statistics, t^2 histogram, genomic
// inflation factor and calibrated p-values.
//
// Reference: test_associations_fused (src/testing.rs:252-528), t_test
// (:1036-1048), TsqHistogram (:114-225), calibrate_batch (:685-728).
//
// The contraction produces, per SNP j, u = Q_C^T y_j where Q_C is an
// orthonormal basis of [1 | X | U_hat] built by Cholesky-Gram-Schmidt in
// that column order (the intercept coordinate is identically zero because
// every standardised column sums to zero).  From u and the exact TSS:
//   RSS     = TSS - ||u||^2                     (= ||y - C theta||^2)
//   SS_cov  = sum_{k<d} u_k^2                   (= ||H_X y||^2)
//   theta_j = (L^-T u)_{1+j},  c_jj = [(C^T C)^-1]_{1+j,1+j}
//   beta    = R ((I - P_U) X)^T Q_C u          (ridge effect, Step 3)
// which is the reference's O(n^2)-per-SNP algebra in O(n (1+d+K)).
#include <mutex>
#include <string>

#include "fp_convert.cuh"
#include "slfmm_internal.h"

namespace slfmm {
namespace {

// Tiles of 64 SNPs; each of 256 threads owns 4 SNPs x 4 traits of theta and
// beta.  The coefficient rows stay in shared memory (transposed, traits
// padded to 64) for the whole persistent CTA; the tile's u values are staged
// k-major, so one k step is three 16-byte loads and 32 FMAs per thread.
constexpr int kTileSnps = 64;
constexpr int kTraitPad = 64;

// Histogram bin of one FP32 t statistic by the reference's rule applied to
// that value: t_sq = t * t in FP64, skipped when not finite, bin =
// min(floor(t_sq / 0.001), last) (src/testing.rs:135-149); -1 when skipped.
// t * t * 1000 in FP32 is within 1.2e-7 relative of t_sq / 0.001, so its
// floor is the bin unless it lies within that distance of a bin edge (about
// one value in 4000 near t^2 = 1); those values, and any whose FP32 square
// overflows, take the FP64 division.
__device__ __forceinline__ int tsq_bin(float t) {
    if (!isfinite(t)) return -1;
    const float xf = t * t * 1000.0f;
    const float fl = floorf(xf);
    const float fr = xf - fl;                 // exact while xf < 2^23
    const float tol = xf * 2.5e-7f;
    if (xf < 8388608.0f && fr > tol && fr < 1.0f - tol)
        return fl >= (float)(kHistBins - 1) ? kHistBins - 1 : (int)fl;
    const double q = floor(((double)t * (double)t) / kHistWidth);
    return q >= (double)(kHistBins - 1) ? kHistBins - 1 : (int)q;
}
constexpr int kUsStride = kTileSnps + 4;  // 16-byte rows, staggered banks


// One block of up to 64 traits per launch: traits [t0, t0 + d) of a model
// with d_model covariates (the first d_model coordinates of u are the
// covariate ones, so SS_cov always sums over d_model); beta and t32 rows
// have d_model entries and point at trait t0; r2 may be null (written by the
// launch of the first block).
__global__ void __launch_bounds__(256, 3) k_assoc_epilogue(
    uint64_t p, const float* __restrict__ u, int ldu, const double* __restrict__ tss,
    const uint8_t* __restrict__ zero_var, int d, int d_model, int w, double df,
    const float* __restrict__ theta_rows, const float* __restrict__ beta_rows,
    const double* __restrict__ cjj, const uint8_t* __restrict__ dropped,
    double* __restrict__ beta, float* __restrict__ t32, double* __restrict__ r2,
    uint32_t* __restrict__ hist) {
    extern __shared__ __align__(16) float sm[];
    float* thT = sm;                          // [w][64]
    float* btT = thT + w * kTraitPad;         // [w][64]
    float* us = btT + w * kTraitPad;          // [w][68]
    float* s2s = us + w * kUsStride;          // [64] sigma^2 per SNP of the tile
    int* zvs = reinterpret_cast<int*>(s2s + kTileSnps);
    float* sss = s2s + 2 * kTileSnps;         // [64] ||u||^2 per SNP of the tile
    float* scs = sss + kTileSnps;             // [64] its covariate part
    __shared__ float cj[kTraitPad];
    __shared__ int dr[kTraitPad];
    const int tid = threadIdx.x;
    for (int e = tid; e < w * kTraitPad; e += blockDim.x) {
        const int k = e / kTraitPad, jj = e % kTraitPad;
        thT[e] = jj < d ? theta_rows[jj * w + k] : 0.f;
        btT[e] = jj < d ? beta_rows[jj * w + k] : 0.f;
    }
    for (int jj = tid; jj < kTraitPad; jj += blockDim.x) {
        cj[jj] = jj < d ? (float)cjj[jj] : 0.f;
        dr[jj] = jj < d ? (int)dropped[jj] : 1;
    }
    const int sg = tid >> 4, tg = tid & 15;
    const uint64_t ntiles = (p + kTileSnps - 1) / kTileSnps;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint64_t j0 = tile * kTileSnps;
        __syncthreads();  // the previous tile's values are consumed (and the tables are in place)
        for (int e = tid; e < w * kTileSnps; e += blockDim.x) {
            const int k = e / kTileSnps, sn = e % kTileSnps;
            us[k * kUsStride + sn] = j0 + sn < p ? u[(j0 + sn) * ldu + k] : 0.f;
        }
        __syncthreads();
        // per-SNP sums, 8 lanes per SNP with stride-8 partials, two rounds of 32
        for (int half = 0; half < 2; ++half) {
            const int sn = half * 32 + (tid >> 3), l8 = tid & 7;
            float ss = 0.f, sc = 0.f;
            for (int k = l8; k < w; k += 8) {
                const float v = us[k * kUsStride + sn];
                ss = fmaf(v, v, ss);
                if (k < d_model) sc = fmaf(v, v, sc);
            }
#pragma unroll
            for (int o = 4; o > 0; o >>= 1) {
                ss += __shfl_xor_sync(0xffffffffu, ss, o);
                sc += __shfl_xor_sync(0xffffffffu, sc, o);
            }
            if (l8 == 0) {
                sss[sn] = ss;
                scs[sn] = sc;
            }
        }
        __syncthreads();
        // the FP64 part per SNP on one lane each (two full warps): this part's
        // FP64 pipe is a small fraction of the FP32 one
        if (tid < kTileSnps) {
            const int sn = tid;
            const uint64_t j = j0 + sn;
            float s2f = 0.f;
            int zv = 1;
            if (j < p) {
                zv = zero_var && zero_var[j];
                const double T = tss[j];
                double rss = T - (double)sss[sn];
                if (rss < 0.0 || zv) rss = 0.0;
                s2f = (float)(rss / df);
                double a = 0.0, b = 0.0, c = 0.0;
                if (T > 1e-300 && !zv) {                        // src/testing.rs:394-404
                    const double ssc = (double)scs[sn];
                    a = ssc / T;
                    b = fmax(T - rss - ssc, 0.0) / T;
                    c = rss / T;
                }
                if (r2) {
                    r2[j * 3 + 0] = a;
                    r2[j * 3 + 1] = b;
                    r2[j * 3 + 2] = c;
                }
            }
            s2s[sn] = s2f;
            zvs[sn] = zv;
        }
        __syncthreads();
        float th[4][4], bb[4][4];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) th[a][b] = bb[a][b] = 0.f;
        // the next k step's loads are issued before this step's FMAs
        float4 un = *reinterpret_cast<const float4*>(us + 4 * sg);
        float4 tn = *reinterpret_cast<const float4*>(thT + 4 * tg);
        float4 bn = *reinterpret_cast<const float4*>(btT + 4 * tg);
        for (int k = 0; k < w; ++k) {
            const float4 uv = un, tv = tn, bv = bn;
            if (k + 1 < w) {
                un = *reinterpret_cast<const float4*>(us + (k + 1) * kUsStride + 4 * sg);
                tn = *reinterpret_cast<const float4*>(thT + (k + 1) * kTraitPad + 4 * tg);
                bn = *reinterpret_cast<const float4*>(btT + (k + 1) * kTraitPad + 4 * tg);
            }
            const float ua[4] = {uv.x, uv.y, uv.z, uv.w};
            const float ta[4] = {tv.x, tv.y, tv.z, tv.w};
            const float ba[4] = {bv.x, bv.y, bv.z, bv.w};
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    th[a][b] = fmaf(ta[b], ua[a], th[a][b]);
                    bb[a][b] = fmaf(ba[b], ua[a], bb[a][b]);
                }
        }
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int sn = 4 * sg + a;
            const uint64_t j = j0 + sn;
            if (j >= p) continue;
            const bool zv = zvs[sn] != 0;
            const float s2f = s2s[sn];
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const int jj = 4 * tg + b;
                if (jj >= d) continue;
                float t = 0.f;
                const float var = s2f * cj[jj];
                if (!zv && !dr[jj] && var > 0.f && isfinite(var)) {  // t_test guards
                    t = th[a][b] * rsqrtf(var);
                    if (!isfinite(t)) t = 0.f;
                }
                beta[j * d_model + jj] = zv ? 0.0 : f64_of_f32(bb[a][b]);
                t32[j * d_model + jj] = t;
                const int bin = tsq_bin(t);
                if (bin >= 0) atomicAdd(&hist[(uint64_t)jj * kHistBins + bin], 1u);
            }
        }
    }
}

// Median of the t^2 histogram of one trait (src/testing.rs:179-224) and the
// raw GIF (median < 1e-10 -> 1, else median / 0.4549).
__global__ void __launch_bounds__(1024) k_gif(const uint32_t* __restrict__ hist,
                                              double* __restrict__ gif_raw) {
    constexpr int kT = 1024;
    constexpr int kSeg = (kHistBins + kT - 1) / kT;
    __shared__ unsigned long long seg[kT];
    __shared__ unsigned long long excl[kT];
    __shared__ long long b1, b2;
    __shared__ unsigned long long total;
    const uint32_t* h = hist + (uint64_t)blockIdx.x * kHistBins;
    const int t = threadIdx.x;
    const int lo = t * kSeg, hi = min(kHistBins, lo + kSeg);
    unsigned long long s = 0;
    for (int b = lo; b < hi; ++b) s += h[b];
    seg[t] = s;
    if (t == 0) { b1 = -1; b2 = -1; }
    __syncthreads();
    if (t == 0) {
        unsigned long long acc = 0;
        for (int i = 0; i < kT; ++i) { excl[i] = acc; acc += seg[i]; }
        total = acc;
    }
    __syncthreads();
    const unsigned long long n = total;
    if (n == 0) {
        if (t == 0) gif_raw[blockIdx.x] = 1.0;  // median 0 -> GIF 1
        return;
    }
    const bool even = (n % 2) == 0;
    const unsigned long long target = even ? n / 2 - 1 : n / 2;
    // first bin whose cumulative count exceeds `target` (and target+1)
    for (int which = 0; which < (even ? 2 : 1); ++which) {
        const unsigned long long tg = target + which;
        if (tg >= excl[t] && tg < excl[t] + seg[t]) {
            unsigned long long cum = excl[t];
            for (int b = lo; b < hi; ++b) {
                cum += h[b];
                if (cum > tg) {
                    if (which == 0) b1 = b; else b2 = b;
                    break;
                }
            }
        }
    }
    __syncthreads();
    if (t == 0) {
        double med;
        if (!even) med = ((double)b1 + 0.5) * kHistWidth;
        else med = (((double)b1 + 0.5) * kHistWidth + ((double)b2 + 0.5) * kHistWidth) / 2.0;
        gif_raw[blockIdx.x] = med < 1e-10 ? 1.0 : med / kGifDivisor;
    }
}

// p = 2 * Phi(-|t| / sqrt(GIF_j)) = erfc(|z| / sqrt 2)  (src/testing.rs:691-712).
// The statistic is FP32, so erfcf carries its precision; the FP64 erfc is
// only used in the far tail where erfcf would leave the normal FP32 range.
constexpr int kMaxCalibTraits = 1024;

// The per-trait factors 1/sqrt(2 GIF) (FP32) and 1/sqrt(GIF) (FP64) are
// formed once per block: FP64 square roots and divisions per element would
// dominate on this part, whose FP64 rate is a small fraction of FP32; the
// widening of t and p to FP64 moves bits with integer operations.
__global__ void k_calibrate(uint64_t p, int d, const float* __restrict__ t32,
                            const double* __restrict__ gif, double* __restrict__ t64,
                            double* __restrict__ pval) {
    __shared__ float zs[kMaxCalibTraits];
    __shared__ double rs[kMaxCalibTraits];
    for (int j = threadIdx.x; j < d; j += blockDim.x) {
        const double r = 1.0 / sqrt(gif[j]);
        rs[j] = r;
        zs[j] = (float)(0.7071067811865476 * r);
    }
    __syncthreads();
    const uint64_t total = p * (uint64_t)d;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < total;
         e += (uint64_t)gridDim.x * blockDim.x) {
        const int jj = (int)(e % d);
        const float tf = t32[e];
        if (t64) t64[e] = f64_of_f32(tf);
        if (pval) {
            const float zf = fabsf(tf) * zs[jj];
            double pv;
            if (zf < 8.0f) pv = f64_of_f32(erfcf(zf));
            else pv = erfc(fabs((double)tf) * rs[jj] * 0.7071067811865476);
            pval[e] = pv;
        }
    }
}

// ---------------------------------------------------------------------------
// Allocation-free GIF (slfmm_gif_noalloc; no counterpart in the reference)
// ---------------------------------------------------------------------------
// The t^2 histogram lives in this fixed device array instead of memory
// allocated per call: kGifNoAllocMaxTraits x kHistBins counters (3.2 MB).
// Every call on a device shares it; each call zeroes the rows it uses first.
static __device__ __align__(256) uint32_t g_noalloc_hist[kGifNoAllocMaxTraits * kHistBins];

// Same binning as the association epilogue (tsq_bin) for every t of trait j.
__global__ void k_tsq_hist(const float* __restrict__ t, uint64_t p, int d, uint32_t* __restrict__ hist) {
    const uint64_t total = p * (uint64_t)d;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < total;
         e += (uint64_t)gridDim.x * blockDim.x) {
        const int jj = (int)(e % d);
        const int bin = tsq_bin(t[e]);
        if (bin >= 0) atomicAdd(&hist[(uint64_t)jj * kHistBins + bin], 1u);
    }
}

}  // namespace

// Device address of g_noalloc_hist on the current device.  The first call on
// a device asks the runtime for it (cudaGetSymbolAddress) and keeps it; later
// calls only read the cached pointer.
static uint32_t* noalloc_hist_address(int device) {
    constexpr int kMaxDevices = 64;
    static std::mutex mu;
    static uint32_t* addr[kMaxDevices] = {};
    SLFMM_REQUIRE(device >= 0 && device < kMaxDevices, SLFMM_ERR_BAD_ARG, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[device]) {
        void* ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_hist);
        if (e != cudaSuccess || !ptr)
            throw Error(SLFMM_ERR_CUDA, std::string("cudaGetSymbolAddress of the GIF histogram failed: ") +
                                            cudaGetErrorString(e));
        addr[device] = static_cast<uint32_t*>(ptr);
    }
    return addr[device];
}

// Context set-up for slfmm_gif_noalloc: the histogram's device address on
// this device, and the module of its two kernels loaded (CUDA loads modules
// lazily, at a kernel's first use; loading allocates device memory for the
// code and for the static histogram).  After this, a call allocates nothing.
void gif_noalloc_prepare(int device) {
    noalloc_hist_address(device);
    cudaFuncAttributes fa{};
    SLFMM_CUDA(cudaFuncGetAttributes(&fa, (const void*)k_tsq_hist));
    SLFMM_CUDA(cudaFuncGetAttributes(&fa, (const void*)k_gif));
}

void launch_gif_noalloc(Ctx& c, const float* t, uint64_t p, int d, double* gif_raw) {
    SLFMM_REQUIRE(d >= 0 && d <= kGifNoAllocMaxTraits, SLFMM_ERR_BAD_ARG,
                  "slfmm_gif_noalloc handles at most " + std::to_string(kGifNoAllocMaxTraits) +
                      " traits (its static histogram holds " + std::to_string(kGifNoAllocMaxTraits) + " x " +
                      std::to_string(kHistBins) + " counters); got " + std::to_string(d));
    if (d == 0) return;
    SLFMM_REQUIRE(gif_raw != nullptr && (p == 0 || t != nullptr), SLFMM_ERR_BAD_ARG, "null device pointer");
    uint32_t* hist = noalloc_hist_address(c.device);
    SLFMM_CUDA(cudaMemsetAsync(hist, 0, (size_t)d * kHistBins * sizeof(uint32_t), c.stream));
    if (p > 0) {
        k_tsq_hist<<<grid_for(c, p * (uint64_t)d, 256), 256, 0, c.stream>>>(t, p, d, hist);
        SLFMM_LAUNCHED(c, "k_tsq_hist");
    }
    k_gif<<<d, 1024, 0, c.stream>>>(hist, gif_raw);
    SLFMM_LAUNCHED(c, "k_gif");
}

void launch_assoc_epilogue(Ctx& c, uint64_t p, const float* u, int ldu, const double* tss,
                           const AssocConsts& k, double* beta, float* t32, double* r2,
                           uint32_t* hist) {
    if (p == 0) return;
    const size_t smem = (size_t)(2 * k.w * kTraitPad + k.w * kUsStride + 4 * kTileSnps) * sizeof(float);
    SLFMM_REQUIRE(smem <= 227 * 1024, SLFMM_ERR_BAD_ARG, "association design too wide for the epilogue");
    raise_dynamic_smem((const void*)k_assoc_epilogue, smem);
    const uint64_t tiles = ceil_div(p, (uint64_t)kTileSnps);
    // one wave of persistent CTAs: as many per SM as fit (registers and
    // shared memory), so no CTA starts its share of tiles after the others
    int per_sm = 0;
    SLFMM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_assoc_epilogue, 256, smem));
    const unsigned grid = (unsigned)std::min<uint64_t>(tiles, (uint64_t)c.sm_count * std::max(per_sm, 1));
    // traits in blocks of 64 (the coefficient tables of one block stay in
    // shared memory); every block reads the same u rows
    for (int t0 = 0; t0 < k.d; t0 += kTraitPad) {
        const int db = std::min(kTraitPad, k.d - t0);
        k_assoc_epilogue<<<grid, 256, smem, c.stream>>>(
            p, u, ldu, tss, k.zero_var, db, k.d, k.w, k.df, k.theta_rows + (size_t)t0 * k.w,
            k.beta_rows + (size_t)t0 * k.w, k.cjj + t0, k.dropped + t0, beta + t0, t32 + t0, t0 == 0 ? r2 : nullptr,
            hist + (size_t)t0 * kHistBins);
        SLFMM_LAUNCHED(c, "k_assoc_epilogue");
    }
}

void launch_gif(Ctx& c, const uint32_t* hist, int d, double* gif_raw) {
    if (d == 0) return;
    k_gif<<<d, 1024, 0, c.stream>>>(hist, gif_raw);
    SLFMM_LAUNCHED(c, "k_gif");
}

void launch_calibrate(Ctx& c, uint64_t p, int d, const float* t32, const double* gif, double* t64,
                      double* pval) {
    if (p == 0 || d == 0) return;
    SLFMM_REQUIRE(d <= kMaxCalibTraits, SLFMM_ERR_BAD_ARG, "too many traits for the calibration kernel");
    // few blocks: each forms the d per-trait factors in FP64 before its loop
    const unsigned grid = (unsigned)std::min<int>(grid_for(c, p * d, 256), c.sm_count * 8);
    k_calibrate<<<grid, 256, 0, c.stream>>>(p, d, t32, gif, t64, pval);
    SLFMM_LAUNCHED(c, "k_calibrate");
}

}  // namespace slfmm
