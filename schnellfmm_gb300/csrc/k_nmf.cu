// NMF imputation (src/nmf.rs:80-455, src/parallel.rs:219-321,
// src/testing.rs:423-487) on the resident genotypes.
//
// The dense products of the multiplicative updates and of the imputed passes
// run through the ordinary contractions with missing calls as 0; the values
// NMF puts at the missing calls, f_ir = W_i . H_r, enter as sparse
// corrections over the missing-call lists (CSR by SNP, CSC by sample), so no
// imputed copy of the matrix is ever formed.  W (n x k) and H (p x k, one row
// per SNP) are FP32 row-major here; k <= kMaxNmfK (kernels are built for
// rank bounds 16 and 32).
#include <cmath>
#include <cstdint>

#include "slfmm_internal.h"
#include "stats_common.cuh"

namespace slfmm {
namespace {

constexpr uint64_t kGamma = 0x9E3779B97F4A7C15ull;

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Draw `ctr` of the counter stream keyed by mix64(seed + gamma) is the
// uniform (m >> 11) 2^-53; it is below `rate` iff (m >> 11) < ceil(rate 2^53)
// -- compared as integers, without forming the FP64 uniform
__device__ __forceinline__ bool draw_below(uint64_t key, uint64_t ctr, uint64_t thresh) {
    return (mix64(key + (ctr + 1) * kGamma) >> 11) < thresh;
}

// The reference's mask stream (src/nmf.rs:433-434, src/testing.rs:437-438):
// ChaCha8Rng::seed_from_u64(seed) sampled by Uniform(0, 1).  Output `ctr` is
// keystream words 2 ctr and 2 ctr + 1 (block ctr / 8: 64-bit block counter in
// state words 12-13, stream id 0), the key 8 PCG32 XSH-RR outputs of the seed
// (the same stream host_rng.cpp draws for the sketches), and the uniform
// (u64 >> 12) 2^-52, below `rate` iff (u64 >> 12) < ceil(rate 2^52).  The
// last block stays in registers, so consecutive counters reuse it.
__device__ __forceinline__ void chacha_quarter(uint32_t& a, uint32_t& b, uint32_t& c, uint32_t& d) {
    a += b; d ^= a; d = __funnelshift_l(d, d, 16);
    c += d; b ^= c; b = __funnelshift_l(b, b, 12);
    a += b; d ^= a; d = __funnelshift_l(d, d, 8);
    c += d; b ^= c; b = __funnelshift_l(b, b, 7);
}

struct ChaCha8Draws {
    uint32_t key[8];
    uint32_t x[16];
    uint64_t blk;
    __device__ explicit ChaCha8Draws(uint64_t seed) : blk(~0ull) {
        uint64_t s = seed;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            s = s * 6364136223846793005ull + 11634580027462260723ull;
            const uint32_t xs = (uint32_t)(((s >> 18) ^ s) >> 27);
            key[j] = __funnelshift_r(xs, xs, (uint32_t)(s >> 59));
        }
    }
    __device__ void refill() {
        const uint32_t in[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u, key[0], key[1], key[2], key[3],
                                 key[4], key[5], key[6], key[7], (uint32_t)blk, (uint32_t)(blk >> 32), 0u, 0u};
#pragma unroll
        for (int i = 0; i < 16; ++i) x[i] = in[i];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            chacha_quarter(x[0], x[4], x[8], x[12]);
            chacha_quarter(x[1], x[5], x[9], x[13]);
            chacha_quarter(x[2], x[6], x[10], x[14]);
            chacha_quarter(x[3], x[7], x[11], x[15]);
            chacha_quarter(x[0], x[5], x[10], x[15]);
            chacha_quarter(x[1], x[6], x[11], x[12]);
            chacha_quarter(x[2], x[7], x[8], x[13]);
            chacha_quarter(x[3], x[4], x[9], x[14]);
        }
#pragma unroll
        for (int i = 0; i < 16; ++i) x[i] += in[i];
    }
    __device__ uint64_t at(uint64_t ctr) {
        if ((ctr >> 3) != blk) {
            blk = ctr >> 3;
            refill();
        }
        return word((int)(ctr & 7));
    }
    // output j (0..7) of the block in registers
    __device__ uint64_t word(int j) const {
        uint32_t lo = x[0], hi = x[1];
#pragma unroll
        for (int w = 1; w < 8; ++w)
            if (w == j) {
                lo = x[2 * w];
                hi = x[2 * w + 1];
            }
        return (uint64_t)lo | ((uint64_t)hi << 32);
    }
};

__device__ __forceinline__ uint32_t code_at(const uint8_t* row, uint64_t s) {
    return (row[s >> 2] >> ((s & 3) * 2)) & 3u;
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// f = W_i . h (h in shared memory, k <= KM)
template <int KM>
__device__ __forceinline__ float fill_dot(const float* __restrict__ Wi, const float* h, int k) {
    float f = 0.f;
#pragma unroll
    for (int c = 0; c < KM; ++c)
        if (c < k) f = fmaf(Wi[c], h[c], f);
    return f;
}

// Per-SNP statistics with the NMF values at the missing calls: every call is
// valid, mu = (S1 + F1) / n, s = scale(mu), TSS = s^2 (S2 + F2 - (S1+F1)^2/n)
// (decode_single_snp with a fill, src/bed.rs:300-379).  One warp per SNP.
template <int KM>
__global__ void __launch_bounds__(256) k_fill_stats(uint64_t p, uint64_t n, int norm, const int32_t* __restrict__ counts,
                                                    const uint64_t* __restrict__ ptr, const uint32_t* __restrict__ idx,
                                                    const float* __restrict__ W, const float* __restrict__ H, int k,
                                                    double* __restrict__ mean, double* __restrict__ scale,
                                                    double* __restrict__ tss, uint8_t* __restrict__ zero_var) {
    __shared__ float hs[8][KM];
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    const uint64_t nw = (uint64_t)gridDim.x * 8;
    for (uint64_t r = (uint64_t)blockIdx.x * 8 + wl; r < p; r += nw) {
        __syncwarp();
        if (lane < k) hs[wl][lane] = H[r * k + lane];
        __syncwarp();
        double f1 = 0.0, f2 = 0.0;
        for (uint64_t e = ptr[r] + lane; e < ptr[r + 1]; e += 32) {
            const float f = fill_dot<KM>(W + (uint64_t)idx[e] * k, hs[wl], k);
            f1 += (double)f;
            f2 += (double)f * (double)f;
        }
        f1 = warp_sum_d(f1);
        f2 = warp_sum_d(f2);
        if (lane == 0) {
            const int64_t c1 = counts[r * 4 + 1], c2 = counts[r * 4 + 2];
            const double s1 = (double)(c1 + 2 * c2) + f1, s2 = (double)(c1 + 4 * c2) + f2;
            const double mu = n > 0 ? s1 / (double)n : 0.0;
            const double sc = scale_from_mean(mu, norm);
            const double css = n > 0 ? fmax(s2 - s1 * s1 / (double)n, 0.0) : 0.0;
            mean[r] = mu;
            scale[r] = sc;
            tss[r] = sc * sc * css;
            zero_var[r] = (sc == 0.0 || !(css > 0.0)) ? 1 : 0;
        }
    }
}

// One round of a correction: add d_t * op[row_t, c] over the round's `cnt`
// (row, d) pairs held by lanes 0..cnt-1.  For operands of width w <= CG
// (CG = 8, 16, 32) the warp splits into 32/CG groups that take different
// entries (lane = group * CG + column); CG = 0 is the wide form (one entry per
// step, columns lane + 32 q, w <= 128).  Steps are unrolled so several
// gathers are in flight.
template <int CG>
__device__ __forceinline__ void round_accum(float (&acc)[4], uint32_t my, float dm, int cnt, const float* __restrict__ op,
                                            int ldop, int w, int lane) {
    if constexpr (CG == 0) {
#pragma unroll 4
        for (int t = 0; t < 32; ++t) {
            if (t >= cnt) break;
            const uint64_t r = __shfl_sync(0xffffffffu, my, t);
            const float d = __shfl_sync(0xffffffffu, dm, t);
            const float* row = op + r * ldop;
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (lane + 32 * q < w) acc[q] = fmaf(d, row[lane + 32 * q], acc[q]);
        }
    } else {
        constexpr int EPI = 32 / CG;
        const int e = lane / CG, c = lane % CG;
#pragma unroll 4
        for (int t = 0; t < 32; t += EPI) {
            if (t >= cnt) break;
            const int te = t + e;
            const uint64_t r = __shfl_sync(0xffffffffu, my, te & 31);
            const float d = __shfl_sync(0xffffffffu, dm, te & 31);
            if (te < cnt && c < w) acc[0] = fmaf(d, op[r * ldop + c], acc[0]);
        }
    }
}

// after the rounds: column c's total in lane c (narrow form) / lane + 32 q (wide)
template <int CG>
__device__ __forceinline__ void round_finish(float (&acc)[4]) {
    if constexpr (CG != 0) {
#pragma unroll
        for (int off = CG; off < 32; off <<= 1) acc[0] += __shfl_xor_sync(0xffffffffu, acc[0], off);
    }
}

// Row pass correction: out[r, c] += s_r * sum_{i in miss(r)} (f_ir - mu_r) Wop[i, c]
// (the base pass counted the missing calls at the mean).  One warp per SNP;
// 32 missing indices and their fills are formed per round and broadcast.
template <int CG, bool W4, int KM>
__global__ void __launch_bounds__(256) k_fill_row_correct(float* __restrict__ out, int ldo, uint64_t p, int w,
                                                          const uint64_t* __restrict__ ptr,
                                                          const uint32_t* __restrict__ idx, const float* __restrict__ Wop,
                                                          int ldw, const float* __restrict__ Wn,
                                                          const float* __restrict__ H, int k,
                                                          const double* __restrict__ mean,
                                                          const double* __restrict__ scale) {
    __shared__ float hs[8][KM];
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    const uint64_t nw = (uint64_t)gridDim.x * 8;
    for (uint64_t r = (uint64_t)blockIdx.x * 8 + wl; r < p; r += nw) {
        __syncwarp();
        if (lane < k) hs[wl][lane] = H[r * k + lane];
        __syncwarp();
        const uint64_t e0 = ptr[r], e1 = ptr[r + 1];
        if (e0 == e1) continue;
        const float mu = (float)mean[r], sc = (float)scale[r];
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        for (uint64_t b = e0; b < e1; b += 32) {
            uint32_t my = 0;
            float dm = 0.f;
            if (b + lane < e1) {
                my = idx[b + lane];
                float f = 0.f;
                if constexpr (W4) {  // 16-byte loads of the W row, summed in fill_dot's order
                    const float4* w4 = reinterpret_cast<const float4*>(Wn + (uint64_t)my * k);
#pragma unroll
                    for (int q = 0; q < KM / 4; ++q) {
                        if (4 * q < k) {
                            const float4 v = w4[q];
                            f = fmaf(v.x, hs[wl][4 * q], f);
                            f = fmaf(v.y, hs[wl][4 * q + 1], f);
                            f = fmaf(v.z, hs[wl][4 * q + 2], f);
                            f = fmaf(v.w, hs[wl][4 * q + 3], f);
                        }
                    }
                } else {
                    f = fill_dot<KM>(Wn + (uint64_t)my * k, hs[wl], k);
                }
                dm = f - mu;
            }
            round_accum<CG>(acc, my, dm, (int)(e1 - b < 32 ? e1 - b : 32), Wop, ldw, w, lane);
        }
        round_finish<CG>(acc);
        float* o = out + r * ldo;
        if constexpr (CG == 0) {
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (lane + 32 * q < w) o[lane + 32 * q] += sc * acc[q];
        } else {
            if (lane < w) o[lane] += sc * acc[0];
        }
    }
}

// Column pass correction: S[i, c] += sum_{r in miss(i)} s_r (f_ir - mu_r) Qop[r, c].
// Per-sample lists can be long (thousands of calls), so each list is cut into
// segments of kColSeg calls, one warp per (sample, segment), and the segment
// sums are added into S with FP64 atomics.
constexpr uint64_t kColSeg = 1024;
// sm[r] = (s_r, mu_r) in FP32 (the values the correction uses), one 8-byte
// gather per call; with H4 the H row (k % 4 == 0, 16-byte aligned) is read as
// 16-byte loads, the products summed in the same order as fill_dot.
template <int CG, bool H4, int KM>
__global__ void __launch_bounds__(256) k_fill_col_correct(double* __restrict__ S, int lds, uint64_t n, int w,
                                                          uint64_t nseg, const uint64_t* __restrict__ cptr,
                                                          const uint32_t* __restrict__ cidx,
                                                          const float* __restrict__ Qop, int ldq,
                                                          const float* __restrict__ Wn, const float* __restrict__ H,
                                                          int k, const float2* __restrict__ sm) {
    __shared__ float ws[8][KM];
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    const uint64_t nw = (uint64_t)gridDim.x * 8;
    for (uint64_t gw = (uint64_t)blockIdx.x * 8 + wl; gw < n * nseg; gw += nw) {
        const uint64_t i = gw / nseg, sg = gw - i * nseg;
        const uint64_t e0 = cptr[i] + sg * kColSeg, e1 = min(cptr[i + 1], e0 + kColSeg);
        if (e0 >= e1) continue;
        __syncwarp();
        if (lane < k) ws[wl][lane] = Wn[i * k + lane];
        __syncwarp();
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        for (uint64_t b = e0; b < e1; b += 32) {
            uint32_t my = 0;
            float dm = 0.f;
            if (b + lane < e1) {
                my = cidx[b + lane];
                float f = 0.f;
                if constexpr (H4) {
                    const float4* h4 = reinterpret_cast<const float4*>(H + (uint64_t)my * k);
#pragma unroll
                    for (int q = 0; q < KM / 4; ++q) {
                        if (4 * q < k) {
                            const float4 v = h4[q];
                            f = fmaf(v.x, ws[wl][4 * q], f);
                            f = fmaf(v.y, ws[wl][4 * q + 1], f);
                            f = fmaf(v.z, ws[wl][4 * q + 2], f);
                            f = fmaf(v.w, ws[wl][4 * q + 3], f);
                        }
                    }
                } else {
                    f = fill_dot<KM>(H + (uint64_t)my * k, ws[wl], k);
                }
                const float2 smv = sm[my];
                dm = smv.x * (f - smv.y);
            }
            round_accum<CG>(acc, my, dm, (int)(e1 - b < 32 ? e1 - b : 32), Qop, ldq, w, lane);
        }
        round_finish<CG>(acc);
        double* o = S + i * lds;
        if constexpr (CG == 0) {
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (lane + 32 * q < w) atomicAdd(o + lane + 32 * q, (double)acc[q]);
        } else {
            if (lane < w) atomicAdd(o + lane, (double)acc[0]);
        }
    }
}

// out[r, c] += mu_r cs_c: a centred pass (missing at the mean) turned into the
// raw mean-filled product (MeanRaw, src/parallel.rs:53-71)
__global__ void k_add_mean_colsum(float* __restrict__ out, int ldo, uint64_t p, int w,
                                  const double* __restrict__ mean, const double* __restrict__ cs) {
    const uint64_t total = p * (uint64_t)w;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < total;
         e += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t r = e / w;
        const int c = (int)(e - r * w);
        out[r * ldo + c] = (float)((double)out[r * ldo + c] + mean[r] * cs[c]);
    }
}

// Multiplicative update (src/nmf.rs:150-230): X <- X num / denom where
// denom > eps, then X <- max(X, eps).  X, denom: m x k (FP64); num: ld ldn.
template <typename TN>
__global__ void k_nmf_update(double* __restrict__ X, uint64_t m, int k, const TN* __restrict__ num, int ldn,
                             const double* __restrict__ denom, double eps) {
    const uint64_t total = m * (uint64_t)k;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < total;
         e += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t r = e / k;
        const int c = (int)(e - r * k);
        double x = X[e];
        const double dn = denom[e];
        if (dn > eps) x = x * ((double)num[r * ldn + c] / dn);
        X[e] = fmax(x, eps);
    }
}

// normalize_w (src/nmf.rs:259-271): W[:, j] /= ||W[:, j]||_1 and
// H[:, j] *= ||W[:, j]||_1 for columns whose L1 norm (W >= 0) exceeds eps
__global__ void k_nmf_normalize(double* __restrict__ W, uint64_t n, double* __restrict__ H, uint64_t p, int k,
                                const double* __restrict__ colsum, double eps) {
    const uint64_t total = (n + p) * (uint64_t)k;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < total;
         e += (uint64_t)gridDim.x * blockDim.x) {
        const int c = (int)(e % k);
        const double cs = colsum[c];
        if (!(cs > eps)) continue;
        if (e < n * (uint64_t)k) W[e] *= 1.0 / cs;
        else H[e - n * (uint64_t)k] *= cs;
    }
}

// X <- |X| (mode 0) or max(X, 0) (mode 1), FP64, with an optional FP32
// source (ld ldsrc) copied into the m x k destination first
template <typename TS>
__global__ void k_nmf_sign(const TS* __restrict__ src, int ldsrc, double* __restrict__ X, uint64_t m, int k,
                           int mode) {
    const uint64_t total = m * (uint64_t)k;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < total;
         e += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t r = e / k;
        const int c = (int)(e - r * k);
        const double v = (double)src[r * ldsrc + c];
        X[e] = mode == 0 ? fabs(v) : fmax(v, 0.0);
    }
}

// Estimation-phase CV (compute_cv_error_masked, src/nmf.rs:379-455).  Chunk
// `seq` of `chunk` SNPs uses the stream of mask_seed + seq (the counter
// stream, or ChaCha8 with kChaCha); entry (i, r) draws counter
// (r - chunk start) n + i (column-major, missing calls included) and is held
// out iff the draw is below `rate` and the call is observed.  Per SNP:
// sum |g - W_i.H_r|, sum |g - mean_r|, count.
template <bool kChaCha, int KM>
__global__ void __launch_bounds__(256) k_nmf_cv(const uint8_t* __restrict__ packed, uint64_t stride, uint64_t n,
                                                uint64_t p, uint64_t chunk, uint64_t mask_seed, uint64_t thresh,
                                                const float* __restrict__ W, const float* __restrict__ H, int k,
                                                const int32_t* __restrict__ counts, double* __restrict__ part) {
    __shared__ float hs[8][KM];
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    const uint64_t nw = (uint64_t)gridDim.x * 8;
    for (uint64_t r = (uint64_t)blockIdx.x * 8 + wl; r < p; r += nw) {
        __syncwarp();
        if (lane < k) hs[wl][lane] = H[r * k + lane];
        __syncwarp();
        const uint64_t seq = r / chunk, col = r - seq * chunk;
        const uint64_t key = mix64(mask_seed + seq + kGamma);
        ChaCha8Draws cc(mask_seed + seq);
        const int64_t c0 = counts[r * 4], c1 = counts[r * 4 + 1], c2 = counts[r * 4 + 2];
        const int64_t nobs = c0 + c1 + c2;
        const double cm = nobs > 0 ? (double)(c1 + 2 * c2) / (double)nobs : 0.0;
        // a lane takes the 16 codes of one 32-bit word at a time; the draw
        // input key + (ctr + 1) gamma of consecutive samples differs by gamma
        const uint32_t* row = reinterpret_cast<const uint32_t*>(packed + r * stride);
        const uint64_t nwords = (n + 15) / 16;
        double e1 = 0.0, e2 = 0.0, cnt = 0.0;
        auto held_out = [&](uint64_t i, uint32_t code) {
            const double g = code == 0 ? 0.0 : (double)(code - 1);
            e1 += fabs(g - (double)fill_dot<KM>(W + i * k, hs[wl], k));
            e2 += fabs(g - cm);
            cnt += 1.0;
        };
        for (uint64_t wd = lane; wd < nwords; wd += 32) {
            const uint32_t v = row[wd];
            const uint64_t i0 = wd * 16;
            const int nb = n - i0 < 16 ? (int)(n - i0) : 16;
            if constexpr (kChaCha) {
                // the word's entries use the blocks e0 / 8 .. (e0 + nb - 1) / 8;
                // every lane refills at the same points (e0 is the same modulo
                // 8 for all lanes of the SNP), so the refills do not diverge
                const uint64_t e0 = col * n + i0, last = (e0 + nb - 1) >> 3;
                for (uint64_t bk = e0 >> 3; bk <= last; ++bk) {
                    cc.blk = bk;
                    cc.refill();
                    const int lo = bk * 8 > e0 ? (int)(bk * 8 - e0) : 0;
                    const int hi = min(nb, (int)((bk + 1) * 8 - e0));
                    for (int b = lo; b < hi; ++b) {
                        const uint32_t code = (v >> (2 * b)) & 3u;
                        if (code == 1u || (cc.word((int)((e0 + b) & 7)) >> 12) >= thresh) continue;
                        held_out(i0 + b, code);
                    }
                }
            } else {
                uint64_t z = key + (col * n + i0 + 1) * kGamma;
                for (int b = 0; b < nb; ++b, z += kGamma) {
                    const uint32_t code = (v >> (2 * b)) & 3u;
                    if (code == 1u || (mix64(z) >> 11) >= thresh) continue;
                    held_out(i0 + b, code);
                }
            }
        }
        e1 = warp_sum_d(e1);
        e2 = warp_sum_d(e2);
        cnt = warp_sum_d(cnt);
        if (lane == 0) {
            part[r * 3] = e1;
            part[r * 3 + 1] = e2;
            part[r * 3 + 2] = cnt;
        }
    }
}

// Observed calls before each SNP within its chunk (the GWAS-phase CV numbers
// its draws by the rank of the observed call in column-major order)
__global__ void k_obs_base(const int32_t* __restrict__ counts, uint64_t p, uint64_t chunk, uint64_t* __restrict__ base) {
    const uint64_t nchunks = (p + chunk - 1) / chunk;
    for (uint64_t b = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; b < nchunks;
         b += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t acc = 0;
        const uint64_t r1 = min(p, (b + 1) * chunk);
        for (uint64_t r = b * chunk; r < r1; ++r) {
            base[r] = acc;
            acc += (uint64_t)(counts[r * 4] + counts[r * 4 + 1] + counts[r * 4 + 2]);
        }
    }
}

// Hold-out draws of the warp's 256 samples i0 .. i0 + 255 with the draws
// laid out so that one ChaCha8 block (eight outputs) serves up to eight of
// them: lane l takes samples i0 + 8 l .. i0 + 8 l + 7, whose observed calls
// (code != 01) have consecutive counters -- `before` (observed calls of the
// SNP's chunk before i0) plus those of the lower lanes, by a warp scan.
// Returns the lane's held-out bits (bit b: sample i0 + 8 l + b) and its 16
// code bits in `codes`; `before` advances past the 256 samples.  The callers
// move the bits back to one sample per lane with shuffles, so their W-row
// loads stay coalesced.
template <bool kChaCha>
__device__ __forceinline__ uint32_t lane_held8(const uint8_t* row, uint64_t n, uint64_t i0, uint64_t& before,
                                               uint64_t key, ChaCha8Draws& cc, uint64_t thresh, uint32_t& codes) {
    const uint64_t ib = i0 + 8 * (uint64_t)(threadIdx.x & 31);
    uint32_t obs = 0;
    codes = 0x5555u;  // past n: "missing", neither observed nor drawn
    if (ib < n) {
        codes = *reinterpret_cast<const uint16_t*>(row + ib / 4);
#pragma unroll
        for (int b = 0; b < 8; ++b)
            if (ib + b < n && ((codes >> (2 * b)) & 3u) != 1u) obs |= 1u << b;
    }
    const int cnt = __popc(obs);
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if ((int)(threadIdx.x & 31) >= o) incl += v;
    }
    const uint64_t c0 = before + (uint64_t)(incl - cnt);
    before += (uint64_t)__shfl_sync(0xffffffffu, incl, 31);
    uint32_t held = 0;
    if constexpr (kChaCha) {
        // at most eight consecutive counters: blocks c0 / 8 and c0 / 8 + 1,
        // computed by every lane together (no divergent refills)
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            cc.blk = (c0 >> 3) + (uint64_t)half;
            cc.refill();
            uint64_t ctr = c0;
#pragma unroll
            for (int b = 0; b < 8; ++b) {
                if (!((obs >> b) & 1u)) continue;
                if ((ctr >> 3) == cc.blk && (cc.word((int)(ctr & 7)) >> 12) < thresh) held |= 1u << b;
                ++ctr;
            }
        }
    } else {
        uint64_t ctr = c0;
        for (int b = 0; b < 8; ++b) {
            if (!((obs >> b) & 1u)) continue;
            if (draw_below(key, ctr, thresh)) held |= 1u << b;
            ++ctr;
        }
    }
    return held;
}

// GWAS-phase CV (src/testing.rs:423-487): per chunk the stream seed + seq,
// one draw per OBSERVED call (counter = its column-major rank in the chunk),
// held out iff the draw is below `rate`; the held-out column is refilled with
// its leave-out mean mu', H = max(0, W+ y~) and the MAE of W_i.H and of mu'
// over the held-out calls accumulate.  W+ y~ = A + mu' B with A = sum over
// kept observed calls of W+_i g, B = sum over missing and held-out calls of
// W+_i.  One warp per SNP, two passes over its codes; the hold-out draws of
// each 256 samples come from lane_held8.  kChaCha draws from the reference's
// ChaCha8 stream instead of the counter stream.
template <bool kChaCha, int KM>
__global__ void __launch_bounds__(256) k_nmf_gwas_cv(const uint8_t* __restrict__ packed, uint64_t stride, uint64_t n,
                                                     uint64_t p, uint64_t chunk, uint64_t seed, uint64_t thresh,
                                                     const float* __restrict__ W, const float* __restrict__ Wpt, int k,
                                                     const uint64_t* __restrict__ base, double* __restrict__ part) {
    __shared__ float hh[8][KM];
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    const uint64_t nw = (uint64_t)gridDim.x * 8;
    for (uint64_t r = (uint64_t)blockIdx.x * 8 + wl; r < p; r += nw) {
        const uint64_t seq = r / chunk;
        const uint64_t key = mix64(seed + seq + kGamma);
        ChaCha8Draws cc(seed + seq);
        const uint8_t* row = packed + r * stride;
        float A[KM], B[KM];
#pragma unroll
        for (int c = 0; c < KM; ++c) A[c] = B[c] = 0.f;
        double s1 = 0.0, nk = 0.0;
        int nmask = 0;
        uint64_t before = base[r];
        for (uint64_t i0 = 0; i0 < n; i0 += 256) {
            uint32_t codes;
            const uint32_t held8 = lane_held8<kChaCha>(row, n, i0, before, key, cc, thresh, codes);
            // the warp's 256 samples in the coalesced layout: sample i0 + 32 j + lane
            for (int j = 0; j < 8; ++j) {
                const uint64_t i = i0 + 32 * (uint64_t)j + lane;
                const int src = 4 * j + (lane >> 3), bit = lane & 7;
                const uint32_t hm = __shfl_sync(0xffffffffu, held8, src);
                const uint32_t cw = __shfl_sync(0xffffffffu, codes, src);
                if (i >= n) continue;
                const uint32_t code = (cw >> (2 * bit)) & 3u;
                const bool held = (hm >> bit) & 1u;
                const float* wp = Wpt + i * k;
                if (code != 1u && !held) {
                    const float g = code == 0 ? 0.f : (float)(code - 1);
                    s1 += (double)g;
                    nk += 1.0;
#pragma unroll
                    for (int c = 0; c < KM; ++c)
                        if (c < k) A[c] = fmaf(wp[c], g, A[c]);
                } else {
#pragma unroll
                    for (int c = 0; c < KM; ++c)
                        if (c < k) B[c] += wp[c];
                }
                nmask += held ? 1 : 0;
            }
        }
        nmask = __reduce_add_sync(0xffffffffu, nmask);
        if (nmask == 0) {
            if (lane == 0) part[r * 3] = part[r * 3 + 1] = part[r * 3 + 2] = 0.0;
            continue;
        }
        s1 = warp_sum_d(s1);
        nk = warp_sum_d(nk);
        const double mu = nk > 0.0 ? s1 / nk : 0.0;
#pragma unroll
        for (int c = 0; c < KM; ++c) {
            if (c < k) {
                const float a = warp_sum_f(A[c]), b = warp_sum_f(B[c]);
                if (lane == 0) hh[wl][c] = fmaxf(a + (float)mu * b, 0.f);
            }
        }
        __syncwarp();
        double e1 = 0.0, e2 = 0.0;
        before = base[r];
        for (uint64_t i0 = 0; i0 < n; i0 += 256) {
            uint32_t codes;
            const uint32_t held8 = lane_held8<kChaCha>(row, n, i0, before, key, cc, thresh, codes);
            for (int j = 0; j < 8; ++j) {
                const uint64_t i = i0 + 32 * (uint64_t)j + lane;
                const int src = 4 * j + (lane >> 3), bit = lane & 7;
                const uint32_t hm = __shfl_sync(0xffffffffu, held8, src);
                const uint32_t cw = __shfl_sync(0xffffffffu, codes, src);
                if (i >= n || !((hm >> bit) & 1u)) continue;
                const uint32_t code = (cw >> (2 * bit)) & 3u;
                const double g = code == 0 ? 0.0 : (double)(code - 1);
                e1 += fabs(g - (double)fill_dot<KM>(W + i * k, hh[wl], k));
                e2 += fabs(g - mu);
            }
        }
        e1 = warp_sum_d(e1);
        e2 = warp_sum_d(e2);
        if (lane == 0) {
            part[r * 3] = e1;
            part[r * 3 + 1] = e2;
            part[r * 3 + 2] = (double)nmask;
        }
        __syncwarp();
    }
}

}  // namespace

// ceil(rate 2^bits): u < rate for u = m 2^-bits iff m < this (bits = 53 for
// the counter stream's uniforms, 52 for the ChaCha8 stream's)
static uint64_t rate_threshold(double rate, int bits = 53) {
    if (!(rate > 0.0)) return 0;
    if (rate >= 1.0) return 1ull << bits;
    return (uint64_t)std::ceil(std::ldexp(rate, bits));
}

void launch_fill_stats(Ctx& c, const Geno& g, int norm, const float* W, const float* H, int k, double* mean,
                       double* scale, double* tss, uint8_t* zero_var) {
    if (!g.p) return;
    SLFMM_REQUIRE(k >= 1 && k <= kMaxNmfK, SLFMM_ERR_BAD_ARG, "NMF rank must be in 1.." + std::to_string(kMaxNmfK));
    if (k <= 16)
        k_fill_stats<16><<<grid_for(c, g.p, 8), 256, 0, c.stream>>>(g.p, g.n, norm, g.counts.get(), g.miss_ptr.get(),
                                                                     g.miss_idx.get(), W, H, k, mean, scale, tss,
                                                                     zero_var);
    else
        k_fill_stats<32><<<grid_for(c, g.p, 8), 256, 0, c.stream>>>(g.p, g.n, norm, g.counts.get(), g.miss_ptr.get(),
                                                                     g.miss_idx.get(), W, H, k, mean, scale, tss,
                                                                     zero_var);
    SLFMM_LAUNCHED(c, "k_fill_stats");
}

// narrow operand group size: the smallest of 8, 16, 32 that holds w, else 0
static int narrow_group(int w) { return w <= 8 ? 8 : w <= 16 ? 16 : w <= 32 ? 32 : 0; }

template <bool W4, int KM>
static void fill_row_correct_launch(Ctx& c, const Geno& g, unsigned grid, float* out, int ldo, int w,
                                    const float* Wop, int ldw, const float* Wn, const float* H, int k,
                                    const double* mean, const double* scale) {
    const uint64_t* mp = g.miss_ptr.get();
    const uint32_t* mi = g.miss_idx.get();
    switch (narrow_group(w)) {
        case 8:
            k_fill_row_correct<8, W4, KM><<<grid, 256, 0, c.stream>>>(out, ldo, g.p, w, mp, mi, Wop, ldw, Wn, H, k, mean,
                                                                  scale);
            break;
        case 16:
            k_fill_row_correct<16, W4, KM><<<grid, 256, 0, c.stream>>>(out, ldo, g.p, w, mp, mi, Wop, ldw, Wn, H, k, mean,
                                                                   scale);
            break;
        case 32:
            k_fill_row_correct<32, W4, KM><<<grid, 256, 0, c.stream>>>(out, ldo, g.p, w, mp, mi, Wop, ldw, Wn, H, k, mean,
                                                                   scale);
            break;
        default:
            k_fill_row_correct<0, W4, KM><<<grid, 256, 0, c.stream>>>(out, ldo, g.p, w, mp, mi, Wop, ldw, Wn, H, k, mean,
                                                                  scale);
    }
}

void launch_fill_row_correct(Ctx& c, const Geno& g, float* out, int ldo, int w, const float* Wop, int ldw,
                             const float* Wn, const float* H, int k, const double* mean, const double* scale) {
    if (!g.p || !w) return;
    SLFMM_REQUIRE(w <= 128 && k >= 1 && k <= kMaxNmfK, SLFMM_ERR_BAD_ARG, "NMF correction shape");
    const unsigned grid = (unsigned)grid_for(c, g.p, 8);
    const bool w4 = k % 4 == 0 && reinterpret_cast<uintptr_t>(Wn) % 16 == 0;
    if (k <= 16) {
        if (w4) fill_row_correct_launch<true, 16>(c, g, grid, out, ldo, w, Wop, ldw, Wn, H, k, mean, scale);
        else fill_row_correct_launch<false, 16>(c, g, grid, out, ldo, w, Wop, ldw, Wn, H, k, mean, scale);
    } else {
        if (w4) fill_row_correct_launch<true, 32>(c, g, grid, out, ldo, w, Wop, ldw, Wn, H, k, mean, scale);
        else fill_row_correct_launch<false, 32>(c, g, grid, out, ldo, w, Wop, ldw, Wn, H, k, mean, scale);
    }
    SLFMM_LAUNCHED(c, "k_fill_row_correct");
}

__global__ void k_scale_mean_f32(const double* __restrict__ mean, const double* __restrict__ scale, uint64_t p,
                                 float2* __restrict__ out) {
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < p; r += (uint64_t)gridDim.x * blockDim.x)
        out[r] = make_float2((float)scale[r], (float)mean[r]);
}

template <bool H4, int KM>
static void fill_col_correct_launch(Ctx& c, const Geno& g, unsigned grid, uint64_t nseg, double* S, int lds, int w,
                                    const float* Qop, int ldq, const float* Wn, const float* H, int k,
                                    const float2* sm) {
    const uint64_t* cp = g.missT_ptr.get();
    const uint32_t* ci = g.missT_idx.get();
    switch (narrow_group(w)) {
        case 8:
            k_fill_col_correct<8, H4, KM><<<grid, 256, 0, c.stream>>>(S, lds, g.n, w, nseg, cp, ci, Qop, ldq, Wn, H, k, sm);
            break;
        case 16:
            k_fill_col_correct<16, H4, KM><<<grid, 256, 0, c.stream>>>(S, lds, g.n, w, nseg, cp, ci, Qop, ldq, Wn, H, k, sm);
            break;
        case 32:
            k_fill_col_correct<32, H4, KM><<<grid, 256, 0, c.stream>>>(S, lds, g.n, w, nseg, cp, ci, Qop, ldq, Wn, H, k, sm);
            break;
        default:
            k_fill_col_correct<0, H4, KM><<<grid, 256, 0, c.stream>>>(S, lds, g.n, w, nseg, cp, ci, Qop, ldq, Wn, H, k, sm);
    }
}

void launch_fill_col_correct(Ctx& c, const Geno& g, double* S, int lds, int w, const float* Qop, int ldq,
                             const float* Wn, const float* H, int k, const double* mean, const double* scale) {
    if (!g.n || !w) return;
    SLFMM_REQUIRE(w <= 128 && k >= 1 && k <= kMaxNmfK, SLFMM_ERR_BAD_ARG, "NMF correction shape");
    const uint64_t nseg = std::max<uint64_t>(1, ceil_div(g.missT_max, kColSeg));
    const unsigned grid = (unsigned)grid_for(c, g.n * nseg, 8);
    DBuf<float2> sm(std::max<uint64_t>(g.p, 1), c.stream);
    k_scale_mean_f32<<<grid_for(c, g.p, 256), 256, 0, c.stream>>>(mean, scale, g.p, sm.get());
    SLFMM_LAUNCHED(c, "k_scale_mean_f32");
    const bool h4 = k % 4 == 0 && reinterpret_cast<uintptr_t>(H) % 16 == 0;
    if (k <= 16) {
        if (h4) fill_col_correct_launch<true, 16>(c, g, grid, nseg, S, lds, w, Qop, ldq, Wn, H, k, sm.get());
        else fill_col_correct_launch<false, 16>(c, g, grid, nseg, S, lds, w, Qop, ldq, Wn, H, k, sm.get());
    } else {
        if (h4) fill_col_correct_launch<true, 32>(c, g, grid, nseg, S, lds, w, Qop, ldq, Wn, H, k, sm.get());
        else fill_col_correct_launch<false, 32>(c, g, grid, nseg, S, lds, w, Qop, ldq, Wn, H, k, sm.get());
    }
    SLFMM_LAUNCHED(c, "k_fill_col_correct");
}

void launch_add_mean_colsum(Ctx& c, float* out, int ldo, uint64_t p, int w, const double* mean, const double* cs) {
    if (!p || !w) return;
    k_add_mean_colsum<<<grid_for(c, p * w, 256), 256, 0, c.stream>>>(out, ldo, p, w, mean, cs);
    SLFMM_LAUNCHED(c, "k_add_mean_colsum");
}

void launch_nmf_update_f64(Ctx& c, double* X, uint64_t m, int k, const double* num, int ldn, const double* denom,
                           double eps) {
    if (!m) return;
    k_nmf_update<double><<<grid_for(c, m * k, 256), 256, 0, c.stream>>>(X, m, k, num, ldn, denom, eps);
    SLFMM_LAUNCHED(c, "k_nmf_update");
}

void launch_nmf_update_f32(Ctx& c, double* X, uint64_t m, int k, const float* num, int ldn, const double* denom,
                           double eps) {
    if (!m) return;
    k_nmf_update<float><<<grid_for(c, m * k, 256), 256, 0, c.stream>>>(X, m, k, num, ldn, denom, eps);
    SLFMM_LAUNCHED(c, "k_nmf_update");
}

void launch_nmf_normalize(Ctx& c, double* W, uint64_t n, double* H, uint64_t p, int k, const double* colsum,
                          double eps) {
    k_nmf_normalize<<<grid_for(c, (n + p) * k, 256), 256, 0, c.stream>>>(W, n, H, p, k, colsum, eps);
    SLFMM_LAUNCHED(c, "k_nmf_normalize");
}

void launch_nmf_abs_f64(Ctx& c, const double* src, int ld, double* X, uint64_t m, int k) {
    if (!m) return;
    k_nmf_sign<double><<<grid_for(c, m * k, 256), 256, 0, c.stream>>>(src, ld, X, m, k, 0);
    SLFMM_LAUNCHED(c, "k_nmf_sign");
}

void launch_nmf_clamp0_f32(Ctx& c, const float* src, int ld, double* X, uint64_t m, int k) {
    if (!m) return;
    k_nmf_sign<float><<<grid_for(c, m * k, 256), 256, 0, c.stream>>>(src, ld, X, m, k, 1);
    SLFMM_LAUNCHED(c, "k_nmf_sign");
}

void launch_nmf_cv(Ctx& c, const Geno& g, uint64_t chunk, uint64_t mask_seed, double rate, const float* W,
                   const float* H, int k, double* part) {
    if (!g.p) return;
    const bool cc = c.rng == SLFMM_RNG_CHACHA8;
    const uint64_t th = cc ? rate_threshold(rate, 52) : rate_threshold(rate);
    const unsigned grid = (unsigned)grid_for(c, g.p, 8);
    auto go = [&](auto kern) {
        kern<<<grid, 256, 0, c.stream>>>(packed_rows(g), g.stride, g.n, g.p, chunk, mask_seed, th, W, H, k,
                                         g.counts.get(), part);
    };
    if (k <= 16) {
        if (cc) go(k_nmf_cv<true, 16>);
        else go(k_nmf_cv<false, 16>);
    } else {
        if (cc) go(k_nmf_cv<true, 32>);
        else go(k_nmf_cv<false, 32>);
    }
    SLFMM_LAUNCHED(c, "k_nmf_cv");
}

void launch_nmf_gwas_cv(Ctx& c, const Geno& g, uint64_t chunk, uint64_t seed, double rate, const float* W,
                        const float* Wpt, int k, double* part) {
    if (!g.p) return;
    DBuf<uint64_t> base(g.p, c.stream);
    const uint64_t nchunks = ceil_div(g.p, chunk);
    k_obs_base<<<grid_for(c, nchunks, 64), 64, 0, c.stream>>>(g.counts.get(), g.p, chunk, base.get());
    SLFMM_LAUNCHED(c, "k_obs_base");
    const bool cc = c.rng == SLFMM_RNG_CHACHA8;
    const uint64_t th = cc ? rate_threshold(rate, 52) : rate_threshold(rate);
    const unsigned grid = (unsigned)grid_for(c, g.p, 8);
    auto go = [&](auto kern) {
        kern<<<grid, 256, 0, c.stream>>>(packed_rows(g), g.stride, g.n, g.p, chunk, seed, th, W, Wpt, k, base.get(),
                                         part);
    };
    if (k <= 16) {
        if (cc) go(k_nmf_gwas_cv<true, 16>);
        else go(k_nmf_gwas_cv<false, 16>);
    } else {
        if (cc) go(k_nmf_gwas_cv<true, 32>);
        else go(k_nmf_gwas_cv<false, 32>);
    }
    SLFMM_LAUNCHED(c, "k_nmf_gwas_cv");
}

}  // namespace slfmm
