// tcgen05 tensor-core contraction of the packed genotype matrix.
//
//   P[r, c] = sum_k g(r, k) * W[k, c]        r = tile row, k = K index
//
// g is read straight from the resident 2-bit matrix (rows = SNPs for the
// sketch / backward / association passes, rows = samples on the transposed
// copy for the forward passes) and expanded to exact BF16 {0, 1, 2} (missing
// calls contribute 0; the host applies the mean / scale / missing-call
// corrections afterwards).  W is split hi + lo into two BF16 matrices so the
// product is accurate to ~2^-16 relative with FP32 accumulation; this replaces
// the reference's per-chunk FP64 dgemms (src/rsvd.rs:61-69, :88-97, :117-125,
// :144-153 and src/testing.rs:355-374).
//
// Per CTA: one 128-row tile, a K range of 128-element stages.
//   warp 0      TMA producer: packed codes (128 rows x 32 B) and the two
//               128B-swizzled halves of the W tile (N rows x 64 BF16 each)
//   warp 1      TMEM allocator + single-thread tcgen05.mma issuer
//   warps 2-5   expand codes -> BF16 pairs -> tcgen05.st into TMEM (the A
//               operand lives in TMEM, so shared memory only carries W),
//               then the epilogue: tcgen05.ld, hi + lo, store FP32
// Every mbarrier wait is bounded by the global timer; on expiry the CTA
// records an error code, drains its own TMA loads, frees TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include "fp_convert.cuh"
#include "slfmm_internal.h"
#include "tc_common.cuh"

namespace slfmm {
namespace {
using namespace tc;

constexpr int kM = 128;                      // tile rows = TMEM lanes
constexpr int kKB = 128;                     // K elements per stage
constexpr int kPackedStage = kM * kKB / 4;   // 4096 B of 2-bit codes
constexpr int kThreads = 192;

struct TcArgs {
    uint32_t rows;          // valid tile rows in the matrix
    uint32_t kb_total;      // K stages in the matrix
    uint32_t kb_per_split;  // K stages per grid.y split
    uint32_t wpad;          // output columns; MMA N = 2 * wpad
    uint32_t stages;        // pipeline depth
    uint32_t tmem_cols;     // TMEM columns allocated
    uint32_t a_col0;        // first TMEM column of the A stages
    uint32_t b_stage_bytes; // 2 * N * 128
    float* out;
    uint32_t ldo;
    uint64_t split_stride;  // elements between split outputs
    int* err;
};

__device__ __forceinline__ uint32_t bf16_of_code(uint32_t c) {
    return c == 2u ? 0x3F80u : (c == 3u ? 0x4000u : 0u);  // 00 -> 0, 01 (missing) -> 0
}

__global__ void __launch_bounds__(kThreads, 1)
    k_tc_rows(const __grid_constant__ CUtensorMap tm_packed, const __grid_constant__ CUtensorMap tm_b, TcArgs a) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const uint32_t S = a.stages, N = 2 * a.wpad;
    uint8_t* bsm = smem;
    uint8_t* psm = bsm + S * a.b_stage_bytes;
    uint2* lut = reinterpret_cast<uint2*>(psm + S * kPackedStage);
    uint64_t* bars = reinterpret_cast<uint64_t*>(reinterpret_cast<uint8_t*>(lut) + 256 * sizeof(uint2));
    uint64_t* full_tma = bars;
    uint64_t* full_a = bars + S;
    uint64_t* empty = bars + 2 * S;
    uint64_t* tmem_full = bars + 3 * S;
    uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(bars + 3 * S + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t row0 = blockIdx.x * kM;
    const uint32_t kb0 = blockIdx.y * a.kb_per_split;
    const uint32_t kb1 = min(a.kb_total, kb0 + a.kb_per_split);
    const uint32_t nkb = kb1 > kb0 ? kb1 - kb0 : 0;

    if (threadIdx.x == 0) {
        for (uint32_t s = 0; s < S; ++s) {
            mbar_init(full_tma + s, 1);
            mbar_init(full_a + s, 128);
            mbar_init(empty + s, 1);
        }
        mbar_init(tmem_full, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_holder)),
                     "r"(a.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    for (int e = threadIdx.x; e < 256; e += blockDim.x) {
        uint2 v;
        v.x = bf16_of_code(e & 3) | (bf16_of_code((e >> 2) & 3) << 16);
        v.y = bf16_of_code((e >> 4) & 3) | (bf16_of_code((e >> 6) & 3) << 16);
        lut[e] = v;
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_holder;

    if (warp == 0) {
        if (lane == 0) {
            uint32_t issued = 0;
            for (uint32_t i = 0; i < nkb; ++i) {
                const uint32_t s = i % S, r = i / S;
                if (r > 0 && !mbar_wait(empty + s, (r - 1) & 1, a.err, 1)) break;
                mbar_arrive_tx(full_tma + s, kPackedStage + a.b_stage_bytes);
                const int kb = (int)(kb0 + i);
                tma_2d(psm + s * kPackedStage, &tm_packed, kb * (kKB / 4), (int)row0, full_tma + s);
                tma_2d(bsm + s * a.b_stage_bytes, &tm_b, kb * kKB, 0, full_tma + s);
                tma_2d(bsm + s * a.b_stage_bytes + N * 128, &tm_b, kb * kKB + 64, 0, full_tma + s);
                issued = i + 1;
            }
            // never leave with loads in flight into this CTA's shared memory
            for (uint32_t i = issued > S ? issued - S : 0; i < issued; ++i)
                mbar_wait(full_tma + i % S, (i / S) & 1, a.err, 2);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = instr_desc(N);
            for (uint32_t i = 0; i < nkb; ++i) {
                const uint32_t s = i % S, r = i / S;
                if (!mbar_wait(full_tma + s, r & 1, a.err, 3)) break;
                if (!mbar_wait(full_a + s, r & 1, a.err, 4)) break;
                fence_after();
                const uint32_t b_base = smem_u32(bsm + s * a.b_stage_bytes);
                const uint32_t a_base = tmem + a.a_col0 + s * (kKB / 2);
#pragma unroll
                for (int kk = 0; kk < kKB / 16; ++kk) {
                    const uint64_t bd = smem_desc(b_base + (kk >> 2) * (N * 128) + (kk & 3) * 32);
                    mma_ts(tmem, a_base + kk * 8, bd, idesc, (i > 0 || kk > 0) ? 1u : 0u);
                }
                mma_commit(empty + s);
            }
            mma_commit(tmem_full);
        }
    } else {
        const uint32_t q = (uint32_t)warp & 3u;          // TMEM sub-partition of this warp
        const uint32_t row = q * 32 + lane;              // tile row == TMEM lane
        const uint32_t lane_base = tmem + ((q * 32) << 16);
        for (uint32_t i = 0; i < nkb; ++i) {
            const uint32_t s = i % S, r = i / S;
            // warp-uniform decisions: the tcgen05.st below is .sync.aligned
            if (!__all_sync(0xffffffffu, r == 0 || mbar_wait(empty + s, (r - 1) & 1, a.err, 5))) break;
            if (!__all_sync(0xffffffffu, mbar_wait(full_tma + s, r & 1, a.err, 6))) break;
            const uint4* src = reinterpret_cast<const uint4*>(psm + s * kPackedStage + row * (kKB / 4));
            const uint4 p0 = src[0], p1 = src[1];
            const uint32_t w8[8] = {p0.x, p0.y, p0.z, p0.w, p1.x, p1.y, p1.z, p1.w};
            uint32_t v[64];
#pragma unroll
            for (int b = 0; b < 32; ++b) {
                const uint2 e = lut[(w8[b >> 2] >> (8 * (b & 3))) & 0xffu];
                v[2 * b] = e.x;
                v[2 * b + 1] = e.y;
            }
            tmem_st_x64(lane_base + a.a_col0 + s * (kKB / 2), v);
            asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
            fence_before();
            mbar_arrive(full_a + s);
        }
        // epilogue: D[row, c] + D[row, wpad + c]
        const bool ok = __all_sync(0xffffffffu, mbar_wait(tmem_full, 0, a.err, 7));
        fence_after();
        const uint32_t grow = row0 + row;
        float* dst = a.out + (uint64_t)blockIdx.y * a.split_stride + (uint64_t)grow * a.ldo;
        for (uint32_t c0 = 0; c0 < a.wpad; c0 += 16) {
            float hi[16], lo[16];
            tmem_ld_x16(lane_base + c0, hi);
            tmem_ld_x16(lane_base + a.wpad + c0, lo);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (ok && grow < a.rows) {
                float4* d4 = reinterpret_cast<float4*>(dst + c0);
#pragma unroll
                for (int t = 0; t < 4; ++t)
                    d4[t] = make_float4(hi[4 * t] + lo[4 * t], hi[4 * t + 1] + lo[4 * t + 1],
                                        hi[4 * t + 2] + lo[4 * t + 2], hi[4 * t + 3] + lo[4 * t + 3]);
            }
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 1) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(a.tmem_cols)
                     : "memory");
    }
}

// W (K x w, row-major, FP32 or FP64, optional per-row scale) -> two BF16
// matrices hi, lo stored as [2 * wpad][K_pad] (K contiguous), zero padded.
template <typename T>
__global__ void k_split_bf16(const T* __restrict__ src, int ld, uint64_t K, int w, int wpad, uint64_t K_pad,
                             const double* __restrict__ kscale, __nv_bfloat16* __restrict__ dst) {
    __shared__ float tile[64][33];
    const uint64_t k0 = (uint64_t)blockIdx.x * 64;
    const int c0 = blockIdx.y * 32;
    for (int e = threadIdx.x; e < 64 * 32; e += blockDim.x) {
        const int kk = e / 32, cc = e % 32;
        const uint64_t k = k0 + kk;
        const int c = c0 + cc;
        float v = 0.f;
        if (k < K && c < w) {
            double x = (double)src[k * ld + c];
            if (kscale) x *= kscale[k];
            v = (float)x;
        }
        tile[kk][cc] = v;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 64 * 32; e += blockDim.x) {
        const int cc = e / 64, kk = e % 64;
        const int c = c0 + cc;
        if (c >= wpad) continue;
        const uint64_t k = k0 + kk;
        if (k >= K_pad) continue;
        const float v = tile[kk][cc];
        const __nv_bfloat16 hi = __float2bfloat16_rn(v);
        const __nv_bfloat16 lo = __float2bfloat16_rn(v - __bfloat162float(hi));
        dst[(uint64_t)c * K_pad + k] = hi;
        dst[(uint64_t)(wpad + c) * K_pad + k] = lo;
    }
}

// Transposed 2-bit matrix: row i (sample) holds the codes of every SNP.
__global__ void k_transpose_packed(const uint8_t* __restrict__ in, uint64_t p, uint64_t stride, uint64_t n,
                                   uint8_t* __restrict__ out, uint64_t strideT) {
    __shared__ uint8_t tile[128][33];
    const uint64_t j0 = (uint64_t)blockIdx.x * 128;  // SNPs
    const uint64_t i0 = (uint64_t)blockIdx.y * 128;  // samples
    for (int e = threadIdx.x; e < 128 * 32; e += blockDim.x) {
        const int r = e / 32, b = e % 32;
        const uint64_t j = j0 + r;
        tile[r][b] = j < p ? in[j * stride + i0 / 4 + b] : 0;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 128 * 32; e += blockDim.x) {
        const int il = e / 32, bj = e % 32;
        const uint64_t i = i0 + il;
        if (i >= n) continue;
        uint32_t byte = 0;
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const uint32_t code = (tile[bj * 4 + t][il >> 2] >> (2 * (il & 3))) & 3u;
            byte |= code << (2 * t);
        }
        out[i * strideT + j0 / 4 + bj] = (uint8_t)byte;
    }
}

// per-row fix of a row pass (mean imputation):
//   out[j, c] = s_j * (P[j, c] - mu_j * (cs_c - sum_{i in miss_j} W[i, c]))
// One warp per row: indices are fetched 32 at a time and broadcast so the W
// row gathers (L2-resident) are independent and overlap.
__global__ void k_rowfix_mean(float* __restrict__ P, int ldp, uint64_t rows, int w,
                              const uint64_t* __restrict__ ptr, const uint32_t* __restrict__ idx,
                              const float* __restrict__ W, int ldw, const double* __restrict__ cs,
                              const double* __restrict__ mean, const double* __restrict__ scale) {
    const uint64_t j = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32;
    const int lane = threadIdx.x & 31;
    if (j >= rows) return;
    const uint64_t e0 = ptr[j], e1 = ptr[j + 1];
    float acc[4] = {0.f, 0.f, 0.f, 0.f};   // columns lane, lane+32, lane+64, lane+96
    for (uint64_t b = e0; b < e1; b += 32) {
        const uint32_t my = b + lane < e1 ? idx[b + lane] : 0u;
        const int cnt = (int)(e1 - b < 32 ? e1 - b : 32);
#pragma unroll 4
        for (int t = 0; t < cnt; ++t) {
            const uint64_t i = __shfl_sync(0xffffffffu, my, t);
            const float* wr = W + i * ldw;
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (lane + 32 * q < w) acc[q] += wr[lane + 32 * q];
        }
    }
    const double mu = mean[j], sc = scale[j];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int c = lane + 32 * q;
        if (c < w) {
            const double v = (double)P[j * ldp + c] - mu * (cs[c] - (double)acc[q]);
            P[j * ldp + c] = (float)(sc * v);
        }
    }
}

// k_rowfix_mean with 16-byte W-row gathers: a group of L lanes (L = 1, 2,
// 4, 8 or 16, the column quads of the block rounded up) covers one W row,
// lane q of the group column quad q (W rows 16-byte aligned), and the 32 / L
// groups of a warp take consecutive missing calls of the same SNP; their
// partial sums are combined by shuffles at the end.  The gathers are bound by
// L2 latency, so the register cap keeps all 64 warps of an SM resident
// (measured 18 % faster than the 40 warps the uncapped build allows).
template <int L>
__global__ void __launch_bounds__(256, 8) k_rowfix_mean4(float* __restrict__ P, int ldp, uint64_t rows, int w,
                               const uint64_t* __restrict__ ptr, const uint32_t* __restrict__ idx,
                               const float* __restrict__ W, int ldw, const double* __restrict__ cs,
                               const double* __restrict__ mean, const double* __restrict__ scale) {
    constexpr int G = 32 / L;  // missing calls per warp step
    const uint64_t j = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32;
    const int lane = threadIdx.x & 31, q = lane % L, grp = lane / L;
    if (j >= rows) return;
    const bool act = 4 * q < w;
    const uint64_t e0 = ptr[j], e1 = ptr[j + 1];
    // each lane's own column quad of W; a missing call's row offset (in
    // 16-byte units, 32 bits: the launcher checks n x ldw / 4 < 2^32) is
    // formed once per batch by the lane that loaded the call
    const float4* Wq = reinterpret_cast<const float4*>(W) + q;
    const uint32_t q4 = (uint32_t)ldw >> 2;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (uint64_t b = e0; b < e1; b += 32) {
        const uint32_t my = b + lane < e1 ? idx[b + lane] * q4 : 0u;
        const int cnt = (int)(e1 - b < 32 ? e1 - b : 32);
#pragma unroll 4
        for (int t = 0; t < cnt; t += G) {
            const int tt = t + grp;
            const uint32_t off = __shfl_sync(0xffffffffu, my, tt & 31);
            if (act && tt < cnt) {
                const float4 v = Wq[off];
                acc.x += v.x;
                acc.y += v.y;
                acc.z += v.z;
                acc.w += v.w;
            }
        }
    }
#pragma unroll
    for (int o = L; o < 32; o <<= 1) {
        acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
        acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
        acc.z += __shfl_xor_sync(0xffffffffu, acc.z, o);
        acc.w += __shfl_xor_sync(0xffffffffu, acc.w, o);
    }
    if (!act || grp != 0) return;
    // FP32 arithmetic, with the FP64 inputs narrowed by integer operations:
    // P carries the FP32 rounding of its contraction, which the FP64 form of
    // this update did not remove, and FP64 arithmetic here ran the FP64 pipe
    // at 69 % of its peak for the whole kernel
    const float mu = f32_of_f64(mean[j]), sc = f32_of_f64(scale[j]);
    const float a4[4] = {acc.x, acc.y, acc.z, acc.w};
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int c = 4 * q + u;
        if (c < w) {
            const float t = f32_of_f64(cs[c]) - a4[u];
            P[j * ldp + c] = sc * fmaf(-mu, t, P[j * ldp + c]);
        }
    }
}

// per-sample fix of a forward pass on the transposed matrix (mean imputation):
//   S[i, c] += sum_{j in missT_i} coef_j Q[j, c] - colterm_c,  coef_j = mu_j s_j
__global__ void k_colfix_mean(double* __restrict__ S, int lds, uint64_t n, int w,
                              const uint64_t* __restrict__ ptr, const uint32_t* __restrict__ idx,
                              const float* __restrict__ Q, int ldq, const double* __restrict__ coef,
                              const double* __restrict__ colterm) {
    const uint64_t i = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32;
    const int lane = threadIdx.x & 31;
    if (i >= n) return;
    const uint64_t e0 = ptr[i], e1 = ptr[i + 1];
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    for (uint64_t b = e0; b < e1; b += 32) {
        const uint32_t myj = b + lane < e1 ? idx[b + lane] : 0u;
        const float myc = b + lane < e1 ? (float)coef[myj] : 0.f;
        const int cnt = (int)(e1 - b < 32 ? e1 - b : 32);
#pragma unroll 4
        for (int t = 0; t < cnt; ++t) {
            const uint64_t j = __shfl_sync(0xffffffffu, myj, t);
            const float cj = __shfl_sync(0xffffffffu, myc, t);
            const float* qr = Q + j * ldq;
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (lane + 32 * q < w) acc[q] = fmaf(cj, qr[lane + 32 * q], acc[q]);
        }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int c = lane + 32 * q;
        if (c < w) S[i * lds + c] += (double)acc[q] - colterm[c];
    }
}

// out[c] = sum_j coef[j] Q[j, c] (w <= 32 T): block partials, one warp per run
// of rows with the row read whole (lane c, c + 32, ...), four rows in flight.
// T column groups of 32 only: GB300's FP64 rate is low, so no FMA is spent on
// absent columns.
template <int T>
__global__ void __launch_bounds__(256) k_weighted_colsum(const float* __restrict__ Q, int ldq, uint64_t p, int w,
                                                         const double* __restrict__ coef, double* __restrict__ part) {
    __shared__ double red[8][32 * T];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double acc[T];
#pragma unroll
    for (int t = 0; t < T; ++t) acc[t] = 0.0;
    const uint64_t nw = (uint64_t)gridDim.x * 8;
    for (uint64_t j = ((uint64_t)blockIdx.x * 8 + warp) * 4; j < p; j += nw * 4) {
        float q[4][T];
        double cf[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const bool ok = j + u < p;
            cf[u] = ok ? coef[j + u] : 0.0;
#pragma unroll
            for (int t = 0; t < T; ++t) {
                const int cc = lane + 32 * t;
                q[u][t] = (ok && cc < w) ? Q[(j + u) * ldq + cc] : 0.f;
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int t = 0; t < T; ++t) acc[t] = fma(cf[u], (double)q[u][t], acc[t]);
    }
#pragma unroll
    for (int t = 0; t < T; ++t) red[warp][lane + 32 * t] = acc[t];
    __syncthreads();
    for (int cc = threadIdx.x; cc < w; cc += blockDim.x) {
        double s = 0.0;
        for (int ww = 0; ww < 8; ++ww) s += red[ww][cc];
        part[(uint64_t)blockIdx.x * w + cc] = s;
    }
}

// out[c] = sum_j coef[j] Q[j, c] for a narrow operand (w <= ldq <= 32,
// ldq % 4 == 0, 16-byte aligned rows): a thread keeps one 16-byte column quad
// and walks rows, four rows in flight; FP32 products and sums over runs of 64
// of its rows (the precision of the tensor-core sums this term is subtracted
// from), FP64 across runs, lanes and warps; one partial per block.
__global__ void __launch_bounds__(256) k_weighted_colsum_quads(const float* __restrict__ Q, int ldq, uint64_t p,
                                                               int w, const double* __restrict__ coef,
                                                               double* __restrict__ part) {
    const int q = ldq >> 2;  // 1, 2, 4 or 8 quads per row
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x / q;
    const int qp = (int)(tid % q);
    const float4* q4 = reinterpret_cast<const float4*>(Q);
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    float f[4] = {0.f, 0.f, 0.f, 0.f};
    int run = 0;
    for (uint64_t j0 = tid / q; j0 < p; j0 += 4 * step) {
        float4 v[4];
        float cf[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint64_t j = j0 + u * step;
            const bool ok = j < p;
            v[u] = ok ? q4[j * q + qp] : make_float4(0.f, 0.f, 0.f, 0.f);
            cf[u] = ok ? (float)coef[j] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            f[0] = fmaf(cf[u], v[u].x, f[0]);
            f[1] = fmaf(cf[u], v[u].y, f[1]);
            f[2] = fmaf(cf[u], v[u].z, f[2]);
            f[3] = fmaf(cf[u], v[u].w, f[3]);
        }
        if (++run == 16) {
#pragma unroll
            for (int i = 0; i < 4; ++i) acc[i] += (double)f[i], f[i] = 0.f;
            run = 0;
        }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) acc[i] += (double)f[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        if (o < q) break;
#pragma unroll
        for (int i = 0; i < 4; ++i) acc[i] += __shfl_xor_sync(0xffffffffu, acc[i], o);
    }
    __shared__ double red[8][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane < q)
#pragma unroll
        for (int i = 0; i < 4; ++i) red[warp][4 * lane + i] = acc[i];
    __syncthreads();
    if (threadIdx.x < w) {
        double t = 0.0;
        for (int wv = 0; wv < 8; ++wv) t += red[wv][threadIdx.x];
        part[(uint64_t)blockIdx.x * w + threadIdx.x] = t;
    }
}

__global__ void k_scale_product(const double* __restrict__ a, const double* __restrict__ b, uint64_t n,
                                double* __restrict__ out) {
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x)
        out[t] = a[t] * b[t];
}

// -------------------------------------------------------------------------
// host side
// -------------------------------------------------------------------------
// thread-safe one-time lookup (contexts may run on several host threads)
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        SLFMM_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
        SLFMM_REQUIRE(q == cudaDriverEntryPointSuccess && p, SLFMM_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

CUtensorMap map_packed(const uint8_t* base, uint64_t stride, uint64_t rows) {
    CUtensorMap m;
    cuuint64_t dims[2] = {stride, rows};
    cuuint64_t strides[1] = {stride};
    cuuint32_t box[2] = {kKB / 4, kM};
    cuuint32_t es[2] = {1, 1};
    CUresult r = encode_fn()(&m, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<uint8_t*>(base), dims, strides, box, es,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    SLFMM_REQUIRE(r == CUDA_SUCCESS, SLFMM_ERR_CUDA, "tensor map (packed) encode failed: " + std::to_string((int)r));
    return m;
}

CUtensorMap map_bsplit(const __nv_bfloat16* base, uint64_t k_pad, uint32_t n_rows) {
    CUtensorMap m;
    cuuint64_t dims[2] = {k_pad, n_rows};
    cuuint64_t strides[1] = {k_pad * 2};
    cuuint32_t box[2] = {64, n_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = encode_fn()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16*>(base), dims, strides,
                             box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    SLFMM_REQUIRE(r == CUDA_SUCCESS, SLFMM_ERR_CUDA, "tensor map (W) encode failed: " + std::to_string((int)r));
    return m;
}

struct TcPlan {
    uint32_t stages, tmem_cols, a_col0, b_stage_bytes;
    size_t smem;
};

TcPlan plan(uint32_t wpad) {
    const uint32_t N = 2 * wpad;
    TcPlan p;
    p.b_stage_bytes = 2 * N * 128;
    const uint32_t dcols = (uint32_t)round_up(N, 64);
    const size_t fixed = 1024 + 256 * 8 + 64 * 8 + 64;
    const size_t per_stage = p.b_stage_bytes + kPackedStage;
    // two CTAs per SM when the stages fit half of TMEM and shared memory
    uint32_t st2 = std::min<uint32_t>((256 - dcols) / (kKB / 2), (uint32_t)((110 * 1024 - fixed) / per_stage));
    if (dcols < 256 && st2 >= 2) {
        p.stages = std::min<uint32_t>(st2, 4);
        p.tmem_cols = 256;
    } else {
        p.stages = std::min<uint32_t>((512 - dcols) / (kKB / 2), (uint32_t)((220 * 1024 - fixed) / per_stage));
        p.stages = std::min<uint32_t>(p.stages, 6);
        p.tmem_cols = 512;
    }
    p.a_col0 = dcols;
    p.smem = fixed + p.stages * per_stage;
    return p;
}

void check_err(Ctx& c, DBuf<int>& err) {
    int h = 0;
    SLFMM_CUDA(cudaMemcpyAsync(&h, err.get(), sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    SLFMM_CUDA(cudaStreamSynchronize(c.stream));
    if (h != 0)
        throw Error(SLFMM_ERR_DEVICE_TIMEOUT,
                    "tensor-core contraction: a bounded device wait expired (site " + std::to_string(h) + ")");
}

}  // namespace

bool tc_available(Ctx& c) { return c.precision == SLFMM_PREC_SPLIT_BF16; }

void launch_split_bf16_f64(Ctx& c, const double* src, int ld, uint64_t K, int w, int wpad, uint64_t K_pad,
                           const double* kscale, __nv_bfloat16* dst) {
    dim3 grid((unsigned)ceil_div(K_pad, 64), (unsigned)ceil_div(wpad, 32));
    k_split_bf16<double><<<grid, 256, 0, c.stream>>>(src, ld, K, w, wpad, K_pad, kscale, dst);
    SLFMM_LAUNCHED(c, "k_split_bf16");
}

void launch_split_bf16_f32(Ctx& c, const float* src, int ld, uint64_t K, int w, int wpad, uint64_t K_pad,
                           const double* kscale, __nv_bfloat16* dst) {
    dim3 grid((unsigned)ceil_div(K_pad, 64), (unsigned)ceil_div(wpad, 32));
    k_split_bf16<float><<<grid, 256, 0, c.stream>>>(src, ld, K, w, wpad, K_pad, kscale, dst);
    SLFMM_LAUNCHED(c, "k_split_bf16");
}

void build_transposed(Ctx& c, const Geno& g) {
    if (g.have_T) return;
    g.strideT = round_up(ceil_div(g.p, 4), 128);
    g.packedT.alloc(g.n * g.strideT, c.stream);
    SLFMM_CUDA(cudaMemsetAsync(g.packedT.get(), 0, g.n * g.strideT, c.stream));
    dim3 grid((unsigned)ceil_div(g.p, 128), (unsigned)ceil_div(g.n, 128));
    k_transpose_packed<<<grid, 256, 0, c.stream>>>(packed_rows(g), g.p, g.stride, g.n, g.packedT.get(), g.strideT);
    SLFMM_LAUNCHED(c, "k_transpose_packed");
    g.have_T = true;
}

// out (rows x ldo, or splits x rows x ldo) = G^T-style product of the packed
// rows with the split W (B operand [2 wpad][K_pad]).
int launch_tc_rows(Ctx& c, const uint8_t* packed, uint64_t stride, uint64_t rows, uint64_t K,
                    const __nv_bfloat16* bsplit, uint64_t K_pad, int wpad, float* out, int ldo, int splits,
                    uint64_t split_stride) {
    SLFMM_REQUIRE(wpad % 16 == 0 && wpad >= 16 && 2 * wpad <= 256, SLFMM_ERR_BAD_ARG,
                  "tensor-core operand width must be a multiple of 16 in [16, 128]");
    SLFMM_REQUIRE(K_pad % kKB == 0 && K_pad >= ceil_div(K, kKB) * kKB, SLFMM_ERR_BAD_ARG, "bad K padding");
    SLFMM_REQUIRE(stride % 16 == 0 && stride * 4 >= ceil_div(K, kKB) * kKB, SLFMM_ERR_BAD_ARG, "bad packed stride");
    SLFMM_REQUIRE(rows < (1ull << 31), SLFMM_ERR_BAD_ARG, "too many rows");
    const TcPlan pl = plan((uint32_t)wpad);
    raise_dynamic_smem((const void*)k_tc_rows, pl.smem);
    const CUtensorMap tp = map_packed(packed, stride, rows);
    const CUtensorMap tb = map_bsplit(bsplit, K_pad, 2 * wpad);
    DBuf<int> err(1, c.stream);
    err.zero();
    TcArgs a;
    a.rows = (uint32_t)rows;
    a.kb_total = (uint32_t)ceil_div(K, kKB);
    a.kb_per_split = (uint32_t)ceil_div(a.kb_total, (uint64_t)std::max(splits, 1));
    a.wpad = (uint32_t)wpad;
    a.stages = pl.stages;
    a.tmem_cols = pl.tmem_cols;
    a.a_col0 = pl.a_col0;
    a.b_stage_bytes = pl.b_stage_bytes;
    a.out = out;
    a.ldo = (uint32_t)ldo;
    a.split_stride = split_stride;
    a.err = err.get();
    const unsigned gy = (unsigned)ceil_div(a.kb_total, a.kb_per_split);
    dim3 grid((unsigned)ceil_div(rows, kM), gy);
    k_tc_rows<<<grid, kThreads, pl.smem, c.stream>>>(tp, tb, a);
    SLFMM_LAUNCHED(c, "k_tc_rows");
    check_err(c, err);
    return (int)gy;
}

int tc_split_count(Ctx& c, uint64_t rows, uint64_t K) {
    // about eight waves of CTAs so the last wave is a small tail
    const uint64_t tiles = ceil_div(rows, kM);
    const uint64_t kb = ceil_div(K, kKB);
    uint64_t want = ceil_div((uint64_t)c.sm_count * 2 * 8, tiles);
    want = std::max<uint64_t>(1, std::min<uint64_t>(want, std::max<uint64_t>(1, kb / 8)));
    return (int)want;
}

void launch_rowfix_mean(Ctx& c, float* P, int ldp, uint64_t rows, int w, const uint64_t* ptr, const uint32_t* idx,
                        const float* W, int ldw, uint64_t n, const double* cs, const double* mean,
                        const double* scale) {
    if (!rows) return;
    const bool quads = ldw % 4 == 0 && reinterpret_cast<uintptr_t>(W) % 16 == 0 &&
                       n * (uint64_t)(ldw / 4) <= 0xffffffffull;
    for (int c0 = 0; c0 < w;) {
        if (quads) {
            // Column blocks that keep the lanes of a group busy: 64 columns
            // (16 lanes), 32 (8 lanes), then the rest in the fewest lanes
            // that hold it.  A warp step gathers 32 / L missing calls, so a
            // block of 32 lanes for w = 71 (18 of them busy) took one call
            // per step and 2.5 times as long as the w = 30 fix; as 64 + 7
            // columns in 16 + 2 lanes the lists are read twice.  Every
            // column's fix is separate.
            const int rem = w - c0;
            const int wb = rem >= 64 ? 64 : (rem > 32 ? 32 : rem);
            const int nq = (wb + 3) / 4;
            const unsigned grid = (unsigned)ceil_div(rows * 32, 256);
#define SLFMM_ROWFIX4(LL)                                                                                     \
    k_rowfix_mean4<LL><<<grid, 256, 0, c.stream>>>(P + c0, ldp, rows, wb, ptr, idx, W + c0, ldw, cs + c0, mean, \
                                                   scale)
            if (nq <= 1) SLFMM_ROWFIX4(1);
            else if (nq <= 2) SLFMM_ROWFIX4(2);
            else if (nq <= 4) SLFMM_ROWFIX4(4);
            else if (nq <= 8) SLFMM_ROWFIX4(8);
            else SLFMM_ROWFIX4(16);
#undef SLFMM_ROWFIX4
            SLFMM_LAUNCHED(c, "k_rowfix_mean4");
            c0 += wb;
            continue;
        }
        // a warp covers 128 columns (4 per lane): wider operands in column blocks
        k_rowfix_mean<<<(unsigned)ceil_div(rows * 32, 256), 256, 0, c.stream>>>(
            P + c0, ldp, rows, std::min(128, w - c0), ptr, idx, W + c0, ldw, cs + c0, mean, scale);
        SLFMM_LAUNCHED(c, "k_rowfix_mean");
        c0 += 128;
    }
}

void launch_colfix_mean(Ctx& c, double* S, int lds, uint64_t n, int w, const uint64_t* ptr, const uint32_t* idx,
                        const float* Q, int ldq, const double* coef, const double* colterm) {
    if (!n) return;
    k_colfix_mean<<<(unsigned)ceil_div(n * 32, 256), 256, 0, c.stream>>>(S, lds, n, w, ptr, idx, Q, ldq, coef,
                                                                        colterm);
    SLFMM_LAUNCHED(c, "k_colfix_mean");
}

void launch_weighted_colsum(Ctx& c, const float* Q, int ldq, uint64_t p, int w, const double* coef, double* out) {
    SLFMM_REQUIRE(w <= 128, SLFMM_ERR_BAD_ARG, "width");
    if (ldq % 4 == 0 && ldq <= 32 && w <= ldq && reinterpret_cast<uintptr_t>(Q) % 16 == 0) {
        const uint64_t qb = std::max<uint64_t>(
            1, std::min<uint64_t>(ceil_div(p * (uint64_t)(ldq / 4), 1024), (uint64_t)c.sm_count * 4));
        DBuf<double> qpart(qb * w, c.stream);
        k_weighted_colsum_quads<<<(unsigned)qb, 256, 0, c.stream>>>(Q, ldq, p, w, coef, qpart.get());
        SLFMM_LAUNCHED(c, "k_weighted_colsum_quads");
        launch_sum_partials(c, qpart.get(), (int)qb, (uint64_t)w, out);
        return;
    }
    const uint64_t blocks = std::max<uint64_t>(1, std::min<uint64_t>(ceil_div(p, 256), (uint64_t)c.sm_count * 4));
    DBuf<double> part(blocks * w, c.stream);
    if (w <= 32) k_weighted_colsum<1><<<(unsigned)blocks, 256, 0, c.stream>>>(Q, ldq, p, w, coef, part.get());
    else if (w <= 64) k_weighted_colsum<2><<<(unsigned)blocks, 256, 0, c.stream>>>(Q, ldq, p, w, coef, part.get());
    else k_weighted_colsum<4><<<(unsigned)blocks, 256, 0, c.stream>>>(Q, ldq, p, w, coef, part.get());
    SLFMM_LAUNCHED(c, "k_weighted_colsum");
    launch_sum_partials(c, part.get(), (int)blocks, (uint64_t)w, out);
}

void launch_scale_product(Ctx& c, const double* a, const double* b, uint64_t n, double* out) {
    if (!n) return;
    k_scale_product<<<grid_for(c, n, 256), 256, 0, c.stream>>>(a, b, n, out);
    SLFMM_LAUNCHED(c, "k_scale_product");
}

}  // namespace slfmm
