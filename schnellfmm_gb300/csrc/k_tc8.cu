// Split-FP8 tcgen05 contraction of the packed genotype matrix (kind::f8f6f4).
//
//   P[r, c] = sum_t s_t[c] * sum_k g(r, k) * B_t[c, k]              (main)
//   M[r, c] = sum_t m_t[c] * sum_k [g(r, k) missing] * E_t[c, k]    (indicator)
//
// Genotypes {0, 1, 2} are exact in E4M3 and are expanded from the 2-bit codes
// in registers (PRMT, no shared-memory tables) straight into TMEM as the A
// operand.  The float operand W is split into power-of-two-scaled E4M3 terms:
// term t holds round_e4m3((W - terms_<t) * 2^(e0 + 4t)), so four terms carry
// about 16 significant bits per column (the "split-FP8" precision pattern);
// the per-(term, column) scales are applied in FP32 in the epilogue.  The
// optional second A operand is the missing-call indicator, multiplied by a
// second set of terms, which makes the mean-imputation correction of missing
// calls exact without any gather over the missing-call lists.
//
// W tiles are shared by the CTAs of a cluster through TMA multicast: each of
// the C CTAs loads 1/C of the rows of every W stage into all C CTAs.  A stage
// is reloaded only after every CTA of the cluster has finished its MMAs on it
// (per-stage "B empty" barriers counting C multicast commits).
//
// Replaces the reference's per-chunk FP64 dgemms (src/rsvd.rs:61-69, :88-97,
// :117-125, :144-153; src/testing.rs:355-374) and, through the indicator
// operand, the NaN -> column-mean fill of decode_single_snp
// (src/bed.rs:349-378) inside them.
#include <cuda.h>
#include <cuda_fp8.h>
#include <cudaTypedefs.h>

#include "slfmm_internal.h"
#include "tc_common.cuh"

namespace slfmm {
namespace {
using namespace tc;

constexpr int kM = 128;
constexpr int kKB = 128;
constexpr int kPacked = kM * kKB / 4;  // 4096 B
constexpr int kThreads = 192;
constexpr int kMainTerms = 4;
constexpr int kIndTerms = 3;
constexpr uint32_t kTabGeno = 0x40380000u;  // code 00,01 -> 0; 10 -> 1.0; 11 -> 2.0 (E4M3 bytes)
constexpr uint32_t kTabMiss = 0x00003800u;  // code 01 (missing) -> 1.0

struct Tc8Args {
    uint32_t rows, kb_total, kb_per_split;
    uint32_t wpad;          // output columns
    uint32_t n_main;        // kMainTerms * wpad
    uint32_t n_ind;         // kIndTerms * wpad or 0
    uint32_t n_total;       // B rows / D columns in use
    uint32_t d_cols;        // TMEM columns reserved for D
    uint32_t a_cols;        // TMEM columns per A stage (32, or 64 with the indicator)
    uint32_t stages, tmem_cols;
    uint32_t b_stage_bytes; // n_total * 128
    uint32_t cluster;       // CTAs sharing W through multicast
    uint32_t box_rows;      // rows per W TMA box
    uint32_t loads;         // W boxes this CTA issues per stage
    const float* inv_scale; // n_total: 2^-(e0 + 4t) per B row
    int mode;               // 0: out = P + M; 1: out = s_r (P - mu_r (cs_c - M))
    const double* row_mean;
    const double* row_scale;
    const double* cs;
    float* out;
    uint32_t ldo;
    uint64_t split_stride;
    int* err;
};

// 8 two-bit codes (low 16 bits) -> 8 nibbles, code i in nibble i
__device__ __forceinline__ uint32_t spread8(uint32_t x) {
    x &= 0xFFFFu;
    x = (x | (x << 8)) & 0x00FF00FFu;
    x = (x | (x << 4)) & 0x0F0F0F0Fu;
    x = (x | (x << 2)) & 0x33333333u;
    return x;
}

__global__ void __launch_bounds__(kThreads, 1)
    k_tc8_rows(const __grid_constant__ CUtensorMap tm_packed, const __grid_constant__ CUtensorMap tm_b, Tc8Args a) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const uint32_t S = a.stages;
    uint8_t* bsm = smem;
    uint8_t* psm = bsm + S * a.b_stage_bytes;
    float* scl = reinterpret_cast<float*>(psm + S * kPacked);                // up to 512 floats
    uint64_t* bars = reinterpret_cast<uint64_t*>(reinterpret_cast<uint8_t*>(scl) + 2048);
    uint64_t* full_tma = bars;
    uint64_t* full_a = bars + S;
    uint64_t* a_empty = bars + 2 * S;
    uint64_t* b_empty = bars + 3 * S;
    uint64_t* tmem_full = bars + 4 * S;
    uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(bars + 4 * S + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t C = a.cluster;
    const uint32_t rank = C > 1 ? cluster_ctarank() : 0;
    const uint16_t mask = (uint16_t)((1u << C) - 1u);
    const uint32_t row0 = blockIdx.x * kM;
    const uint32_t kb0 = blockIdx.y * a.kb_per_split;
    const uint32_t kb1 = min(a.kb_total, kb0 + a.kb_per_split);
    const uint32_t nkb = kb1 > kb0 ? kb1 - kb0 : 0;
    const bool ind = a.n_ind != 0;

    if (threadIdx.x == 0) {
        for (uint32_t s = 0; s < S; ++s) {
            mbar_init(full_tma + s, 1);
            mbar_init(full_a + s, 128);
            mbar_init(a_empty + s, 1);
            mbar_init(b_empty + s, C);
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
    for (uint32_t e = threadIdx.x; e < a.n_total; e += blockDim.x) scl[e] = a.inv_scale[e];
    fence_before();
    __syncthreads();
    fence_after();
    cluster_sync();  // every peer's barriers exist before any multicast lands
    const uint32_t tmem = *tmem_holder;

    if (warp == 0) {
        if (lane == 0) {
            const uint32_t y_begin = rank * a.box_rows * a.loads;
            uint32_t issued = 0;
            for (uint32_t i = 0; i < nkb; ++i) {
                const uint32_t s = i % S, r = i / S;
                if (r > 0 && !mbar_wait(b_empty + s, (r - 1) & 1, a.err, 11)) break;
                mbar_arrive_tx(full_tma + s, kPacked + a.b_stage_bytes);
                const int kb = (int)(kb0 + i);
                tma_2d(psm + s * kPacked, &tm_packed, kb * (kKB / 4), (int)row0, full_tma + s);
                for (uint32_t l = 0; l < a.loads; ++l) {
                    const uint32_t y = y_begin + l * a.box_rows;
                    uint8_t* dst = bsm + s * a.b_stage_bytes + y * 128;
                    if (C > 1) tma_2d_mc(dst, &tm_b, kb * kKB, (int)y, full_tma + s, mask);
                    else tma_2d(dst, &tm_b, kb * kKB, (int)y, full_tma + s);
                }
                issued = i + 1;
            }
            for (uint32_t i = issued > S ? issued - S : 0; i < issued; ++i)
                mbar_wait(full_tma + i % S, (i / S) & 1, a.err, 12);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t nchunk = (a.n_main + 255) / 256;
            const uint32_t chunk = a.n_main / nchunk;   // host guarantees divisibility
            const uint32_t id_main = instr_desc_e4m3(chunk);
            const uint32_t id_ind = ind ? instr_desc_e4m3(a.n_ind) : 0u;
            for (uint32_t i = 0; i < nkb; ++i) {
                const uint32_t s = i % S, r = i / S;
                if (!mbar_wait(full_tma + s, r & 1, a.err, 13)) break;
                if (!mbar_wait(full_a + s, r & 1, a.err, 14)) break;
                fence_after();
                const uint32_t b_base = smem_u32(bsm + s * a.b_stage_bytes);
                const uint32_t a_base = tmem + a.d_cols + s * a.a_cols;
#pragma unroll
                for (int kk = 0; kk < kKB / 32; ++kk) {
                    const uint32_t acc = (i > 0 || kk > 0) ? 1u : 0u;
                    for (uint32_t ch = 0; ch < nchunk; ++ch)
                        mma_ts_f8(tmem + ch * chunk, a_base + kk * 8, smem_desc(b_base + ch * chunk * 128 + kk * 32),
                                  id_main, acc);
                    if (ind)
                        mma_ts_f8(tmem + a.n_main, a_base + 32 + kk * 8,
                                  smem_desc(b_base + a.n_main * 128 + kk * 32), id_ind, acc);
                }
                mma_commit(a_empty + s);
                if (C > 1) mma_commit_mc(b_empty + s, mask);
                else mma_commit(b_empty + s);
            }
            mma_commit(tmem_full);
        }
    } else {
        const uint32_t q = (uint32_t)warp & 3u;
        const uint32_t row = q * 32 + lane;
        const uint32_t lane_base = tmem + ((q * 32) << 16);
        for (uint32_t i = 0; i < nkb; ++i) {
            const uint32_t s = i % S, r = i / S;
            if (!__all_sync(0xffffffffu, r == 0 || mbar_wait(a_empty + s, (r - 1) & 1, a.err, 15))) break;
            if (!__all_sync(0xffffffffu, mbar_wait(full_tma + s, r & 1, a.err, 16))) break;
            const uint4* src = reinterpret_cast<const uint4*>(psm + s * kPacked + row * (kKB / 4));
            const uint4 p0 = src[0], p1 = src[1];
            const uint32_t w8[8] = {p0.x, p0.y, p0.z, p0.w, p1.x, p1.y, p1.z, p1.w};
            uint32_t g[32];
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                const uint32_t s0 = spread8(w8[t]), s1 = spread8(w8[t] >> 16);
                g[4 * t + 0] = __byte_perm(kTabGeno, 0u, s0);
                g[4 * t + 1] = __byte_perm(kTabGeno, 0u, s0 >> 16);
                g[4 * t + 2] = __byte_perm(kTabGeno, 0u, s1);
                g[4 * t + 3] = __byte_perm(kTabGeno, 0u, s1 >> 16);
            }
            const uint32_t a_col = lane_base + a.d_cols + s * a.a_cols;
            tmem_st_x32(a_col, g);
            if (ind) {
#pragma unroll
                for (int t = 0; t < 8; ++t) {
                    const uint32_t s0 = spread8(w8[t]), s1 = spread8(w8[t] >> 16);
                    g[4 * t + 0] = __byte_perm(kTabMiss, 0u, s0);
                    g[4 * t + 1] = __byte_perm(kTabMiss, 0u, s0 >> 16);
                    g[4 * t + 2] = __byte_perm(kTabMiss, 0u, s1);
                    g[4 * t + 3] = __byte_perm(kTabMiss, 0u, s1 >> 16);
                }
                tmem_st_x32(a_col + 32, g);
            }
            asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
            fence_before();
            mbar_arrive(full_a + s);
        }
        // epilogue
        const bool ok = __all_sync(0xffffffffu, mbar_wait(tmem_full, 0, a.err, 17));
        fence_after();
        const uint32_t grow = row0 + row;
        const bool live = ok && grow < a.rows;
        double rm = 0.0, rs = 0.0;
        if (a.mode == 1 && live) {
            rm = a.row_mean[grow];
            rs = a.row_scale[grow];
        }
        float* dst = a.out + (uint64_t)blockIdx.y * a.split_stride + (uint64_t)grow * a.ldo;
        for (uint32_t c0 = 0; c0 < a.wpad; c0 += 16) {
            float pm[16], pi[16], v[16];
#pragma unroll
            for (int k = 0; k < 16; ++k) pm[k] = pi[k] = 0.f;
            for (int t = 0; t < kMainTerms; ++t) {
                const uint32_t col = t * a.wpad + c0;
                tmem_ld_x16(lane_base + col, v);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int k = 0; k < 16; ++k) pm[k] = fmaf(scl[col + k], v[k], pm[k]);
            }
            if (ind) {
                for (int t = 0; t < kIndTerms; ++t) {
                    const uint32_t col = a.n_main + t * a.wpad + c0;
                    tmem_ld_x16(lane_base + col, v);
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                    for (int k = 0; k < 16; ++k) pi[k] = fmaf(scl[col + k], v[k], pi[k]);
                }
            }
            if (live) {
#pragma unroll
                for (int k = 0; k < 16; ++k) {
                    if (a.mode == 1)
                        v[k] = (float)(rs * ((double)pm[k] - rm * (a.cs[c0 + k] - (double)pi[k])));
                    else
                        v[k] = pm[k] + pi[k];
                }
                float4* d4 = reinterpret_cast<float4*>(dst + c0);
#pragma unroll
                for (int t = 0; t < 4; ++t) d4[t] = make_float4(v[4 * t], v[4 * t + 1], v[4 * t + 2], v[4 * t + 3]);
            }
        }
    }
    fence_before();
    __syncthreads();
    cluster_sync();  // no peer multicasts or commits into this CTA after this point
    if (warp == 1) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(a.tmem_cols)
                     : "memory");
    }
}

// per-column max |x * kscale| as float bits (non-negative floats order as ints)
template <typename T>
__global__ void k_colmax_abs(const T* __restrict__ src, int ld, uint64_t K, int w, const double* __restrict__ kscale,
                             unsigned* __restrict__ colmax) {
    const int c = threadIdx.x % w;
    const int rstep = blockDim.x / w;
    const int r0 = threadIdx.x / w;
    if (r0 >= rstep) return;
    float m = 0.f;
    for (uint64_t k = (uint64_t)blockIdx.x * rstep + r0; k < K; k += (uint64_t)gridDim.x * rstep) {
        double x = (double)src[k * ld + c];
        if (kscale) x *= kscale[k];
        m = fmaxf(m, fabsf((float)x));
    }
    atomicMax(colmax + c, __float_as_uint(m));
}

__device__ __forceinline__ int term_e0(unsigned bits) {
    const float cm = __uint_as_float(bits);
    if (!(cm > 0.f)) return 0;
    int E;
    frexpf(cm, &E);
    return 8 - E;  // cm * 2^e0 in [128, 256)
}

// W (K x w) -> `terms` E4M3 rows per column at B rows row_off + t * wpad + c,
// K contiguous, zero padded to K_pad; inv_scale[row] = 2^-(e0 + 4t).
template <typename T>
__global__ void k_fp8_terms(const T* __restrict__ src, int ld, uint64_t K, int w, int wpad, uint64_t K_pad,
                            const double* __restrict__ kscale, int terms, int row_off,
                            const unsigned* __restrict__ colmax, uint8_t* __restrict__ B, float* __restrict__ inv_scale) {
    __shared__ uint8_t tile[kMainTerms][32][129];
    const uint64_t k0 = (uint64_t)blockIdx.x * 128;
    const int c0 = blockIdx.y * 32;
    for (int e = threadIdx.x; e < 128 * 32; e += blockDim.x) {
        const int kk = e / 32, cc = e % 32;
        const uint64_t k = k0 + kk;
        const int c = c0 + cc;
        float r = 0.f;
        if (k < K && c < w) {
            double x = (double)src[k * ld + c];
            if (kscale) x *= kscale[k];
            r = (float)x;
        }
        const int e0 = c < w ? term_e0(colmax[c]) : 0;
        for (int t = 0; t < terms; ++t) {
            const int ex = e0 + 4 * t;
            const __nv_fp8_storage_t qv = __nv_cvt_float_to_fp8(ldexpf(r, ex), __NV_SATFINITE, __NV_E4M3);
            const __half_raw hr = __nv_cvt_fp8_to_halfraw(qv, __NV_E4M3);
            r -= ldexpf(__half2float(__half(hr)), -ex);
            tile[t][cc][kk] = (uint8_t)qv;
        }
    }
    __syncthreads();
    if (blockIdx.x == 0)
        for (int e = threadIdx.x; e < terms * 32; e += blockDim.x) {
            const int t = e / 32, cc = e % 32, c = c0 + cc;
            if (c < wpad) inv_scale[row_off + t * wpad + c] = c < w ? ldexpf(1.f, -(term_e0(colmax[c]) + 4 * t)) : 1.f;
        }
    for (int e = threadIdx.x; e < terms * 32 * 128; e += blockDim.x) {
        const int t = e / (32 * 128), rem = e % (32 * 128), cc = rem / 128, kk = rem % 128;
        const int c = c0 + cc;
        const uint64_t k = k0 + kk;
        if (c < wpad && k < K_pad) B[(uint64_t)(row_off + t * wpad + c) * K_pad + k] = tile[t][cc][kk];
    }
}

__global__ void k_sub_colterm(double* __restrict__ S, int lds, uint64_t n, int w, const double* __restrict__ colterm) {
    const uint64_t total = n * w;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total; t += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = t / w;
        const int c = (int)(t - i * w);
        S[i * lds + c] -= colterm[c];
    }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn8() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        SLFMM_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
        SLFMM_REQUIRE(q == cudaDriverEntryPointSuccess && p, SLFMM_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
        fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

CUtensorMap map2d_u8(const uint8_t* base, uint64_t inner, uint64_t rows, uint32_t box_inner, uint32_t box_rows,
                     bool swizzle128) {
    CUtensorMap m;
    cuuint64_t dims[2] = {inner, rows};
    cuuint64_t strides[1] = {inner};
    cuuint32_t box[2] = {box_inner, box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = encode_fn8()(&m, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<uint8_t*>(base), dims, strides, box, es,
                              CU_TENSOR_MAP_INTERLEAVE_NONE,
                              swizzle128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    SLFMM_REQUIRE(r == CUDA_SUCCESS, SLFMM_ERR_CUDA, "tensor map encode failed: " + std::to_string((int)r));
    return m;
}

}  // namespace

Fp8Plan fp8_plan(int wpad, bool ind, uint64_t tiles) {
    Fp8Plan p{};
    p.wpad = (uint32_t)wpad;
    p.n_main = kMainTerms * wpad;
    p.n_ind = ind ? kIndTerms * wpad : 0;
    p.n_total = p.n_main + p.n_ind;
    p.d_cols = (uint32_t)round_up(p.n_total, 32);
    p.a_cols = ind ? 64 : 32;
    p.b_stage_bytes = p.n_total * 128;
    const size_t fixed = 1024 + 2048 + 64 * 8 + 64;
    const size_t per_stage = p.b_stage_bytes + kPacked;
    const uint32_t st2 = p.d_cols < 256 ? std::min<uint32_t>((256 - p.d_cols) / p.a_cols,
                                                              (uint32_t)((110 * 1024 - fixed) / per_stage))
                                        : 0;
    if (st2 >= 3) {
        p.stages = std::min<uint32_t>(st2, 6);
        p.tmem_cols = 256;
    } else {
        p.stages = p.d_cols < 512 ? std::min<uint32_t>((512 - p.d_cols) / p.a_cols,
                                                       (uint32_t)((220 * 1024 - fixed) / per_stage))
                                  : 0;
        p.stages = std::min<uint32_t>(p.stages, 6);
        p.tmem_cols = 512;
    }
    p.smem = fixed + p.stages * per_stage;
    // cluster multicast of W when there are enough tiles and rows split evenly
    p.cluster = 1;
    for (uint32_t c : {4u, 2u})
        if (tiles >= 2 * c && p.n_total % (8 * c) == 0) {
            p.cluster = c;
            break;
        }
    const uint32_t rows_mine = p.n_total / p.cluster;
    p.loads = (uint32_t)ceil_div(rows_mine, 256);
    while (rows_mine % p.loads != 0 || (rows_mine / p.loads) % 8 != 0) ++p.loads;
    p.box_rows = rows_mine / p.loads;
    p.ok = p.stages >= 2 && p.n_main % ceil_div(p.n_main, 256) == 0 && (p.n_main / ceil_div(p.n_main, 256)) % 16 == 0 &&
           p.n_ind <= 256;
    return p;
}

void launch_fp8_terms_f64(Ctx& c, const double* src, int ld, uint64_t K, int w, int wpad, uint64_t K_pad,
                          const double* kscale, int terms, int row_off, uint8_t* B, float* inv_scale) {
    DBuf<unsigned> cm(wpad, c.stream);
    cm.zero();
    const int rstep = 256 / w;
    k_colmax_abs<double><<<grid_for(c, ceil_div(K, rstep), 1), w * rstep, 0, c.stream>>>(src, ld, K, w, kscale, cm.get());
    SLFMM_LAUNCHED(c, "k_colmax_abs");
    dim3 grid((unsigned)ceil_div(K_pad, 128), (unsigned)ceil_div(wpad, 32));
    k_fp8_terms<double><<<grid, 256, 0, c.stream>>>(src, ld, K, w, wpad, K_pad, kscale, terms, row_off, cm.get(), B,
                                                    inv_scale);
    SLFMM_LAUNCHED(c, "k_fp8_terms");
}

void launch_fp8_terms_f32(Ctx& c, const float* src, int ld, uint64_t K, int w, int wpad, uint64_t K_pad,
                          const double* kscale, int terms, int row_off, uint8_t* B, float* inv_scale) {
    DBuf<unsigned> cm(wpad, c.stream);
    cm.zero();
    const int rstep = 256 / w;
    k_colmax_abs<float><<<grid_for(c, ceil_div(K, rstep), 1), w * rstep, 0, c.stream>>>(src, ld, K, w, kscale, cm.get());
    SLFMM_LAUNCHED(c, "k_colmax_abs");
    dim3 grid((unsigned)ceil_div(K_pad, 128), (unsigned)ceil_div(wpad, 32));
    k_fp8_terms<float><<<grid, 256, 0, c.stream>>>(src, ld, K, w, wpad, K_pad, kscale, terms, row_off, cm.get(), B,
                                                   inv_scale);
    SLFMM_LAUNCHED(c, "k_fp8_terms");
}

int launch_tc8_rows(Ctx& c, const Fp8Plan& pl, const uint8_t* packed, uint64_t stride, uint64_t rows, uint64_t K,
                     const uint8_t* B, const float* inv_scale, uint64_t K_pad, int mode, const double* row_mean,
                     const double* row_scale, const double* cs, float* out, int ldo, int splits,
                     uint64_t split_stride) {
    SLFMM_REQUIRE(pl.ok, SLFMM_ERR_BAD_ARG, "no feasible split-FP8 tile plan for this width");
    SLFMM_REQUIRE(K_pad % kKB == 0 && K_pad >= ceil_div(K, kKB) * kKB, SLFMM_ERR_BAD_ARG, "bad K padding");
    SLFMM_REQUIRE(stride % 16 == 0 && stride * 4 >= ceil_div(K, kKB) * kKB, SLFMM_ERR_BAD_ARG, "bad packed stride");
    SLFMM_REQUIRE(mode == 0 || pl.n_ind != 0, SLFMM_ERR_BAD_ARG, "row correction needs the indicator operand");
    static thread_local size_t configured = 0;
    if (configured < pl.smem) {
        SLFMM_CUDA(cudaFuncSetAttribute(k_tc8_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.smem));
        configured = pl.smem;
    }
    const CUtensorMap tp = map2d_u8(packed, stride, rows, kKB / 4, kM, false);
    const CUtensorMap tb = map2d_u8(B, K_pad, pl.n_total, 128, pl.box_rows, true);
    DBuf<int> err(1, c.stream);
    err.zero();
    Tc8Args a{};
    a.rows = (uint32_t)rows;
    a.kb_total = (uint32_t)ceil_div(K, kKB);
    a.kb_per_split = (uint32_t)ceil_div(a.kb_total, (uint64_t)std::max(splits, 1));
    a.wpad = pl.wpad;
    a.n_main = pl.n_main;
    a.n_ind = pl.n_ind;
    a.n_total = pl.n_total;
    a.d_cols = pl.d_cols;
    a.a_cols = pl.a_cols;
    a.stages = pl.stages;
    a.tmem_cols = pl.tmem_cols;
    a.b_stage_bytes = pl.b_stage_bytes;
    a.cluster = pl.cluster;
    a.box_rows = pl.box_rows;
    a.loads = pl.loads;
    a.inv_scale = inv_scale;
    a.mode = mode;
    a.row_mean = row_mean;
    a.row_scale = row_scale;
    a.cs = cs;
    a.out = out;
    a.ldo = (uint32_t)ldo;
    a.split_stride = split_stride;
    a.err = err.get();
    const unsigned gy = (unsigned)ceil_div(a.kb_total, a.kb_per_split);
    const unsigned gx = (unsigned)round_up(ceil_div(rows, kM), pl.cluster);
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(gx, gy, 1);
    cfg.blockDim = dim3(kThreads, 1, 1);
    cfg.dynamicSmemBytes = pl.smem;
    cfg.stream = c.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = pl.cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    SLFMM_CUDA(cudaLaunchKernelEx(&cfg, k_tc8_rows, tp, tb, a));
    SLFMM_LAUNCHED(c, "k_tc8_rows");
    int h = 0;
    SLFMM_CUDA(cudaMemcpyAsync(&h, err.get(), sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    SLFMM_CUDA(cudaStreamSynchronize(c.stream));
    if (h != 0)
        throw Error(SLFMM_ERR_DEVICE_TIMEOUT,
                    "split-FP8 contraction: a bounded device wait expired (site " + std::to_string(h) + ")");
    return (int)gy;
}

void launch_sub_colterm(Ctx& c, double* S, int lds, uint64_t n, int w, const double* colterm) {
    if (!n || !w) return;
    k_sub_colterm<<<grid_for(c, n * w, 256), 256, 0, c.stream>>>(S, lds, n, w, colterm);
    SLFMM_LAUNCHED(c, "k_sub_colterm");
}

}  // namespace slfmm
