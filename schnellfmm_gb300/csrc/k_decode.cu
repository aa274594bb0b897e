// Stage (a): PLINK 2-bit ingest, allele counting, missing-call lists,
// per-SNP mean / scale / TSS and standardised decode.
//
// Reference behaviour: src/bed.rs:262-395 (decode_raw_single_snp,
// decode_single_snp, compute_scale), src/parallel.rs:53-71 and :129-146.
#include <cub/cub.cuh>

#include <vector>

#include "slfmm_internal.h"
#include "stats_common.cuh"

namespace slfmm {

namespace {

constexpr uint32_t kLo = 0x55555555u;

__device__ __forceinline__ uint32_t code_at(const uint8_t* row, uint64_t s) {
    return (row[s >> 2] >> ((s & 3) * 2)) & 3u;
}

// Re-pack `rows` physical SNP rows (in_bps bytes each, contiguous) into the
// device layout: `stride` bytes per row, samples in sample_keep order (or
// physical order), codes of samples >= n_out forced to 00.
__global__ void k_repack(const uint8_t* __restrict__ in, uint64_t rows, uint64_t in_bps,
                         const uint32_t* __restrict__ keep, uint64_t n_out,
                         uint8_t* __restrict__ out, uint64_t stride) {
    const uint64_t words_per_row = stride / 4;
    const uint64_t total = rows * words_per_row;
    const uint64_t out_bps = (n_out + 3) / 4;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
         t += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t r = t / words_per_row;
        const uint64_t w = t - r * words_per_row;
        const uint8_t* src = in + r * in_bps;
        uint32_t word = 0;
        if (keep == nullptr) {
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const uint64_t byte = w * 4 + b;
                if (byte < out_bps) {
                    uint32_t v = src[byte];
                    if (byte == out_bps - 1 && (n_out & 3)) v &= (1u << (2 * (n_out & 3))) - 1u;
                    word |= v << (8 * b);
                }
            }
        } else {
            const uint64_t s0 = w * 16;
#pragma unroll 4
            for (int k = 0; k < 16; ++k) {
                const uint64_t s = s0 + k;
                if (s < n_out) word |= code_at(src, keep[s]) << (2 * k);
            }
        }
        reinterpret_cast<uint32_t*>(out + r * stride)[w] = word;
    }
}

// Re-pack with a sample subset, one block per row (grid-stride): the row's
// in_bps bytes and the kept sample indices are staged in shared memory, the
// indices transposed (ks[k * words + w] = keep[16 w + k]) so that the threads
// of a warp, one output word each, read consecutive entries.  Host side checks
// that both arrays fit.
__global__ void __launch_bounds__(256) k_repack_keep(const uint8_t* __restrict__ in, uint64_t rows, uint64_t in_bps,
                                                     const uint32_t* __restrict__ keep, uint64_t n_out,
                                                     uint8_t* __restrict__ out, uint64_t stride) {
    extern __shared__ __align__(16) uint8_t sm_keep[];
    const uint64_t words = (n_out + 15) / 16;           // output words holding kept samples
    uint32_t* ks = reinterpret_cast<uint32_t*>(sm_keep);  // 16 x words indices
    uint8_t* row_s = sm_keep + ((words * 16 * 4 + 15) / 16) * 16;
    for (uint64_t e = threadIdx.x; e < words * 16; e += blockDim.x) {
        const uint64_t w = e / 16, k = e % 16, s = w * 16 + k;
        ks[k * words + w] = s < n_out ? keep[s] : 0xFFFFFFFFu;
    }
    const uint64_t out_words = stride / 4;
    const bool w4 = in_bps % 4 == 0 && reinterpret_cast<uintptr_t>(in) % 4 == 0;
    for (uint64_t r = blockIdx.x; r < rows; r += gridDim.x) {
        __syncthreads();  // the previous row's codes are consumed (and the indices staged)
        const uint8_t* src = in + r * in_bps;
        if (w4) {
            for (uint64_t i = threadIdx.x; i < in_bps / 4; i += blockDim.x)
                reinterpret_cast<uint32_t*>(row_s)[i] = reinterpret_cast<const uint32_t*>(src)[i];
        } else {
            for (uint64_t i = threadIdx.x; i < in_bps; i += blockDim.x) row_s[i] = src[i];
        }
        __syncthreads();
        uint32_t* dst = reinterpret_cast<uint32_t*>(out + r * stride);
        for (uint64_t w = threadIdx.x; w < out_words; w += blockDim.x) {
            uint32_t word = 0;
            if (w < words) {
#pragma unroll
                for (int k = 0; k < 16; ++k) {
                    const uint32_t idx = ks[k * words + w];
                    if (idx != 0xFFFFFFFFu) word |= (uint32_t)((row_s[idx >> 2] >> ((idx & 3) * 2)) & 3u) << (2 * k);
                }
            }
            dst[w] = word;
        }
    }
}

// Straight copy without a sample subset when the payload rows are V-aligned:
// rows of in_bps bytes -> rows of `stride` bytes, the payload's last 32-bit
// word masked to the codes of n_out samples and the rest of the row zero.
// One block per row (grid-stride), V-wide loads and stores.
template <typename V>
__global__ void k_repack_vec(const uint8_t* __restrict__ in, uint64_t rows, uint64_t in_bps, uint64_t n_out,
                             uint8_t* __restrict__ out, uint64_t stride) {
    constexpr int kw = sizeof(V) / 4;
    const uint64_t in_vecs = in_bps / sizeof(V), out_vecs = stride / sizeof(V);
    const uint64_t last_word = in_bps / 4 - 1;
    const uint64_t valid = n_out - 16 * last_word;  // codes in the last word
    const uint32_t tail = valid >= 16 ? 0xffffffffu : (1u << (2 * valid)) - 1u;
    for (uint64_t r = blockIdx.x; r < rows; r += gridDim.x) {
        const V* src = reinterpret_cast<const V*>(in + r * in_bps);
        V* dst = reinterpret_cast<V*>(out + r * stride);
        for (uint64_t v = threadIdx.x; v < out_vecs; v += blockDim.x) {
            V x{};
            if (v < in_vecs) {
                x = src[v];
                uint32_t* xw = reinterpret_cast<uint32_t*>(&x);
#pragma unroll
                for (int k = 0; k < kw; ++k)
                    if (v * kw + k == last_word) xw[k] &= tail;
            }
            dst[v] = x;
        }
    }
}

// One warp per SNP: popcount the 2-bit codes.  Padding codes are 00, so c0
// is derived as n - c1 - c2 - cmiss.
__global__ void k_snp_counts(const uint8_t* __restrict__ packed, uint64_t p, uint64_t stride,
                             uint64_t n, int32_t* __restrict__ counts,
                             uint64_t* __restrict__ miss_count) {
    const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32;
    const int lane = threadIdx.x & 31;
    if (warp >= p) return;
    // rows are 16-byte aligned (the stride is a multiple of 128 bytes)
    const uint4* row = reinterpret_cast<const uint4*>(packed + warp * stride);
    const uint64_t nwords = (n + 15) / 16, nvec = (nwords + 3) / 4;
    uint32_t c1 = 0, c2 = 0, cm = 0;
    for (uint64_t v = lane; v < nvec; v += 32) {
        const uint4 x = row[v];
        const uint32_t xs[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (v * 4 + k < nwords) {
                const uint32_t lo = xs[k] & kLo, hi = (xs[k] >> 1) & kLo;
                c1 += __popc(hi & ~lo);
                c2 += __popc(hi & lo);
                cm += __popc(~hi & lo);
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        c1 += __shfl_xor_sync(0xffffffffu, c1, o);
        c2 += __shfl_xor_sync(0xffffffffu, c2, o);
        cm += __shfl_xor_sync(0xffffffffu, cm, o);
    }
    if (lane == 0) {
        counts[warp * 4 + 0] = (int32_t)(n - c1 - c2 - cm);
        counts[warp * 4 + 1] = (int32_t)c1;
        counts[warp * 4 + 2] = (int32_t)c2;
        counts[warp * 4 + 3] = (int32_t)cm;
        if (miss_count) miss_count[warp] = cm;
    }
}

// One warp per SNP: write the ascending sample indices of missing calls
// (positions at or beyond cap are not written).
__global__ void k_miss_fill(const uint8_t* __restrict__ packed, uint64_t p, uint64_t stride,
                            uint64_t n, const uint64_t* __restrict__ ptr,
                            uint32_t* __restrict__ idx, uint32_t* __restrict__ rowid, uint64_t cap) {
    const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32;
    const int lane = threadIdx.x & 31;
    if (warp >= p) return;
    // 4 words (64 codes) per lane and step; rows are 16-byte aligned
    const uint4* row = reinterpret_cast<const uint4*>(packed + warp * stride);
    const uint64_t nwords = (n + 15) / 16, nvec = (nwords + 3) / 4;
    uint64_t base = ptr[warp];
    for (uint64_t v0 = 0; v0 < nvec; v0 += 32) {
        const uint64_t v = v0 + lane;
        uint32_t m[4] = {0u, 0u, 0u, 0u};
        if (v < nvec) {
            const uint4 x = row[v];
            const uint32_t xs[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (v * 4 + k < nwords) m[k] = ~(xs[k] >> 1) & xs[k] & kLo;
        }
        const uint32_t cnt = __popc(m[0]) + __popc(m[1]) + __popc(m[2]) + __popc(m[3]);
        uint32_t incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
        uint64_t pos = base + incl - cnt;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            uint32_t mk = m[k];
            while (mk) {
                const int b = __ffs(mk) - 1;
                mk &= mk - 1;
                if (pos < cap) {
                    idx[pos] = (uint32_t)((v * 4 + k) * 16 + (b >> 1));
                    if (rowid) rowid[pos] = (uint32_t)warp;
                }
                ++pos;
            }
        }
        base += total;
    }
}

// List offsets of rows [0, rows) of an upload chunk from their missing-call
// counts (counts[4 r + 3]): ptr[r + 1] = ptr[0] + sum of the counts of rows
// 0..r, where ptr[0] holds the previous chunk's end.  One block of 1024
// threads walks the chunk in tiles of 4096 rows with a running carry.
__global__ void __launch_bounds__(1024) k_miss_ptr_chunk(const int32_t* __restrict__ counts, uint64_t rows,
                                                         uint64_t* __restrict__ ptr) {
    __shared__ uint64_t warp_sum[32];
    const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
    uint64_t carry = ptr[0];
    for (uint64_t base = 0; base < rows; base += 4096) {
        uint64_t v[4], s = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint64_t r = base + (uint64_t)t * 4 + k;
            v[k] = r < rows ? (uint64_t)counts[r * 4 + 3] : 0ull;
            s += v[k];
        }
        uint64_t incl = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint64_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) warp_sum[wid] = incl;
        __syncthreads();
        if (wid == 0) {
            uint64_t ws = warp_sum[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint64_t y = __shfl_up_sync(0xffffffffu, ws, o);
                if (lane >= o) ws += y;
            }
            warp_sum[lane] = ws;  // inclusive over warps
        }
        __syncthreads();
        uint64_t run = carry + (wid ? warp_sum[wid - 1] : 0ull) + incl - s;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint64_t r = base + (uint64_t)t * 4 + k;
            run += v[k];
            if (r < rows) ptr[r + 1] = run;
        }
        carry += warp_sum[31];
        __syncthreads();  // warp_sum is rewritten by the next tile
    }
}

__global__ void k_count_keys(const uint32_t* __restrict__ keys, uint64_t nnz,
                             uint32_t* __restrict__ cnt) {
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < nnz;
         t += (uint64_t)gridDim.x * blockDim.x)
        atomicAdd(&cnt[keys[t]], 1u);
}

__global__ void k_u32_to_u64(const uint32_t* __restrict__ a, uint64_t m, uint64_t* __restrict__ b) {
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < m;
         t += (uint64_t)gridDim.x * blockDim.x)
        b[t] = a[t];
}

// Per-SNP mean over observed calls, scale and TSS, with the reference's
// operation order (src/bed.rs:349-361, :382-395) in round-to-nearest FP64
// intrinsics so that no FMA contraction changes the bits.
__global__ void k_stats_mean(const int32_t* __restrict__ counts, uint64_t p, int norm,
                             double* __restrict__ mean, double* __restrict__ scale,
                             double* __restrict__ tss, uint8_t* __restrict__ zero_var) {
    for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < p;
         j += (uint64_t)gridDim.x * blockDim.x) {
        const int64_t c0 = counts[j * 4 + 0], c1 = counts[j * 4 + 1], c2 = counts[j * 4 + 2];
        const int64_t nobs = c0 + c1 + c2;
        const int64_t s1 = c1 + 2 * c2, s2 = c1 + 4 * c2;
        const double mu = nobs > 0 ? __ddiv_rn((double)s1, (double)nobs) : 0.0;
        const double sc = scale_from_mean(mu, norm);
        const int64_t num = nobs * s2 - s1 * s1;  // exact: n_obs * centred sum of squares
        if (mean) mean[j] = mu;
        if (scale) scale[j] = sc;
        if (tss) tss[j] = nobs > 0 ? __dmul_rn(__dmul_rn(sc, sc), __ddiv_rn((double)num, (double)nobs)) : 0.0;
        if (zero_var) zero_var[j] = (num == 0 || sc == 0.0) ? 1 : 0;
    }
}

__global__ void k_decode_chunk(const uint8_t* __restrict__ packed, uint64_t stride, uint64_t n,
                               uint64_t snp0, uint64_t ncols, const double* __restrict__ mean,
                               const double* __restrict__ scale, double* __restrict__ out) {
    const uint64_t total = n * ncols;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
         t += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = t / ncols, c = t - i * ncols;
        const uint64_t j = snp0 + c;
        const uint32_t code = code_at(packed + j * stride, i);
        double v = 0.0;
        if (code != 1u) {
            const double g = code == 0 ? 0.0 : (double)(code - 1);
            v = __dmul_rn(__dsub_rn(g, mean[j]), scale[j]);
        }
        out[t] = v;
    }
}

__global__ void k_lut_std(uint64_t p, const double* __restrict__ mean,
                          const double* __restrict__ scale, float* __restrict__ lut) {
    for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < p;
         j += (uint64_t)gridDim.x * blockDim.x) {
        const double mu = mean[j], sc = scale[j];
        float4 v;
        v.x = (float)((0.0 - mu) * sc);
        v.y = 0.0f;
        v.z = (float)((1.0 - mu) * sc);
        v.w = (float)((2.0 - mu) * sc);
        reinterpret_cast<float4*>(lut)[j] = v;
    }
}

}  // namespace

void launch_repack(Ctx& c, const uint8_t* in, uint64_t rows, uint64_t in_bps, uint64_t /*n_phys*/,
                   const uint32_t* keep, uint64_t n_out, uint8_t* out, uint64_t stride) {
    if (rows == 0) return;
    const uintptr_t al = reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out) | in_bps | stride;
    if (keep == nullptr && in_bps == (n_out + 3) / 4 && al % 4 == 0) {
        const unsigned grid = (unsigned)std::min<uint64_t>(rows, (uint64_t)c.sm_count * 8);
        if (al % 16 == 0)
            k_repack_vec<uint4><<<grid, 256, 0, c.stream>>>(in, rows, in_bps, n_out, out, stride);
        else if (al % 8 == 0)
            k_repack_vec<uint2><<<grid, 256, 0, c.stream>>>(in, rows, in_bps, n_out, out, stride);
        else
            k_repack_vec<uint32_t><<<grid, 256, 0, c.stream>>>(in, rows, in_bps, n_out, out, stride);
        SLFMM_LAUNCHED(c, "k_repack_vec");
        return;
    }
    const size_t keep_smem = ((ceil_div(n_out, 16) * 16 * 4 + 15) / 16) * 16 + in_bps;
    if (keep != nullptr && keep_smem <= 200 * 1024) {
        raise_dynamic_smem((const void*)k_repack_keep, keep_smem);
        const uint64_t per_sm = std::max<uint64_t>(1, std::min<uint64_t>(4, (220 * 1024) / keep_smem));
        const unsigned grid = (unsigned)std::min<uint64_t>(rows, (uint64_t)c.sm_count * per_sm);
        k_repack_keep<<<grid, 256, keep_smem, c.stream>>>(in, rows, in_bps, keep, n_out, out, stride);
        SLFMM_LAUNCHED(c, "k_repack_keep");
        return;
    }
    const uint64_t work = rows * (stride / 4);
    k_repack<<<grid_for(c, work, 256), 256, 0, c.stream>>>(in, rows, in_bps, keep, n_out, out, stride);
    SLFMM_LAUNCHED(c, "k_repack");
}

void launch_snp_counts(Ctx& c, const Geno& g, uint64_t* miss_count_out) {
    if (g.p == 0) return;
    const int block = 256;
    const uint64_t grid = ceil_div(g.p * 32, block);
    k_snp_counts<<<(unsigned)grid, block, 0, c.stream>>>(packed_rows(g), g.p, g.stride, g.n,
                                                         g.counts.get(), miss_count_out);
    SLFMM_LAUNCHED(c, "k_snp_counts");
}

void launch_snp_counts_range(Ctx& c, const Geno& g, uint64_t r0, uint64_t rows) {
    if (rows == 0) return;
    const int block = 256;
    const uint64_t grid = ceil_div(rows * 32, block);
    k_snp_counts<<<(unsigned)grid, block, 0, c.stream>>>(packed_rows(g) + r0 * g.stride, rows, g.stride, g.n,
                                                         g.counts.get() + r0 * 4, nullptr);
    SLFMM_LAUNCHED(c, "k_snp_counts");
}

void build_missing_lists(Ctx& c, const Geno& g) {
    if (g.have_csr) return;
    DBuf<uint64_t> mc(g.p + 1, c.stream);
    SLFMM_CUDA(cudaMemsetAsync(mc.get() + g.p, 0, sizeof(uint64_t), c.stream));
    // a matrix held only as tiles (a per-trait sample subset) has its counts
    const bool tiles_only = g.packed.get() == nullptr;
    if (tiles_only) launch_miss_counts_of(c, g, mc.get());
    else launch_snp_counts(c, g, mc.get());
    g.miss_ptr.alloc(g.p + 1, c.stream);
    size_t tmp_bytes = 0;
    SLFMM_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, mc.get(), g.miss_ptr.get(),
                                             (int64_t)(g.p + 1), c.stream));
    DBuf<uint8_t> tmp(tmp_bytes, c.stream);
    SLFMM_CUDA(cub::DeviceScan::ExclusiveSum(tmp.get(), tmp_bytes, mc.get(), g.miss_ptr.get(),
                                             (int64_t)(g.p + 1), c.stream));
    uint64_t nnz = 0;
    SLFMM_CUDA(cudaMemcpyAsync(&nnz, g.miss_ptr.get() + g.p, sizeof(uint64_t),
                               cudaMemcpyDeviceToHost, c.stream));
    SLFMM_CUDA(cudaStreamSynchronize(c.stream));
    g.nnz = nnz;
    g.miss_idx.alloc(std::max<uint64_t>(nnz, 1), c.stream);
    if (nnz && g.p && tiles_only) {
        launch_miss_fill_tiles(c, g);
    } else if (nnz && g.p) {
        const int block = 256;
        k_miss_fill<<<(unsigned)ceil_div(g.p * 32, block), block, 0, c.stream>>>(
            packed_rows(g), g.p, g.stride, g.n, g.miss_ptr.get(), g.miss_idx.get(), nullptr, ~0ull);
        SLFMM_LAUNCHED(c, "k_miss_fill");
    }
    g.have_csr = true;
}

void csr_chunk_offsets(Ctx& c, const Geno& g, uint64_t r0, uint64_t rows) {
    if (rows == 0) return;
    k_miss_ptr_chunk<<<1, 1024, 0, c.stream>>>(g.counts.get() + r0 * 4, rows, g.miss_ptr.get() + r0);
    SLFMM_LAUNCHED(c, "k_miss_ptr_chunk");
}

void csr_chunk_fill(Ctx& c, const Geno& g, uint64_t r0, uint64_t rows, uint64_t cap) {
    if (rows == 0 || cap == 0) return;
    const int block = 256;
    k_miss_fill<<<(unsigned)ceil_div(rows * 32, block), block, 0, c.stream>>>(
        packed_rows(g) + r0 * g.stride, rows, g.stride, g.n, g.miss_ptr.get() + r0, g.miss_idx.get(), nullptr, cap);
    SLFMM_LAUNCHED(c, "k_miss_fill");
}

void build_missing_csc(Ctx& c, const Geno& g) {
    if (g.have_csc) return;
    build_missing_lists(c, g);
    g.missT_ptr.alloc(g.n + 1, c.stream);
    g.missT_ptr.zero();
    g.missT_idx.alloc(std::max<uint64_t>(g.nnz, 1), c.stream);
    if (g.nnz == 0) { g.have_csc = true; return; }
    SLFMM_REQUIRE(g.nnz < (1ull << 31), SLFMM_ERR_BAD_ARG, "too many missing calls for the sort");
    DBuf<uint32_t> rowid(g.nnz, c.stream), keys_out(g.nnz, c.stream);
    const int block = 256;
    k_miss_fill<<<(unsigned)ceil_div(g.p * 32, block), block, 0, c.stream>>>(
        packed_rows(g), g.p, g.stride, g.n, g.miss_ptr.get(), keys_out.get(), rowid.get(), ~0ull);
    SLFMM_LAUNCHED(c, "k_miss_fill");
    int end_bit = 1;
    while ((1ull << end_bit) < g.n) ++end_bit;
    size_t tmp_bytes = 0;
    DBuf<uint32_t> keys_sorted(g.nnz, c.stream);
    SLFMM_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys_out.get(), keys_sorted.get(),
                                               rowid.get(), g.missT_idx.get(), (int64_t)g.nnz, 0,
                                               end_bit, c.stream));
    DBuf<uint8_t> tmp(tmp_bytes, c.stream);
    SLFMM_CUDA(cub::DeviceRadixSort::SortPairs(tmp.get(), tmp_bytes, keys_out.get(), keys_sorted.get(),
                                               rowid.get(), g.missT_idx.get(), (int64_t)g.nnz, 0,
                                               end_bit, c.stream));
    DBuf<uint32_t> cnt(g.n + 1, c.stream);
    cnt.zero();
    k_count_keys<<<grid_for(c, g.nnz, 256), 256, 0, c.stream>>>(keys_sorted.get(), g.nnz, cnt.get());
    SLFMM_LAUNCHED(c, "k_count_keys");
    DBuf<uint64_t> cnt64(g.n + 1, c.stream);
    k_u32_to_u64<<<grid_for(c, g.n + 1, 256), 256, 0, c.stream>>>(cnt.get(), g.n + 1, cnt64.get());
    SLFMM_LAUNCHED(c, "k_u32_to_u64");
    size_t tb2 = 0;
    SLFMM_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tb2, cnt64.get(), g.missT_ptr.get(),
                                             (int64_t)(g.n + 1), c.stream));
    DBuf<uint8_t> tmp2(tb2, c.stream);
    SLFMM_CUDA(cub::DeviceScan::ExclusiveSum(tmp2.get(), tb2, cnt64.get(), g.missT_ptr.get(),
                                             (int64_t)(g.n + 1), c.stream));
    // longest per-sample list (splits the per-sample correction passes)
    std::vector<uint64_t> hp(g.n + 1);
    SLFMM_CUDA(cudaMemcpyAsync(hp.data(), g.missT_ptr.get(), (g.n + 1) * sizeof(uint64_t), cudaMemcpyDeviceToHost,
                               c.stream));
    SLFMM_CUDA(cudaStreamSynchronize(c.stream));
    g.missT_max = 0;
    for (uint64_t i = 0; i < g.n; ++i) g.missT_max = std::max<uint64_t>(g.missT_max, hp[i + 1] - hp[i]);
    g.have_csc = true;
}

void launch_stats_mean(Ctx& c, const Geno& g, int norm, double* mean, double* scale, double* tss,
                       uint8_t* zero_var) {
    if (g.p == 0) return;
    k_stats_mean<<<grid_for(c, g.p, 256), 256, 0, c.stream>>>(g.counts.get(), g.p, norm, mean,
                                                              scale, tss, zero_var);
    SLFMM_LAUNCHED(c, "k_stats_mean");
}

void launch_stats_mean_range(Ctx& c, const Geno& g, uint64_t r0, uint64_t rows, int norm, double* mean,
                             double* scale, double* tss, uint8_t* zero_var) {
    if (rows == 0) return;
    k_stats_mean<<<grid_for(c, rows, 256), 256, 0, c.stream>>>(g.counts.get() + r0 * 4, rows, norm, mean + r0,
                                                               scale + r0, tss + r0, zero_var + r0);
    SLFMM_LAUNCHED(c, "k_stats_mean");
}

void launch_decode_chunk(Ctx& c, const Geno& g, uint64_t snp0, uint64_t ncols, const double* mean,
                         const double* scale, double* out) {
    if (ncols == 0 || g.n == 0) return;
    k_decode_chunk<<<grid_for(c, g.n * ncols, 256), 256, 0, c.stream>>>(
        packed_rows(g), g.stride, g.n, snp0, ncols, mean, scale, out);
    SLFMM_LAUNCHED(c, "k_decode_chunk");
}

void launch_lut_std(Ctx& c, uint64_t p, const double* mean, const double* scale, float* lut) {
    if (p == 0) return;
    k_lut_std<<<grid_for(c, p, 256), 256, 0, c.stream>>>(p, mean, scale, lut);
    SLFMM_LAUNCHED(c, "k_lut_std");
}

}  // namespace slfmm
