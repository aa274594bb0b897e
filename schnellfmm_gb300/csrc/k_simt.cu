// Plain FP32 SIMT contractions over the packed genotype matrix.
//
// This is the straightforward GPU formulation of the reference's per-chunk
// dgemms (src/rsvd.rs:61-69, :88-97, :117-125, :144-153 and
// src/testing.rs:355-374): every 2-bit code is mapped through a per-SNP
// 4-entry lookup table (the standardised value of that genotype, 0 for a
// missing call under mean imputation) and multiplied in FP32.  It serves as
// the "plain FP32 GPU path" the tensor-core path is measured against and as
// an independent second implementation for parity checks.
#include "fp_convert.cuh"
#include "slfmm_internal.h"

namespace slfmm {
namespace {

constexpr int kRowSnps = 128;    // SNPs per CTA
constexpr int kRowSamples = 128; // samples per smem stage (32 bytes per SNP row)

// out[j, c] = sum_i lut_j[code_ij] * W[i, c]; W is (n_pad x WP) row-major
// with zero rows beyond n.  256 threads = 16 SNP groups (8 SNPs each) x 16
// column lanes (CPT columns each, stride 16).
template <int CPT>
__global__ void __launch_bounds__(256) k_row_lut(const uint8_t* __restrict__ packed, uint64_t stride,
                                                 uint64_t p, uint64_t n,
                                                 const float4* __restrict__ lut,
                                                 const float* __restrict__ W,
                                                 float* __restrict__ out) {
    constexpr int WP = CPT * 16;
    extern __shared__ float4 smem_f4[];
    float* Ws = reinterpret_cast<float*>(smem_f4);                 // [kRowSamples][WP]
    __shared__ uint32_t codes[kRowSnps][9];                         // 8 words + pad
    __shared__ float luts[kRowSnps][4];

    const int tid = threadIdx.x;
    const int ty = tid >> 4, tx = tid & 15;
    const uint64_t j0 = (uint64_t)blockIdx.x * kRowSnps;
    if (tid < kRowSnps) {
        const uint64_t j = j0 + tid;
        const float4 v = j < p ? lut[j] : make_float4(0.f, 0.f, 0.f, 0.f);
        luts[tid][0] = v.x; luts[tid][1] = v.y; luts[tid][2] = v.z; luts[tid][3] = v.w;
    }
    float acc[8][CPT];
#pragma unroll
    for (int r = 0; r < 8; ++r)
#pragma unroll
        for (int q = 0; q < CPT; ++q) acc[r][q] = 0.f;

    const uint64_t nblk = (n + kRowSamples - 1) / kRowSamples;
    for (uint64_t blk = 0; blk < nblk; ++blk) {
        __syncthreads();
        for (int e = tid; e < kRowSnps * 8; e += 256) {
            const int r = e >> 3, w = e & 7;
            const uint64_t j = j0 + r;
            codes[r][w] = j < p ? reinterpret_cast<const uint32_t*>(packed + j * stride + blk * 32)[w] : 0u;
        }
        const float4* Wsrc = reinterpret_cast<const float4*>(W + blk * kRowSamples * WP);
        for (int e = tid; e < kRowSamples * WP / 4; e += 256) smem_f4[e] = Wsrc[e];
        __syncthreads();
#pragma unroll 1
        for (int w = 0; w < 8; ++w) {
            uint32_t cw[8];
#pragma unroll
            for (int r = 0; r < 8; ++r) cw[r] = codes[ty * 8 + r][w];
#pragma unroll 4
            for (int k = 0; k < 16; ++k) {
                float wv[CPT];
#pragma unroll
                for (int q = 0; q < CPT; ++q) wv[q] = Ws[(w * 16 + k) * WP + tx + 16 * q];
#pragma unroll
                for (int r = 0; r < 8; ++r) {
                    const float v = luts[ty * 8 + r][(cw[r] >> (2 * k)) & 3u];
#pragma unroll
                    for (int q = 0; q < CPT; ++q) acc[r][q] = fmaf(v, wv[q], acc[r][q]);
                }
            }
        }
    }
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const uint64_t j = j0 + ty * 8 + r;
        if (j < p) {
#pragma unroll
            for (int q = 0; q < CPT; ++q) out[j * WP + tx + 16 * q] = acc[r][q];
        }
    }
}

constexpr int kColSamples = 128; // samples per CTA (32 bytes per SNP row)
constexpr int kColSnps = 32;     // SNPs per smem stage

// part[split, i, c] = sum_{j in split} lut_j[code_ij] * Q[j, c]; Q is p x WP.
// 256 threads = 32 sample groups (one byte = 4 samples) x 8 column lanes.
template <int CPT>
__global__ void __launch_bounds__(256) k_col_lut(const uint8_t* __restrict__ packed, uint64_t stride,
                                                 uint64_t p, uint64_t n_pad,
                                                 const float4* __restrict__ lut,
                                                 const float* __restrict__ Q, uint64_t per_split,
                                                 float* __restrict__ part) {
    constexpr int WP = CPT * 8;
    __shared__ float Qs[kColSnps][WP];
    __shared__ uint32_t codes[kColSnps][8];
    __shared__ float luts[kColSnps][4];
    const int tid = threadIdx.x;
    const int tg = tid >> 3, tq = tid & 7;
    const uint64_t tile = blockIdx.x;
    const uint64_t s0 = (uint64_t)blockIdx.y * per_split;
    const uint64_t s1 = min(p, s0 + per_split);
    float acc[4][CPT];
#pragma unroll
    for (int s = 0; s < 4; ++s)
#pragma unroll
        for (int q = 0; q < CPT; ++q) acc[s][q] = 0.f;

    for (uint64_t j0 = s0; j0 < s1; j0 += kColSnps) {
        __syncthreads();
        {
            const int r = tid >> 3, w = tid & 7;
            const uint64_t j = j0 + r;
            codes[r][w] = j < s1 ? reinterpret_cast<const uint32_t*>(packed + j * stride + tile * 32)[w] : 0u;
        }
        if (tid < kColSnps) {
            const uint64_t j = j0 + tid;
            const float4 v = j < s1 ? lut[j] : make_float4(0.f, 0.f, 0.f, 0.f);
            luts[tid][0] = v.x; luts[tid][1] = v.y; luts[tid][2] = v.z; luts[tid][3] = v.w;
        }
        for (int e = tid; e < kColSnps * WP; e += 256) {
            const int r = e / WP, cc = e - r * WP;
            const uint64_t j = j0 + r;
            Qs[r][cc] = j < s1 ? Q[j * WP + cc] : 0.f;
        }
        __syncthreads();
#pragma unroll 4
        for (int jj = 0; jj < kColSnps; ++jj) {
            const uint32_t b = (codes[jj][tg >> 2] >> (8 * (tg & 3))) & 0xffu;
            float qv[CPT];
#pragma unroll
            for (int q = 0; q < CPT; ++q) qv[q] = Qs[jj][tq + 8 * q];
#pragma unroll
            for (int s = 0; s < 4; ++s) {
                const float v = luts[jj][(b >> (2 * s)) & 3u];
#pragma unroll
                for (int q = 0; q < CPT; ++q) acc[s][q] = fmaf(v, qv[q], acc[s][q]);
            }
        }
    }
    float* dst = part + (uint64_t)blockIdx.y * n_pad * WP;
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        const uint64_t i = tile * kColSamples + tg * 4 + s;
#pragma unroll
        for (int q = 0; q < CPT; ++q) dst[i * WP + tq + 8 * q] = acc[s][q];
    }
}

__global__ void k_reduce_splits(const float* __restrict__ part, int splits, uint64_t n, int wp,
                                uint64_t n_pad, double* __restrict__ S) {
    const uint64_t total = n * (uint64_t)wp;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
         t += (uint64_t)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int s = 0; s < splits; ++s) acc += f64_of_f32(part[(uint64_t)s * n_pad * wp + t]);
        S[t] = acc;
    }
}

template <int CPT>
void row_lut_impl(Ctx& c, const Geno& g, const float* lut, const float* W, float* out) {
    constexpr int WP = CPT * 16;
    const size_t smem = (size_t)kRowSamples * WP * sizeof(float);
    raise_dynamic_smem((const void*)k_row_lut<CPT>, smem);
    const unsigned grid = (unsigned)ceil_div(g.p, kRowSnps);
    k_row_lut<CPT><<<grid, 256, smem, c.stream>>>(packed_rows(g), g.stride, g.p, g.n,
                                                  reinterpret_cast<const float4*>(lut), W, out);
    SLFMM_LAUNCHED(c, "k_row_lut");
}

template <int CPT>
void col_lut_impl(Ctx& c, const Geno& g, const float* lut, const float* Q, double* S) {
    constexpr int WP = CPT * 8;
    const uint64_t tiles = ceil_div(g.n, kColSamples);
    const uint64_t n_pad = tiles * kColSamples;
    // split the SNP range so each thread accumulates at most ~16k SNPs in
    // FP32 and the grid fills the device
    uint64_t splits = std::max<uint64_t>(ceil_div(g.p, 16384),
                                         ceil_div((uint64_t)c.sm_count * 4, tiles));
    splits = std::max<uint64_t>(1, std::min<uint64_t>(splits, std::max<uint64_t>(1, ceil_div(g.p, kColSnps))));
    const uint64_t per_split = round_up(ceil_div(g.p, splits), kColSnps);
    splits = ceil_div(g.p, per_split);
    DBuf<float> part(splits * n_pad * WP, c.stream);
    dim3 grid((unsigned)tiles, (unsigned)splits);
    k_col_lut<CPT><<<grid, 256, 0, c.stream>>>(packed_rows(g), g.stride, g.p, n_pad,
                                               reinterpret_cast<const float4*>(lut), Q, per_split,
                                               part.get());
    SLFMM_LAUNCHED(c, "k_col_lut");
    k_reduce_splits<<<grid_for(c, g.n * WP, 256), 256, 0, c.stream>>>(part.get(), (int)splits, g.n,
                                                                     WP, n_pad, S);
    SLFMM_LAUNCHED(c, "k_reduce_splits");
}

}  // namespace

void launch_reduce_splits(Ctx& c, const float* part, int splits, uint64_t n, int wp, uint64_t n_pad, double* S) {
    if (!n) return;
    k_reduce_splits<<<grid_for(c, n * wp, 256), 256, 0, c.stream>>>(part, splits, n, wp, n_pad, S);
    SLFMM_LAUNCHED(c, "k_reduce_splits");
}

void launch_row_lut(Ctx& c, const Geno& g, const float* lut, const float* W, int wp, float* out) {
    if (g.p == 0) return;
    switch (wp) {
        case 16: row_lut_impl<1>(c, g, lut, W, out); break;
        case 32: row_lut_impl<2>(c, g, lut, W, out); break;
        case 48: row_lut_impl<3>(c, g, lut, W, out); break;
        case 64: row_lut_impl<4>(c, g, lut, W, out); break;
        case 80: row_lut_impl<5>(c, g, lut, W, out); break;
        case 96: row_lut_impl<6>(c, g, lut, W, out); break;
        case 112: row_lut_impl<7>(c, g, lut, W, out); break;
        case 128: row_lut_impl<8>(c, g, lut, W, out); break;
        default: throw Error(SLFMM_ERR_BAD_ARG, "row contraction width must be a multiple of 16 <= 128");
    }
}

void launch_col_lut(Ctx& c, const Geno& g, const float* lut, const float* Q, int wp, double* S) {
    if (g.n == 0) return;
    if (g.p == 0) { SLFMM_CUDA(cudaMemsetAsync(S, 0, g.n * wp * sizeof(double), c.stream)); return; }
    switch (wp) {
        case 16: col_lut_impl<2>(c, g, lut, Q, S); break;
        case 32: col_lut_impl<4>(c, g, lut, Q, S); break;
        case 48: col_lut_impl<6>(c, g, lut, Q, S); break;
        case 64: col_lut_impl<8>(c, g, lut, Q, S); break;
        case 80: col_lut_impl<10>(c, g, lut, Q, S); break;
        case 96: col_lut_impl<12>(c, g, lut, Q, S); break;
        case 112: col_lut_impl<14>(c, g, lut, Q, S); break;
        case 128: col_lut_impl<16>(c, g, lut, Q, S); break;
        default: throw Error(SLFMM_ERR_BAD_ARG, "column contraction width must be a multiple of 16 <= 128");
    }
}

}  // namespace slfmm
