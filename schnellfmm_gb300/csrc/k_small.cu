// FP64 dense helpers for the small / tall-skinny linear algebra of the path:
// covariate centring (src/lib.rs:102-117), Step 0 (src/precompute.rs:30-88),
// Cholesky-QR2 of the sketches (replacing the LAPACK QR of
// src/rsvd.rs:75,105,131), the small SVD (src/rsvd.rs:162, src/nmf.rs:321)
// and safe_inv (src/testing.rs:996-1024).  GB300's FP64 rate is low, so
// these only ever touch n x w, w x w or p x w objects with tiny w.
#include "slfmm_internal.h"

namespace slfmm {
namespace {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// block-wide sum with a fixed reduction order (deterministic)
__device__ double block_sum(double v, double* red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    double t = 0.0;
    if (wid == 0) {
        t = lane < nw ? red[lane] : 0.0;
        t = warp_sum(t);
    }
    __syncthreads();
    if (threadIdx.x == 0) red[0] = t;
    __syncthreads();
    const double r = red[0];
    __syncthreads();
    return r;
}

__global__ void k_colmeans(const double* __restrict__ A, uint64_t m, int lda, double* __restrict__ out,
                           int divide) {
    __shared__ double red[32];
    const int col = blockIdx.x;
    double s = 0.0;
    for (uint64_t i = threadIdx.x; i < m; i += blockDim.x) s += A[i * lda + col];
    s = block_sum(s, red);
    if (threadIdx.x == 0) out[col] = divide ? (m ? s / (double)m : 0.0) : s;
}

__global__ void k_center_cols(double* __restrict__ A, uint64_t m, int a, int lda,
                              const double* __restrict__ means) {
    const uint64_t total = m * a;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
         t += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = t / a;
        const int c = (int)(t - i * a);
        A[i * lda + c] -= means[c];
    }
}

// divide a column by its sample sd (n-1 denominator) unless sd <= 1e-14
__global__ void k_scale_cols_sd(double* __restrict__ A, uint64_t m, int lda) {
    __shared__ double red[32];
    const int col = blockIdx.x;
    double s = 0.0;
    for (uint64_t i = threadIdx.x; i < m; i += blockDim.x) {
        const double v = A[i * lda + col];
        s += v * v;
    }
    s = block_sum(s, red);
    const double sd = sqrt(s / ((double)m - 1.0));
    if (sd > 1e-14)
        for (uint64_t i = threadIdx.x; i < m; i += blockDim.x) A[i * lda + col] /= sd;
}

// Tiled A^T B over a row range: 32x32 output tile per CTA, 16x16 threads,
// FP64 accumulation; partial[split] written, reduced by k_sum_partials.
template <typename T>
__global__ void __launch_bounds__(256) k_atb(const T* __restrict__ A, int lda, const T* __restrict__ B,
                                             int ldb, uint64_t m, int a, int b, uint64_t rows_per_split,
                                             double* __restrict__ part) {
    __shared__ double As[32][33];
    __shared__ double Bs[32][33];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
    const uint64_t i0 = (uint64_t)blockIdx.z * rows_per_split;
    const uint64_t i1 = min(m, i0 + rows_per_split);
    double acc[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
    for (uint64_t ib = i0; ib < i1; ib += 32) {
        __syncthreads();
        for (int e = threadIdx.x; e < 32 * 32; e += 256) {
            const int ii = e >> 5, cc = e & 31;
            const uint64_t i = ib + ii;
            As[ii][cc] = (i < i1 && r0 + cc < a) ? (double)A[i * lda + r0 + cc] : 0.0;
            Bs[ii][cc] = (i < i1 && c0 + cc < b) ? (double)B[i * ldb + c0 + cc] : 0.0;
        }
        __syncthreads();
#pragma unroll 8
        for (int ii = 0; ii < 32; ++ii) {
            const double a0 = As[ii][ty], a1 = As[ii][ty + 16];
            const double b0 = Bs[ii][tx], b1 = Bs[ii][tx + 16];
            acc[0][0] = fma(a0, b0, acc[0][0]);
            acc[0][1] = fma(a0, b1, acc[0][1]);
            acc[1][0] = fma(a1, b0, acc[1][0]);
            acc[1][1] = fma(a1, b1, acc[1][1]);
        }
    }
    double* dst = part + (uint64_t)blockIdx.z * a * b;
#pragma unroll
    for (int u = 0; u < 2; ++u)
#pragma unroll
        for (int v = 0; v < 2; ++v) {
            const int r = r0 + ty + 16 * u, cc = c0 + tx + 16 * v;
            if (r < a && cc < b) dst[r * b + cc] = acc[u][v];
        }
}

// A^T B over a row range with the a x b outputs laid flat: thread t of the
// CTA owns outputs o0 + t + 256 k (k < R), rows of A and B are staged 32 at
// a time in shared memory, and every FMA issued is one of the a x b (the
// 32 x 32 output tiles of k_atb spend 39-61 % of their FP64 FMAs on padding
// at the widths used here: 20, 50, 71).  FP64 accumulation in row order
// within the range; partial[split] written, reduced by k_sum_partials.
template <typename T, int R>
__global__ void __launch_bounds__(256) k_atb_flat(const T* __restrict__ A, int lda, const T* __restrict__ B,
                                                  int ldb, uint64_t m, int a, int b, uint64_t rows_per_split,
                                                  double* __restrict__ part) {
    extern __shared__ double stage[];
    double* As = stage;             // [32][a]
    double* Bs = stage + 32 * a;    // [32][b]
    const int tid = threadIdx.x;
    const int ab = a * b;
    const int o0 = blockIdx.x * 256 * R;
    const uint64_t i0 = (uint64_t)blockIdx.y * rows_per_split;
    const uint64_t i1 = min(m, i0 + rows_per_split);
    int ra[R], cb[R];
    double acc[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int o = o0 + tid + 256 * k;
        ra[k] = o < ab ? o / b : 0;
        cb[k] = o < ab ? o % b : 0;
        acc[k] = 0.0;
    }
    // warp-uniform: the last k with an output in this warp
    const int wfirst = o0 + (tid & ~31);
    for (uint64_t ib = i0; ib < i1; ib += 32) {
        __syncthreads();
        for (int e = tid; e < 32 * a; e += 256) {
            const int ii = e / a, cc = e % a;
            const uint64_t i = ib + ii;
            As[e] = i < i1 ? (double)A[i * lda + cc] : 0.0;
        }
        for (int e = tid; e < 32 * b; e += 256) {
            const int ii = e / b, cc = e % b;
            const uint64_t i = ib + ii;
            Bs[e] = i < i1 ? (double)B[i * ldb + cc] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < R; ++k) {
            if (wfirst + 256 * k >= ab) break;
#pragma unroll 8
            for (int ii = 0; ii < 32; ++ii) acc[k] = fma(As[ii * a + ra[k]], Bs[ii * b + cb[k]], acc[k]);
        }
    }
    double* dst = part + (uint64_t)blockIdx.y * ab;
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int o = o0 + tid + 256 * k;
        if (o < ab) dst[o] = acc[k];
    }
}

// FP32 Gram with FP32 products summed over 32-row tiles and FP64 across
// tiles (used for the p x l sketches, whose FP64 Gram would dominate).
__global__ void __launch_bounds__(256) k_gram_f32(const float* __restrict__ A, int lda, uint64_t m, int a,
                                                  uint64_t rows_per_split, double* __restrict__ part) {
    __shared__ float As[32][33];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
    const uint64_t i0 = (uint64_t)blockIdx.z * rows_per_split;
    const uint64_t i1 = min(m, i0 + rows_per_split);
    __shared__ float Bs[32][33];
    double acc[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
    for (uint64_t ib = i0; ib < i1; ib += 32) {
        __syncthreads();
        for (int e = threadIdx.x; e < 32 * 32; e += 256) {
            const int ii = e >> 5, cc = e & 31;
            const uint64_t i = ib + ii;
            As[ii][cc] = (i < i1 && r0 + cc < a) ? A[i * lda + r0 + cc] : 0.f;
            Bs[ii][cc] = (i < i1 && c0 + cc < a) ? A[i * lda + c0 + cc] : 0.f;
        }
        __syncthreads();
        float t[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
#pragma unroll 8
        for (int ii = 0; ii < 32; ++ii) {
            const float a0 = As[ii][ty], a1 = As[ii][ty + 16];
            const float b0 = Bs[ii][tx], b1 = Bs[ii][tx + 16];
            t[0][0] = fmaf(a0, b0, t[0][0]);
            t[0][1] = fmaf(a0, b1, t[0][1]);
            t[1][0] = fmaf(a1, b0, t[1][0]);
            t[1][1] = fmaf(a1, b1, t[1][1]);
        }
#pragma unroll
        for (int u = 0; u < 2; ++u)
#pragma unroll
            for (int v = 0; v < 2; ++v) acc[u][v] += (double)t[u][v];
    }
    double* dst = part + (uint64_t)blockIdx.z * a * a;
#pragma unroll
    for (int u = 0; u < 2; ++u)
#pragma unroll
        for (int v = 0; v < 2; ++v) {
            const int r = r0 + ty + 16 * u, cc = c0 + tx + 16 * v;
            if (r < a && cc < a) dst[r * a + cc] = acc[u][v];
        }
}

// Elements 4 q .. 4 q + 3 of a row (16-byte aligned, 4 q < lda), the ones at
// or past column a zero (no load when the whole quad is past a).
__device__ __forceinline__ float4 row_quad(const float* row, int q, int a) {
    if (4 * q >= a) return make_float4(0.f, 0.f, 0.f, 0.f);
    float4 b = reinterpret_cast<const float4*>(row)[q];
    if (4 * q + 4 > a) {
        b.y = 4 * q + 1 < a ? b.y : 0.f;
        b.z = 4 * q + 2 < a ? b.z : 0.f;
        b.w = 4 * q + 3 < a ? b.w : 0.f;
    }
    return b;
}

// Narrow (a <= 32) FP32 Gram, one warp per run of rows: lane c holds row
// element c and takes row[k] by shuffle.  FP32 sums over runs of 256 rows,
// FP64 across runs; the block's warps reduce through shared memory into one
// partial.  (Rows of any stride; the tiled kernel below covers 16-byte
// aligned rows of at most 32 floats.)
constexpr int kGramRun = 256;
constexpr size_t kGramNarrowSmem = 8 * 32 * 33 * sizeof(double);
__global__ void __launch_bounds__(256, 2) k_gram_narrow(const float* __restrict__ A, int lda, uint64_t m, int a,
                                                        double* __restrict__ part) {
    extern __shared__ double gsm[];  // [8 warps][32][33] FP64 sums
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double* mine = gsm + warp * 32 * 33;
#pragma unroll
    for (int k = 0; k < 32; ++k) mine[k * 33 + lane] = 0.0;
    const uint64_t nruns = (m + kGramRun - 1) / kGramRun;
    for (uint64_t run = (uint64_t)blockIdx.x * 8 + warp; run < nruns; run += (uint64_t)gridDim.x * 8) {
        float acc[32];
#pragma unroll
        for (int k = 0; k < 32; ++k) acc[k] = 0.f;
        const uint64_t i0 = run * kGramRun, i1 = min(m, i0 + kGramRun);
        for (uint64_t i = i0; i < i1; i += 8) {
            float v[8];  // eight rows in flight per warp
#pragma unroll
            for (int u = 0; u < 8; ++u) v[u] = (lane < a && i + u < i1) ? A[(i + u) * lda + lane] : 0.f;
#pragma unroll
            for (int u = 0; u < 8; ++u)
#pragma unroll
                for (int k = 0; k < 32; ++k) acc[k] = fmaf(__shfl_sync(0xffffffffu, v[u], k), v[u], acc[k]);
        }
#pragma unroll
        for (int k = 0; k < 32; ++k) mine[k * 33 + lane] += (double)acc[k];
    }
    __syncthreads();
    // warps summed in a fixed order (deterministic)
    double* dst = part + (uint64_t)blockIdx.x * a * a;
    for (int e = threadIdx.x; e < a * a; e += blockDim.x) {
        const int k = e / a, cc = e % a;
        double t = 0.0;
        for (int w = 0; w < 8; ++w) t += gsm[w * 32 * 33 + k * 33 + cc];
        dst[e] = t;
    }
}

// A (m x a, a <= 32) <- A Linv^T in place, one warp per row: lane c holds
// column c of Linv^T (FP32) and accumulates out[c] = sum_k row[k] Linv[c][k]
// from the broadcast row elements; loads and stores are whole rows.
__global__ void __launch_bounds__(256) k_trmul_narrow(float* __restrict__ A, int lda, uint64_t m, int a,
                                                      const double* __restrict__ Linv) {
    const int lane = threadIdx.x & 31;
    float R[32];
#pragma unroll
    for (int k = 0; k < 32; ++k) R[k] = (k < a && lane < a) ? (float)Linv[lane * a + k] : 0.f;
    // each warp takes runs of 4 consecutive rows (four loads in flight)
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t i = ((uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 4; i < m; i += warps * 4) {
        float v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) v[u] = (lane < a && i + u < m) ? A[(i + u) * lda + lane] : 0.f;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            float out = 0.f;
#pragma unroll
            for (int k = 0; k < 32; ++k) out = fmaf(__shfl_sync(0xffffffffu, v[u], k), R[k], out);
            if (lane < a && i + u < m) A[(i + u) * lda + lane] = out;
        }
    }
}

// Tiles of 128 rows of a narrow matrix (a <= lda <= 32, lda % 4 == 0, rows
// 16-byte aligned) stream through a ring of kPipe shared-memory stages with
// asynchronous 16-byte copies (cp.async, completion awaited by wait_group):
// tile i + kPipe - 1 is in flight while tile i is used.  One persistent block
// of 512 threads per SM takes tiles blockIdx.x, + gridDim.x, ...; each of its
// 16 warps uses 8 rows of a tile.  Rows past m are neither copied nor used.
__device__ __forceinline__ uint32_t smem_addr32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

constexpr int kNarrowTile = 128;
constexpr int kPipe = 4;
constexpr int kPipeThreads = 512;
constexpr size_t kPipeRing = (size_t)kPipe * kNarrowTile * 32 * sizeof(float);

__device__ __forceinline__ void pipe_issue(const float* A, int lda, uint64_t m, uint64_t t, float* stage) {
    const int q = lda >> 2, nf4 = kNarrowTile * q;
    const float4* src = reinterpret_cast<const float4*>(A) + t * kNarrowTile * q;
    const uint64_t rows = min((uint64_t)kNarrowTile, m - t * kNarrowTile);
#pragma unroll
    for (int r = 0; r < 1024 / kPipeThreads; ++r) {
        const int e = threadIdx.x + kPipeThreads * r;
        if (e < nf4 && (uint64_t)(e / q) < rows)
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr32(stage + 4 * e)), "l"(src + e)
                         : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

__device__ __forceinline__ void pipe_commit_empty() { asm volatile("cp.async.commit_group;" ::: "memory"); }

// wait for tile i (its copy group) and make every thread's copies visible
__device__ __forceinline__ void pipe_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(kPipe - 2) : "memory");
    __syncthreads();
}

// Gram over tiles: lane = 8 ky + cx of each warp owns the block
// G[8 ky + i][4 cx + j] (i < 8, j < 4) and reads its 12 row elements as three
// 16-byte shared-memory loads per row.  Elements past column a (padding, or
// the next row when lda < 32) only reach entries that are never written out.
// FP32 sums over up to 16 tiles, then into per-warp FP64 sums in shared
// memory; the warps are added in a fixed order into one partial per block.
__global__ void __launch_bounds__(kPipeThreads, 1) k_gram_tile(const float* __restrict__ A, int lda, uint64_t m, int a,
                                                            double* __restrict__ part) {
    extern __shared__ __align__(16) float ring[];  // [kPipe][128 rows][lda], then [16 warps][32][32] FP64
    double* dsum = reinterpret_cast<double*>(reinterpret_cast<uint8_t*>(ring) + kPipeRing);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int ky = lane >> 3, cx = lane & 7;
    double* mine = dsum + warp * 32 * 32;  // [entry][lane]
#pragma unroll
    for (int k = 0; k < 32; ++k) mine[k * 32 + lane] = 0.0;
    const uint64_t ntiles = (m + kNarrowTile - 1) / kNarrowTile;
    const int tsz = kNarrowTile * lda;
    float acc[32];
#pragma unroll
    for (int k = 0; k < 32; ++k) acc[k] = 0.f;
    for (int k = 0; k < kPipe - 1; ++k) {
        const uint64_t t = blockIdx.x + (uint64_t)k * gridDim.x;
        if (t < ntiles) pipe_issue(A, lda, m, t, ring + k * tsz);
        else pipe_commit_empty();
    }
    int since = 0;
    for (uint64_t i = 0;; ++i) {
        const uint64_t t = blockIdx.x + i * gridDim.x;
        if (t >= ntiles) break;
        pipe_wait();
        const uint64_t tn = t + (uint64_t)(kPipe - 1) * gridDim.x;
        if (tn < ntiles) pipe_issue(A, lda, m, tn, ring + ((i + kPipe - 1) % kPipe) * tsz);
        else pipe_commit_empty();
        const int r0 = warp * 8;
        const uint64_t gr = t * kNarrowTile + r0;
        const int nrows = gr >= m ? 0 : (m - gr >= 8 ? 8 : (int)(m - gr));
        const float* base = ring + (i % kPipe) * tsz + r0 * lda;
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            if (u < nrows) {
                const float4* row = reinterpret_cast<const float4*>(base + u * lda);
                const float4 ka = row[2 * ky], kb = row[2 * ky + 1], cv = row[cx];
                const float kk[8] = {ka.x, ka.y, ka.z, ka.w, kb.x, kb.y, kb.z, kb.w};
                const float cc[4] = {cv.x, cv.y, cv.z, cv.w};
#pragma unroll
                for (int ii = 0; ii < 8; ++ii)
#pragma unroll
                    for (int jj = 0; jj < 4; ++jj) acc[ii * 4 + jj] = fmaf(kk[ii], cc[jj], acc[ii * 4 + jj]);
            }
        }
        if (++since == 32) {
#pragma unroll
            for (int k = 0; k < 32; ++k) mine[k * 32 + lane] += (double)acc[k], acc[k] = 0.f;
            since = 0;
        }
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 32; ++k) mine[k * 32 + lane] += (double)acc[k];
    __syncthreads();
    // entry (k, c) of the block partial: lane 8 (k / 8) + c / 4, slot (k % 8) 4 + c % 4
    for (int e = threadIdx.x; e < a * a; e += kPipeThreads) {
        const int k = e / a, c = e % a;
        const int ln = 8 * (k >> 3) + (c >> 2), slot = (k & 7) * 4 + (c & 3);
        double tsum = 0.0;
        for (int w = 0; w < kPipeThreads / 32; ++w) tsum += dsum[w * 32 * 32 + slot * 32 + ln];
        part[(uint64_t)blockIdx.x * a * a + e] = tsum;
    }
}

// A (m x a, a <= 32, lda % 4 == 0, rows 16-byte aligned) <- A Linv^T in
// place for a lower-triangular Linv, one row per thread: the row is read as
// 16-byte loads (elements past a zero), out[c] = sum_{k <= c} row[k] R[c][k]
// with R = Linv in FP32 passed as a kernel parameter -- every FMA takes its R
// operand from the constant bank, the same for the whole warp -- and the row
// is written back.
struct Mat32 {
    float v[32][32];
};
__global__ void __launch_bounds__(256) k_trmul_rows(float* __restrict__ A, int lda, uint64_t m, int a,
                                                    const __grid_constant__ Mat32 R) {
    for (uint64_t i = (uint64_t)blockIdx.x * 256 + threadIdx.x; i < m; i += (uint64_t)gridDim.x * 256) {
        float* row = A + i * lda;
        float x[32];
#pragma unroll
        for (int kq = 0; kq < 8; ++kq) {
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (4 * kq < a) {
                v = reinterpret_cast<const float4*>(row)[kq];
                if (4 * kq + 4 > a) {
                    v.y = 4 * kq + 1 < a ? v.y : 0.f;
                    v.z = 4 * kq + 2 < a ? v.z : 0.f;
                    v.w = 4 * kq + 3 < a ? v.w : 0.f;
                }
            }
            x[4 * kq] = v.x;
            x[4 * kq + 1] = v.y;
            x[4 * kq + 2] = v.z;
            x[4 * kq + 3] = v.w;
        }
        float o[32];
#pragma unroll
        for (int c = 0; c < 32; ++c) o[c] = 0.f;
        // Linv is lower triangular: R[c][k] = 0 for k > c (528 products)
#pragma unroll
        for (int k = 0; k < 32; ++k)
#pragma unroll
            for (int c = k; c < 32; ++c) o[c] = fmaf(x[k], R.v[c][k], o[c]);
#pragma unroll
        for (int cq = 0; cq < 8; ++cq) {
            if (4 * cq + 4 <= a) {
                reinterpret_cast<float4*>(row)[cq] = make_float4(o[4 * cq], o[4 * cq + 1], o[4 * cq + 2], o[4 * cq + 3]);
            } else if (4 * cq < a) {
#pragma unroll
                for (int jj = 0; jj < 4; ++jj)
                    if (4 * cq + jj < a) row[4 * cq + jj] = o[4 * cq + jj];
            }
        }
    }
}

// one block per entry: thread t sums partials t, t + 128, ... in order, then
// a fixed-shape tree (warp shuffles, then the four warps in order)
__global__ void __launch_bounds__(128) k_sum_partials_wide(const double* __restrict__ part, int splits,
                                                           uint64_t count, double* __restrict__ out) {
    __shared__ double ws[4];
    for (uint64_t e = blockIdx.x; e < count; e += gridDim.x) {
        double s = 0.0;
        for (int k = threadIdx.x; k < splits; k += 128) s += part[(uint64_t)k * count + e];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x == 0) out[e] = (ws[0] + ws[1]) + (ws[2] + ws[3]);
        __syncthreads();
    }
}

__global__ void k_sum_partials(const double* __restrict__ part, int splits, uint64_t count,
                               double* __restrict__ out) {
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < count;
         t += (uint64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int k = 0; k < splits; ++k) s += part[(uint64_t)k * count + t];
        out[t] = s;
    }
}

// C = alpha * A B + beta * C with A (m x a), B (a x b) small; one thread per output.
template <typename TO>
__global__ void k_gemm_small(const double* __restrict__ A, int lda, uint64_t m, int a,
                             const double* __restrict__ B, int ldb, int b, double alpha, double beta,
                             TO* __restrict__ C, int ldc) {
    extern __shared__ double Bsm[];  // a x b
    for (int e = threadIdx.x; e < a * b; e += blockDim.x) Bsm[e] = B[(e / b) * ldb + (e % b)];
    __syncthreads();
    const uint64_t total = m * b;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
         t += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = t / b;
        const int cc = (int)(t - i * b);
        double s = 0.0;
        const double* ar = A + i * lda;
        for (int k = 0; k < a; ++k) s = fma(ar[k], Bsm[k * b + cc], s);
        const double prev = beta != 0.0 ? (double)C[i * ldc + cc] : 0.0;
        C[i * ldc + cc] = (TO)(alpha * s + beta * prev);
    }
}

// A (m x a, FP32) <- A * Linv^T with Linv lower-triangular (a x a, FP64),
// i.e. A <- A R^-1 for the Cholesky factor R = L^T of A^T A.  The row lives
// in registers (fully unrolled up to AMAX columns).
template <int AMAX>
__global__ void __launch_bounds__(128) k_trmul_f32(float* __restrict__ A, int lda, uint64_t m, int a,
                                                   const double* __restrict__ Linv) {
    __shared__ float R[AMAX * AMAX];  // R[k][c] = Linv[c][k], zero padded
    for (int e = threadIdx.x; e < AMAX * AMAX; e += blockDim.x) {
        const int k = e / AMAX, cc = e % AMAX;
        R[e] = (k < a && cc < a) ? (float)Linv[cc * a + k] : 0.f;
    }
    __syncthreads();
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
         i += (uint64_t)gridDim.x * blockDim.x) {
        float row[AMAX], out[AMAX];
        float* ar = A + i * lda;
#pragma unroll
        for (int k = 0; k < AMAX; ++k) {
            row[k] = k < a ? ar[k] : 0.f;
            out[k] = 0.f;
        }
#pragma unroll
        for (int k = 0; k < AMAX; ++k)
#pragma unroll
            for (int cc = k; cc < AMAX; ++cc) out[cc] = fmaf(row[k], R[k * AMAX + cc], out[cc]);
#pragma unroll
        for (int k = 0; k < AMAX; ++k)
            if (k < a) ar[k] = out[k];
    }
}

// In-place Cholesky (lower) of an a x a SPD matrix in one CTA.  status[0] =
// number of pivots that were not positive (replaced by a tiny positive value).
// With drop_tol >= 0 a column whose residual pivot is <= drop_tol times its
// original diagonal is dropped instead: L_kk = 1, L_ik = 0, dropped[k] = 1
// (rank-deficient design columns).  status[0] counts replaced/dropped pivots.
__global__ void k_cholesky(double* __restrict__ G, int a, int* __restrict__ status,
                           double drop_tol, int* __restrict__ dropped, double* __restrict__ work) {
    extern __shared__ double S_sm[];
    double* S = work ? work : S_sm;   // global scratch for matrices wider than kMaxSmall
    __shared__ double piv;
    __shared__ int bad;
    __shared__ int drop_k;
    for (int e = threadIdx.x; e < a * a; e += blockDim.x) S[e] = G[e];
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    double dmax = 0.0;
    for (int k = 0; k < a; ++k) dmax = fmax(dmax, fabs(S[k * a + k]));
    for (int k = 0; k < a; ++k) {
        if (threadIdx.x == 0) {
            double v = S[k * a + k];
            drop_k = 0;
            if (drop_tol >= 0.0) {
                if (!(v > drop_tol * fabs(G[k * a + k])) || !(v > 1e-300)) { drop_k = 1; ++bad; v = 1.0; }
            } else if (!(v > 1e-300 + 1e-28 * dmax)) {
                v = 1e-28 * dmax + 1e-300;
                ++bad;
            }
            if (dropped) dropped[k] = drop_k;
            piv = sqrt(v);
            S[k * a + k] = piv;
        }
        __syncthreads();
        for (int i = k + 1 + threadIdx.x; i < a; i += blockDim.x) S[i * a + k] = drop_k ? 0.0 : S[i * a + k] / piv;
        __syncthreads();
        const int rem = a - k - 1;
        for (int e = threadIdx.x; e < rem * rem; e += blockDim.x) {
            const int i = k + 1 + e / rem, j = k + 1 + e % rem;
            if (j <= i) S[i * a + j] -= S[i * a + k] * S[j * a + k];
        }
        __syncthreads();
    }
    for (int e = threadIdx.x; e < a * a; e += blockDim.x) {
        const int i = e / a, j = e % a;
        G[e] = j <= i ? S[e] : 0.0;
    }
    if (threadIdx.x == 0 && status) status[0] = bad;
}

// Inverse of a lower-triangular matrix: one thread per column.
__global__ void k_tri_inv_lower(const double* __restrict__ L, int a, double* __restrict__ X, int in_smem) {
    extern __shared__ double S_sm[];
    const double* S = in_smem ? S_sm : L;   // matrices wider than kMaxSmall are read in place
    if (in_smem) {
        for (int e = threadIdx.x; e < a * a; e += blockDim.x) S_sm[e] = L[e];
        __syncthreads();
    }
    for (int cc = threadIdx.x; cc < a; cc += blockDim.x) {
        for (int i = 0; i < cc; ++i) X[i * a + cc] = 0.0;
        for (int i = cc; i < a; ++i) {
            double s = (i == cc) ? 1.0 : 0.0;
            for (int k = cc; k < i; ++k) s -= S[i * a + k] * X[k * a + cc];
            X[i * a + cc] = s / S[i * a + i];
        }
    }
}

// LU with partial pivoting in smem; returns 0 if an exactly zero pivot was met.
__device__ bool lu_smem(double* S, int* piv, int a) {
    __shared__ int p_sh;
    __shared__ int ok;
    if (threadIdx.x == 0) ok = 1;
    __syncthreads();
    for (int k = 0; k < a; ++k) {
        if (threadIdx.x == 0) {
            int p = k;
            double best = fabs(S[k * a + k]);
            for (int i = k + 1; i < a; ++i) {
                const double v = fabs(S[i * a + k]);
                if (v > best) { best = v; p = i; }
            }
            p_sh = p;
            piv[k] = p;
            if (best == 0.0) ok = 0;
        }
        __syncthreads();
        if (!ok) return false;
        const int p = p_sh;
        if (p != k)
            for (int j = threadIdx.x; j < a; j += blockDim.x) {
                const double t = S[k * a + j];
                S[k * a + j] = S[p * a + j];
                S[p * a + j] = t;
            }
        __syncthreads();
        const double d = S[k * a + k];
        for (int i = k + 1 + threadIdx.x; i < a; i += blockDim.x) S[i * a + k] /= d;
        __syncthreads();
        const int rem = a - k - 1;
        for (int e = threadIdx.x; e < rem * rem; e += blockDim.x) {
            const int i = k + 1 + e / rem, j = k + 1 + e % rem;
            S[i * a + j] -= S[i * a + k] * S[k * a + j];
        }
        __syncthreads();
    }
    return true;
}

// safe_inv (src/testing.rs:996-1024): invert; on an exactly zero pivot add
// eps = 1e-8 * max(max|diag|, 1e-300) to the diagonal and retry.
// status: 0 ok, 1 regularised, 2 failed.  eps_used[0] = eps (0 if none).
// Matrices wider than kMaxSmall work in `work` (a x a doubles then a ints,
// global memory) instead of shared memory.
__global__ void k_inverse(const double* __restrict__ A, int a, double* __restrict__ X,
                          int* __restrict__ status, double* __restrict__ eps_used, double* __restrict__ work) {
    extern __shared__ double S_sm[];
    __shared__ int piv_sm[kMaxSmall];
    double* S = work ? work : S_sm;
    int* piv = work ? reinterpret_cast<int*>(work + (size_t)a * a) : piv_sm;
    __shared__ double eps;
    for (int attempt = 0; attempt < 2; ++attempt) {
        if (threadIdx.x == 0) {
            double dmax = 0.0;
            for (int k = 0; k < a; ++k) dmax = fmax(dmax, fabs(A[k * a + k]));
            dmax = fmax(dmax, 1e-300);
            eps = attempt == 0 ? 0.0 : 1e-8 * dmax;
        }
        __syncthreads();
        for (int e = threadIdx.x; e < a * a; e += blockDim.x)
            S[e] = A[e] + ((e / a == e % a) ? eps : 0.0);
        __syncthreads();
        if (lu_smem(S, piv, a)) {
            // solve for each unit vector: one thread per column
            for (int cc = threadIdx.x; cc < a; cc += blockDim.x) {
                double* x = X;  // column cc written strided
                // b = P e_cc
                for (int i = 0; i < a; ++i) x[i * a + cc] = (i == cc) ? 1.0 : 0.0;
                for (int k = 0; k < a; ++k) {
                    const int p = piv[k];
                    if (p != k) {
                        const double t = x[k * a + cc];
                        x[k * a + cc] = x[p * a + cc];
                        x[p * a + cc] = t;
                    }
                }
                for (int i = 0; i < a; ++i) {
                    double s = x[i * a + cc];
                    for (int k = 0; k < i; ++k) s -= S[i * a + k] * x[k * a + cc];
                    x[i * a + cc] = s;
                }
                for (int i = a - 1; i >= 0; --i) {
                    double s = x[i * a + cc];
                    for (int k = i + 1; k < a; ++k) s -= S[i * a + k] * x[k * a + cc];
                    x[i * a + cc] = s / S[i * a + i];
                }
            }
            if (threadIdx.x == 0) {
                if (status) status[0] = attempt;
                if (eps_used) eps_used[0] = eps;
            }
            return;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        if (status) status[0] = 2;
        if (eps_used) eps_used[0] = eps;
    }
}

// safe_inv by Gauss-Jordan elimination on [A + eps I | I] in shared memory
// (a <= kMaxGaussJordan), every thread of the CTA on each pivot step.  The
// pivot search (first largest |value| in the column, from the diagonal down)
// and the updates of the rows below the pivot are those of lu_smem, so the
// pivots, and the exact-zero test that triggers the eps retry, are the same
// as the LU's; the rows above the pivot are eliminated in the same sweep, so
// the inverse needs no triangular solves.
constexpr int kMaxGaussJordan = 112;  // 16 a^2 bytes of shared memory
__global__ void __launch_bounds__(1024) k_inverse_gj(const double* __restrict__ A, int a, double* __restrict__ X,
                                                     int* __restrict__ status, double* __restrict__ eps_used) {
    extern __shared__ double S[];  // a rows x 2a columns
    __shared__ double f[kMaxGaussJordan];
    __shared__ double eps;
    __shared__ int p_sh, ok;
    const int ld = 2 * a, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int attempt = 0; attempt < 2; ++attempt) {
        if (threadIdx.x == 0) {
            double dmax = 0.0;
            for (int k = 0; k < a; ++k) dmax = fmax(dmax, fabs(A[k * a + k]));
            dmax = fmax(dmax, 1e-300);
            eps = attempt == 0 ? 0.0 : 1e-8 * dmax;
            ok = 1;
        }
        __syncthreads();
        for (int e = threadIdx.x; e < a * ld; e += blockDim.x) {
            const int i = e / ld, j = e % ld;
            S[e] = j < a ? A[i * a + j] + (i == j ? eps : 0.0) : (j - a == i ? 1.0 : 0.0);
        }
        __syncthreads();
        for (int k = 0; k < a; ++k) {
            if (warp == 0) {
                int p = -1;
                double best = -1.0;
                for (int i = k + lane; i < a; i += 32) {
                    const double v = fabs(S[i * ld + k]);
                    if (v > best) { best = v; p = i; }
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    const double ob = __shfl_xor_sync(0xffffffffu, best, o);
                    const int op = __shfl_xor_sync(0xffffffffu, p, o);
                    if (ob > best || (ob == best && op >= 0 && (p < 0 || op < p))) { best = ob; p = op; }
                }
                if (lane == 0) {
                    p_sh = p;
                    if (best == 0.0) ok = 0;
                }
            }
            __syncthreads();
            if (!ok) break;
            const int p = p_sh;
            if (p != k)
                for (int j = k + threadIdx.x; j < ld; j += blockDim.x) {
                    const double t = S[k * ld + j];
                    S[k * ld + j] = S[p * ld + j];
                    S[p * ld + j] = t;
                }
            __syncthreads();
            const double d = S[k * ld + k];
            for (int i = threadIdx.x; i < a; i += blockDim.x) f[i] = i == k ? 0.0 : S[i * ld + k] / d;
            __syncthreads();
            const int span = ld - k - 1;
            for (int e = threadIdx.x; e < a * span; e += blockDim.x) {
                const int i = e / span, j = k + 1 + e % span;
                if (i != k) S[i * ld + j] -= f[i] * S[k * ld + j];
            }
            __syncthreads();
            for (int j = k + 1 + threadIdx.x; j < ld; j += blockDim.x) S[k * ld + j] /= d;
            __syncthreads();
        }
        if (ok) {
            for (int e = threadIdx.x; e < a * a; e += blockDim.x) X[e] = S[(e / a) * ld + a + e % a];
            if (threadIdx.x == 0) {
                if (status) status[0] = attempt;
                if (eps_used) eps_used[0] = eps;
            }
            return;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        if (status) status[0] = 2;
        if (eps_used) eps_used[0] = eps;
    }
}

// One-sided (Hestenes) Jacobi SVD of a square a x a matrix in one
// CTA: A V = U diag(sig).  Outputs V (a x a), sig (descending) and U = A V
// / sig in place of A.  Pairs are rotated in parallel with a round-robin
// ordering, one warp per pair.
//
// GB300 runs FP64 at a small fraction of its FP32 rate, so the sweeps run in
// FP32 first (to ~1e-5 relative orthogonality, at most 12 sweeps); V is then
// re-orthonormalised in FP64 (classical Gram-Schmidt, twice), M = A V formed
// in FP64, and FP64 sweeps polish to the FP64 tolerance -- typically two or
// three, against the ~10 a cold FP64 start needs.
__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// one Jacobi sweep-set on column-major M (ap x ap, rows a used) with
// accumulated V; returns after convergence or max_sweeps
template <typename F>
__device__ void jacobi_sweeps(F* M, F* Vs, int a, int ap, F tol, int max_sweeps, int* rotated, F abs_tol = 0) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    const int npairs = ap / 2;
    for (int sweep = 0; sweep < max_sweeps; ++sweep) {
        if (threadIdx.x == 0) *rotated = 0;
        __syncthreads();
        for (int round = 0; round < ap - 1; ++round) {
            for (int pr = warp; pr < npairs; pr += nwarps) {
                // round-robin tournament: player 0 fixed, the others rotate
                auto pos = [&](int idx) { return idx == 0 ? 0 : 1 + ((idx - 1 + round) % (ap - 1)); };
                int pcol = pos(pr), qcol = pos(ap - 1 - pr);
                if (pcol > qcol) { const int t = pcol; pcol = qcol; qcol = t; }
                F* mp = M + pcol * ap;
                F* mq = M + qcol * ap;
                F al = 0, be = 0, ga = 0;
                for (int r = lane; r < a; r += 32) {
                    al += mp[r] * mp[r];
                    be += mq[r] * mq[r];
                    ga += mp[r] * mq[r];
                }
                if constexpr (sizeof(F) == 8) {
                    al = warp_sum(al); be = warp_sum(be); ga = warp_sum(ga);
                } else {
                    al = warp_sumf(al); be = warp_sumf(be); ga = warp_sumf(ga);
                }
                const F tiny = sizeof(F) == 8 ? (F)1e-300 : (F)1e-37;
                if (fabs(ga) > tol * sqrt(al * be) && fabs(ga) > tiny && fabs(ga) > abs_tol) {
                    const F zeta = (be - al) / (2 * ga);
                    const F t = (zeta >= 0 ? (F)1 : (F)-1) / (fabs(zeta) + sqrt((F)1 + zeta * zeta));
                    const F cs = (F)1 / sqrt((F)1 + t * t), sn = cs * t;
                    for (int r = lane; r < ap; r += 32) {
                        const F x = mp[r], y = mq[r];
                        mp[r] = cs * x - sn * y;
                        mq[r] = sn * x + cs * y;
                        F* vp = Vs + pcol * ap;
                        F* vq = Vs + qcol * ap;
                        const F vx = vp[r], vy = vq[r];
                        vp[r] = cs * vx - sn * vy;
                        vq[r] = sn * vx + cs * vy;
                    }
                    if (lane == 0) *rotated = 1;
                }
            }
            __syncthreads();
        }
        if (!*rotated) break;
        __syncthreads();
    }
}

// classical Gram-Schmidt, twice, of the ap columns of column-major Vs (FP64)
__device__ void gs_columns(double* Vs, int ap, double* dots) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    for (int j = 0; j < ap; ++j) {
        double* vj = Vs + j * ap;
        for (int pass = 0; pass < 2; ++pass) {
            for (int i = warp; i < j; i += nwarps) {
                const double* vi = Vs + i * ap;
                double t = 0.0;
                for (int r = lane; r < ap; r += 32) t += vi[r] * vj[r];
                t = warp_sum(t);
                if (lane == 0) dots[i] = t;
            }
            __syncthreads();
            for (int r = threadIdx.x; r < ap; r += blockDim.x) {
                double t = vj[r];
                for (int i = 0; i < j; ++i) t -= dots[i] * Vs[i * ap + r];
                vj[r] = t;
            }
            __syncthreads();
        }
        if (warp == 0) {
            double t = 0.0;
            for (int r = lane; r < ap; r += 32) t += vj[r] * vj[r];
            t = warp_sum(t);
            const double inv = t > 0.0 ? 1.0 / sqrt(t) : 0.0;
            for (int r = lane; r < ap; r += 32) vj[r] *= inv;
        }
        __syncthreads();
    }
}

// Eigen-decomposition of a symmetric positive semi-definite a x a matrix
// (a <= kMaxDesign; the Gram matrices of Step 0, the RSVD and the NMF probe) in one
// CTA: A V = V diag(sig), sig descending, V orthonormal; A is overwritten by V
// (its left singular vectors).
//
// GB300 runs FP64 at a small fraction of its FP32 rate, so the bulk of the
// rotation work runs as FP32 one-sided Jacobi sweeps (pairs in parallel,
// round-robin order, one warp per pair) to ~1e-5 (at most 12 sweeps: with
// Gram matrices of condition 1e6 and more, FP32 rounding keeps rotating the
// small columns, and the FP64 phase converges quadratically from there
// anyway); V is re-orthonormalised in FP64 (Gram-Schmidt, twice) and
// B = V^T A V formed in FP64.  B is then diagonal up to ~1e-5 of its norm,
// and two-sided cyclic Jacobi sweeps in
// FP64 (Golub & Van Loan, Algorithm 8.5.2 with the parallel round-robin
// ordering) finish it -- quadratic convergence, typically two sweeps --
// accumulating their rotations into R; V <- V R and a final Gram-Schmidt.
// Jacobi rotations are bounded (|tan| <= 1), so clusters of equal or nearly
// equal eigenvalues need no special case.  Eigenvalues are v_j^T A v_j of the
// final vectors.
// Matrices wider than 64 columns work in `ws` (global memory, L2-resident:
// 2 ap^2 doubles + 2 ap^2 floats) instead of shared memory.
__global__ void __launch_bounds__(1024) k_jacobi_svd(double* __restrict__ A, int a,
                                                     double* __restrict__ V, double* __restrict__ sig,
                                                     double* __restrict__ ws) {
    extern __shared__ double sm_dyn[];
    double* sm = ws ? ws : sm_dyn;
    const int ap = a + (a & 1);     // even number of columns (padded column is zero)
    double* M = sm;                 // column-major ap x ap scratch
    double* Vs = sm + ap * ap;      // column-major eigenvectors
    float* M32 = reinterpret_cast<float*>(Vs + ap * ap);
    float* V32 = M32 + ap * ap;
    double* B = reinterpret_cast<double*>(M32);  // reuses the FP32 area after phase 1
    __shared__ int rotated;
    __shared__ double sg[kMaxDesign];
    __shared__ double dots[kMaxDesign];
    __shared__ double bmax;
    __shared__ int order[kMaxDesign];
    __shared__ int jp[kMaxDesign / 2], jq[kMaxDesign / 2];
    __shared__ double jc[kMaxDesign / 2], js[kMaxDesign / 2];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    // phase 1: FP32 sweeps
    for (int e = threadIdx.x; e < ap * ap; e += blockDim.x) {
        const int col = e / ap, row = e % ap;
        M32[e] = (row < a && col < a) ? (float)A[row * a + col] : 0.f;
        V32[e] = (row == col) ? 1.f : 0.f;
    }
    // FP32 resolution of the whole matrix: couplings below 1e-7 of the largest
    // squared column norm are left to the FP64 sweeps (columns of a rank-deficient
    // Gram that are zero up to FP32 rounding would otherwise keep rotating
    // until the sweep limit)
    __shared__ float colmax2;
    if (threadIdx.x == 0) colmax2 = 0.f;
    __syncthreads();
    if (warp < ap) {
        for (int cc = warp; cc < ap; cc += nwarps) {
            float t = 0.f;
            for (int r = lane; r < a; r += 32) t += M32[cc * ap + r] * M32[cc * ap + r];
            t = warp_sumf(t);
            if (lane == 0) atomicMax(reinterpret_cast<int*>(&colmax2), __float_as_int(t));
        }
    }
    __syncthreads();
    jacobi_sweeps<float>(M32, V32, a, ap, 1.0e-5f, 12, &rotated, 1e-7f * colmax2);
    // phase 2: FP64 orthonormal V
    for (int e = threadIdx.x; e < ap * ap; e += blockDim.x) Vs[e] = (double)V32[e];
    __syncthreads();
    gs_columns(Vs, ap, dots);
    // phase 3: T = A V (in M), B = V^T T (over the FP32 area)
    for (int e = threadIdx.x; e < ap * ap; e += blockDim.x) {
        const int col = e / ap, row = e % ap;
        double t = 0.0;
        if (row < a)
            for (int k = 0; k < a; ++k) t += A[row * a + k] * Vs[col * ap + k];
        M[e] = t;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < ap * ap; e += blockDim.x) {
        const int col = e / ap, row = e % ap;
        double t = 0.0;
        for (int k = 0; k < ap; ++k) t += Vs[row * ap + k] * M[col * ap + k];
        B[e] = t;  // B[col * ap + row] = v_row^T A v_col
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = 0.0;
        for (int j = 0; j < ap; ++j) m = fmax(m, fabs(B[j * ap + j]));
        bmax = m;
    }
    __syncthreads();
    // phase 4: FP64 two-sided Jacobi on B, rotations accumulated in R (in M).
    // Each sweep pairs only the active columns, those with an off-diagonal
    // entry above the skip level, in the round-robin order over them: a
    // column whose couplings are all at that level stays there while the
    // others rotate (a rotation of p and q mixes B_ip and B_iq and keeps
    // their norm), and the sweeps after the first usually have a few
    // columns left, the ones of the small eigenvalues the FP32 phase could
    // not resolve -- a sweep over all columns costs ap - 1 rounds of block
    // barriers and FP64 rotation angles whatever the number rotated.
    double* R = M;
    for (int e = threadIdx.x; e < ap * ap; e += blockDim.x) R[e] = (e / ap == e % ap) ? 1.0 : 0.0;
    const double skip = 4e-16 * bmax;  // off-diagonals at the rounding level of B
    __shared__ int act[kMaxDesign];
    __shared__ int actflag[kMaxDesign];
    __shared__ int nact;
    for (int sweep = 0; sweep < 12; ++sweep) {
        if (threadIdx.x == 0) rotated = 0;
        __syncthreads();
        for (int cc = warp; cc < ap; cc += nwarps) {
            bool any = false;
            for (int r = lane; r < ap; r += 32) any |= r != cc && fabs(B[cc * ap + r]) > skip;
            any = __any_sync(0xffffffffu, any);
            if (lane == 0) actflag[cc] = any ? 1 : 0;
        }
        __syncthreads();
        if (warp == 0) {  // the active columns in ascending order
            int run = 0;
            for (int base = 0; base < ap; base += 32) {
                const bool f = base + lane < ap && actflag[base + lane];
                const unsigned m = __ballot_sync(0xffffffffu, f);
                if (f) act[run + __popc(m & ((1u << lane) - 1u))] = base + lane;
                run += __popc(m);
            }
            if (lane == 0) nact = run;
        }
        __syncthreads();
        const int na = nact;
        if (na < 2) break;
        const int nap = na + (na & 1);  // even; position na (odd na) pairs with no column
        const int npairs = nap / 2;
        for (int round = 0; round < nap - 1; ++round) {
            auto pos = [&](int idx) { return idx == 0 ? 0 : 1 + ((idx - 1 + round) % (nap - 1)); };
            for (int k = threadIdx.x; k < npairs; k += blockDim.x) {
                const int x = pos(k), y = pos(nap - 1 - k);
                double cs = 1.0, sn = 0.0;
                int pc = 0, qc = 0;
                if (x < na && y < na) {
                    pc = act[x];
                    qc = act[y];
                    if (pc > qc) { const int t = pc; pc = qc; qc = t; }
                    const double app = B[pc * ap + pc], aqq = B[qc * ap + qc], apq = B[qc * ap + pc];
                    if (fabs(apq) > skip && apq != 0.0) {
                        const double tau = (aqq - app) / (2.0 * apq);
                        const double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
                        cs = 1.0 / sqrt(1.0 + t * t);
                        sn = t * cs;
                        rotated = 1;
                    }
                }
                jp[k] = pc; jq[k] = qc; jc[k] = cs; js[k] = sn;
            }
            __syncthreads();
            // B <- B J and R <- R J (columns p, q of each pair)
            for (int e = threadIdx.x; e < npairs * ap; e += blockDim.x) {
                const int k = e / ap, i = e % ap;
                if (js[k] == 0.0) continue;
                const double cs = jc[k], sn = js[k];
                double* bp = B + jp[k] * ap;
                double* bq = B + jq[k] * ap;
                double x = bp[i], y = bq[i];
                bp[i] = cs * x - sn * y;
                bq[i] = sn * x + cs * y;
                double* rp = R + jp[k] * ap;
                double* rq = R + jq[k] * ap;
                x = rp[i]; y = rq[i];
                rp[i] = cs * x - sn * y;
                rq[i] = sn * x + cs * y;
            }
            __syncthreads();
            // B <- J^T B (rows p, q of each pair)
            for (int e = threadIdx.x; e < npairs * ap; e += blockDim.x) {
                const int k = e / ap, j = e % ap;
                if (js[k] == 0.0) continue;
                const double cs = jc[k], sn = js[k];
                const int pr = jp[k], qr = jq[k];
                const double x = B[j * ap + pr], y = B[j * ap + qr];
                B[j * ap + pr] = cs * x - sn * y;
                B[j * ap + qr] = sn * x + cs * y;
            }
            __syncthreads();
        }
        if (!rotated) break;
    }
    // V <- V R (into B's area, no longer needed)
    for (int e = threadIdx.x; e < ap * ap; e += blockDim.x) {
        const int col = e / ap, row = e % ap;
        double t = 0.0;
        for (int i = 0; i < ap; ++i) t += Vs[i * ap + row] * R[col * ap + i];
        B[e] = t;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < ap * ap; e += blockDim.x) Vs[e] = B[e];
    __syncthreads();
    gs_columns(Vs, ap, dots);
    // phase 5: eigenvalues v_j^T A v_j, descending order
    for (int cc = warp; cc < ap; cc += nwarps) {
        double s = 0.0;
        for (int r = lane; r < a; r += 32) {
            double t = 0.0;
            for (int k = 0; k < a; ++k) t += A[r * a + k] * Vs[cc * ap + k];
            s += Vs[cc * ap + r] * t;
        }
        s = warp_sum(s);
        if (lane == 0) sg[cc] = fabs(s);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 0; i < a; ++i) order[i] = i;
        for (int i = 0; i < a; ++i) {
            int best = i;
            for (int j = i + 1; j < a; ++j)
                if (sg[order[j]] > sg[order[best]]) best = j;
            const int t = order[i]; order[i] = order[best]; order[best] = t;
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < a * a; e += blockDim.x) {
        const int row = e / a, cc = e % a;
        V[row * a + cc] = Vs[order[cc] * ap + row];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < a * a; e += blockDim.x) A[e] = V[e];
    for (int cc = threadIdx.x; cc < a; cc += blockDim.x) sig[cc] = sg[order[cc]];
}

// SplitMix64 counter RNG + Box-Muller (identical stream definition in the
// CPU oracle): element (i, c) of a rows x cols matrix is draw i*cols+c.
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__global__ void k_normal(uint64_t seed, uint64_t total, double* __restrict__ out) {
    const uint64_t key = mix64(seed + 0x9E3779B97F4A7C15ull);
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
         t += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t a = mix64(key + (2 * t + 1) * 0x9E3779B97F4A7C15ull);
        const uint64_t b = mix64(key + (2 * t + 2) * 0x9E3779B97F4A7C15ull);
        const double u1 = ((double)(a >> 11) + 1.0) * 0x1.0p-53;
        const double u2 = (double)(b >> 11) * 0x1.0p-53;
        out[t] = sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
    }
}

__global__ void k_f64_to_f32_pad(const double* __restrict__ A, uint64_t m, int a, int lda,
                                 float* __restrict__ out, uint64_t m_pad, int ldo) {
    const uint64_t total = m_pad * ldo;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
         t += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = t / ldo;
        const int cc = (int)(t - i * ldo);
        out[t] = (i < m && cc < a) ? (float)A[i * lda + cc] : 0.f;
    }
}

__global__ void k_f32_to_f64(const float* __restrict__ A, uint64_t m, int a, int lda,
                             double* __restrict__ out, int ldo) {
    const uint64_t total = m * a;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
         t += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = t / a;
        const int cc = (int)(t - i * a);
        out[i * ldo + cc] = (double)A[i * lda + cc];
    }
}

__global__ void k_transpose(const double* __restrict__ A, int rows, int cols, double* __restrict__ At) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < rows * cols; e += gridDim.x * blockDim.x) {
        const int i = e / cols, j = e % cols;
        At[j * rows + i] = A[e];
    }
}

__global__ void k_scale_cols(double* __restrict__ A, uint64_t m, int a, int lda,
                             const double* __restrict__ f) {
    const uint64_t total = m * a;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
         t += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = t / a;
        const int cc = (int)(t - i * a);
        A[i * lda + cc] *= f[cc];
    }
}

// C = [1 | X | U] (n x (1+d+K))
__global__ void k_build_design(const double* __restrict__ X, int d, const double* __restrict__ U, int K,
                               uint64_t n, double* __restrict__ C) {
    const int w = 1 + d + K;
    const uint64_t total = n * w;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
         t += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = t / w;
        const int cc = (int)(t - i * w);
        C[t] = cc == 0 ? 1.0 : (cc <= d ? X[i * d + cc - 1] : U[i * K + cc - 1 - d]);
    }
}

size_t smem_sq(int a) { return (size_t)a * a * sizeof(double); }

// rows of a narrow FP32 matrix the tiled kernels can take
bool narrow_tiled(const float* A, int lda) {
    return lda % 4 == 0 && lda <= 32 && reinterpret_cast<uintptr_t>(A) % 16 == 0;
}

void set_smem(const void* fn, size_t bytes) { raise_dynamic_smem(fn, bytes); }

}  // namespace

// column means of a tall matrix: rows in ranges of kColRows per block, then
// the partials summed in order and divided by m (one block per column left
// too few blocks on the GPU: 30 blocks each walking 20 000 rows)
constexpr uint64_t kColRows = 2048;

__global__ void k_colsum_split(const double* __restrict__ A, uint64_t m, int a, int lda, uint64_t per,
                               double* __restrict__ part);

__global__ void k_mean_partials(const double* __restrict__ part, int splits, int a, uint64_t m,
                                double* __restrict__ out) {
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= a) return;
    double s = 0.0;
    for (int k = 0; k < splits; ++k) s += part[(uint64_t)k * a + col];
    out[col] = m ? s / (double)m : 0.0;
}

void launch_colmeans(Ctx& c, const double* A, uint64_t m, int a, int lda, double* out) {
    if (a == 0) return;
    if (m <= 2 * kColRows) {
        k_colmeans<<<a, 256, 0, c.stream>>>(A, m, lda, out, 1);
        SLFMM_LAUNCHED(c, "k_colmeans");
        return;
    }
    const uint64_t splits = std::min<uint64_t>(ceil_div(m, kColRows), 512);
    const uint64_t per = ceil_div(m, splits);
    DBuf<double> part(splits * a, c.stream);
    k_colsum_split<<<dim3(a, (unsigned)splits), 256, 0, c.stream>>>(A, m, a, lda, per, part.get());
    SLFMM_LAUNCHED(c, "k_colsum_split");
    k_mean_partials<<<(unsigned)ceil_div((uint64_t)a, 128), 128, 0, c.stream>>>(part.get(), (int)splits, a, m,
                                                                                 out);
    SLFMM_LAUNCHED(c, "k_mean_partials");
}

// column sums of a tall matrix: row ranges of `per` rows in parallel, then
// the partials summed in order
__global__ void k_colsum_split(const double* __restrict__ A, uint64_t m, int a, int lda, uint64_t per,
                               double* __restrict__ part) {
    __shared__ double red[32];
    const int col = blockIdx.x;
    const uint64_t r0 = (uint64_t)blockIdx.y * per, r1 = min(m, r0 + per);
    double s = 0.0;
    for (uint64_t i = r0 + threadIdx.x; i < r1; i += blockDim.x) s += A[i * lda + col];
    s = block_sum(s, red);
    if (threadIdx.x == 0) part[(uint64_t)blockIdx.y * a + col] = s;
}

void launch_colsums(Ctx& c, const double* A, uint64_t m, int a, int lda, double* out) {
    if (a == 0) return;
    if (m <= 2 * kColRows) {
        k_colmeans<<<a, 256, 0, c.stream>>>(A, m, lda, out, 0);
        SLFMM_LAUNCHED(c, "k_colsums");
        return;
    }
    const uint64_t splits = std::min<uint64_t>(ceil_div(m, m <= 65536 ? kColRows : 16384), 512);
    const uint64_t per = ceil_div(m, splits);
    DBuf<double> part(splits * a, c.stream);
    k_colsum_split<<<dim3(a, (unsigned)splits), 256, 0, c.stream>>>(A, m, a, lda, per, part.get());
    SLFMM_LAUNCHED(c, "k_colsum_split");
    launch_sum_partials(c, part.get(), (int)splits, (uint64_t)a, out);
}

void launch_sum_partials(Ctx& c, const double* part, int splits, uint64_t count, double* out) {
    if (!count) return;
    if (splits >= 32) {
        k_sum_partials_wide<<<(unsigned)std::min<uint64_t>(count, 65535), 128, 0, c.stream>>>(part, splits, count,
                                                                                             out);
        SLFMM_LAUNCHED(c, "k_sum_partials_wide");
        return;
    }
    k_sum_partials<<<grid_for(c, count, 256), 256, 0, c.stream>>>(part, splits, count, out);
    SLFMM_LAUNCHED(c, "k_sum_partials");
}

void launch_center_cols(Ctx& c, double* A, uint64_t m, int a, int lda, const double* means) {
    if (a == 0 || m == 0) return;
    k_center_cols<<<grid_for(c, m * a, 256), 256, 0, c.stream>>>(A, m, a, lda, means);
    SLFMM_LAUNCHED(c, "k_center_cols");
}

void launch_scale_cols_sd(Ctx& c, double* A, uint64_t m, int a, int lda) {
    if (a == 0) return;
    k_scale_cols_sd<<<a, 256, 0, c.stream>>>(A, m, lda);
    SLFMM_LAUNCHED(c, "k_scale_cols_sd");
}

template <typename T>
static void atb_impl(Ctx& c, const T* A, int lda, const T* B, int ldb, uint64_t m, int a, int b,
                     double* out) {
    // FP64-bound (GB300 runs FP64 at a small fraction of FP32): enough row
    // splits that every SM holds a few CTAs (64 rows each at least)
    if (a > 0 && b > 0 && a * b <= 256 * 16 * 4 && a <= 128 && b <= 128) {
        const int ab = a * b;
        const int R = ab <= 256 ? 1 : ab <= 512 ? 2 : ab <= 1024 ? 4 : ab <= 2048 ? 8 : 16;
        const int blocks_o = (int)ceil_div((uint64_t)ab, (uint64_t)256 * R);
        uint64_t splits = std::max<uint64_t>(
            1, std::min<uint64_t>(ceil_div(m, 64), ceil_div((uint64_t)c.sm_count * 8, (uint64_t)blocks_o)));
        splits = std::min<uint64_t>(splits, 65535);
        const uint64_t per = round_up(ceil_div(std::max<uint64_t>(m, 1), splits), 32);
        splits = std::max<uint64_t>(1, ceil_div(m, per));
        DBuf<double> part(splits * ab, c.stream);
        const size_t smem = (size_t)32 * (a + b) * sizeof(double);
        dim3 grid(blocks_o, (unsigned)splits);
#define SLFMM_ATB_FLAT(RR)                                                                        \
    do {                                                                                          \
        raise_dynamic_smem((const void*)k_atb_flat<T, RR>, smem);                                 \
        k_atb_flat<T, RR><<<grid, 256, smem, c.stream>>>(A, lda, B, ldb, m, a, b, per, part.get()); \
    } while (0)
        switch (R) {
            case 1: SLFMM_ATB_FLAT(1); break;
            case 2: SLFMM_ATB_FLAT(2); break;
            case 4: SLFMM_ATB_FLAT(4); break;
            case 8: SLFMM_ATB_FLAT(8); break;
            default: SLFMM_ATB_FLAT(16); break;
        }
#undef SLFMM_ATB_FLAT
        SLFMM_LAUNCHED(c, "k_atb_flat");
        launch_sum_partials(c, part.get(), (int)splits, (uint64_t)ab, out);
        return;
    }
    const int ta = (int)ceil_div(a, 32), tb = (int)ceil_div(b, 32);
    uint64_t splits = std::max<uint64_t>(1, std::min<uint64_t>(ceil_div(m, 64),
                                          ceil_div((uint64_t)c.sm_count * 8, (uint64_t)ta * tb)));
    splits = std::min<uint64_t>(splits, 65535);
    const uint64_t per = round_up(ceil_div(std::max<uint64_t>(m, 1), splits), 32);
    splits = std::max<uint64_t>(1, ceil_div(m, per));
    DBuf<double> part(splits * a * b, c.stream);
    dim3 grid(ta, tb, (unsigned)splits);
    k_atb<T><<<grid, 256, 0, c.stream>>>(A, lda, B, ldb, m, a, b, per, part.get());
    SLFMM_LAUNCHED(c, "k_atb");
    launch_sum_partials(c, part.get(), (int)splits, (uint64_t)a * b, out);
}

void launch_atb(Ctx& c, const double* A, int lda, const double* B, int ldb, uint64_t m, int a, int b,
                double* out) {
    atb_impl<double>(c, A, lda, B, ldb, m, a, b, out);
}

void launch_gram_f32(Ctx& c, const float* A, int lda, uint64_t m, int a, double* out) {
    if (a <= 32) {
        if (narrow_tiled(A, lda)) {
            const uint64_t tb = std::max<uint64_t>(1, std::min<uint64_t>(ceil_div(m, (uint64_t)kNarrowTile),
                                                                        (uint64_t)c.sm_count));
            const size_t sm = kPipeRing + (size_t)(kPipeThreads / 32) * 32 * 32 * sizeof(double);
            DBuf<double> tpart(tb * a * a, c.stream);
            set_smem((const void*)k_gram_tile, sm);
            k_gram_tile<<<(unsigned)tb, kPipeThreads, sm, c.stream>>>(A, lda, m, a, tpart.get());
            SLFMM_LAUNCHED(c, "k_gram_tile");
            launch_sum_partials(c, tpart.get(), (int)tb, (uint64_t)a * a, out);
            return;
        }
        const uint64_t runs = std::max<uint64_t>(1, ceil_div(m, (uint64_t)kGramRun));
        const uint64_t blocks = std::max<uint64_t>(1, std::min<uint64_t>(ceil_div(runs, 8), (uint64_t)c.sm_count * 4));
        DBuf<double> part(blocks * a * a, c.stream);
        set_smem((const void*)k_gram_narrow, kGramNarrowSmem);
        k_gram_narrow<<<(unsigned)blocks, 256, kGramNarrowSmem, c.stream>>>(A, lda, m, a, part.get());
        SLFMM_LAUNCHED(c, "k_gram_narrow");
        launch_sum_partials(c, part.get(), (int)blocks, (uint64_t)a * a, out);
        return;
    }
    const int ta = (int)ceil_div(a, 32);
    uint64_t splits = std::max<uint64_t>(1, std::min<uint64_t>(ceil_div(m, 1024),
                                          ceil_div((uint64_t)c.sm_count * 8, (uint64_t)ta * ta)));
    splits = std::min<uint64_t>(splits, 65535);
    const uint64_t per = round_up(ceil_div(std::max<uint64_t>(m, 1), splits), 32);
    splits = std::max<uint64_t>(1, ceil_div(m, per));
    DBuf<double> part(splits * a * a, c.stream);
    dim3 grid(ta, ta, (unsigned)splits);
    k_gram_f32<<<grid, 256, 0, c.stream>>>(A, lda, m, a, per, part.get());
    SLFMM_LAUNCHED(c, "k_gram_f32");
    launch_sum_partials(c, part.get(), (int)splits, (uint64_t)a * a, out);
}

void launch_gemm_small(Ctx& c, const double* A, int lda, uint64_t m, int a, const double* B, int ldb,
                       int b, double alpha, double beta, double* C, int ldc) {
    if (m == 0 || b == 0) return;
    // B in shared memory: column blocks of B (and C) for wide products
    const int bb = std::max(1, std::min(b, (int)((200 * 1024) / (sizeof(double) * (size_t)std::max(a, 1)))));
    for (int c0 = 0; c0 < b; c0 += bb) {
        const int nb = std::min(bb, b - c0);
        const size_t sm = (size_t)a * nb * sizeof(double);
        set_smem((const void*)k_gemm_small<double>, sm);
        k_gemm_small<double><<<grid_for(c, m * nb, 256), 256, sm, c.stream>>>(A, lda, m, a, B + c0, ldb, nb, alpha,
                                                                              beta, C + c0, ldc);
        SLFMM_LAUNCHED(c, "k_gemm_small");
    }
}

void launch_trmul_f32(Ctx& c, float* A, int lda, uint64_t m, int a, const double* Linv) {
    SLFMM_REQUIRE(a <= 64, SLFMM_ERR_BAD_ARG, "sketch width must be <= 64");
    if (m == 0) return;
    if (a <= 32) {
        if (narrow_tiled(A, lda)) {
            // the factor travels in the launch (a x a doubles on the device)
            std::vector<double> L((size_t)a * a);
            SLFMM_CUDA(cudaMemcpyAsync(L.data(), Linv, L.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
            SLFMM_CUDA(cudaStreamSynchronize(c.stream));
            Mat32 R{};
            for (int i = 0; i < a; ++i)
                for (int k = 0; k <= i; ++k) R.v[i][k] = (float)L[(size_t)i * a + k];
            k_trmul_rows<<<grid_for(c, m, 256), 256, 0, c.stream>>>(A, lda, m, a, R);
            SLFMM_LAUNCHED(c, "k_trmul_rows");
            return;
        }
        k_trmul_narrow<<<grid_for(c, m, 32), 256, 0, c.stream>>>(A, lda, m, a, Linv);
        SLFMM_LAUNCHED(c, "k_trmul_narrow");
        return;
    }
    k_trmul_f32<64><<<grid_for(c, m, 128), 128, 0, c.stream>>>(A, lda, m, a, Linv);
    SLFMM_LAUNCHED(c, "k_trmul_f32");
}

// The small dense solvers keep the matrix in shared memory up to kMaxSmall
// columns and work in global memory (L2-resident) up to kMaxDesign.
void launch_cholesky(Ctx& c, double* A, int a, int* status, double drop_tol, int* dropped) {
    SLFMM_REQUIRE(a <= kMaxDesign, SLFMM_ERR_BAD_ARG, "matrix too large for the small Cholesky");
    if (a <= kMaxSmall) {
        set_smem((const void*)k_cholesky, smem_sq(a));
        k_cholesky<<<1, 512, smem_sq(a), c.stream>>>(A, a, status, drop_tol, dropped, nullptr);
    } else {
        DBuf<double> work((size_t)a * a, c.stream);
        k_cholesky<<<1, 1024, 0, c.stream>>>(A, a, status, drop_tol, dropped, work.get());
    }
    SLFMM_LAUNCHED(c, "k_cholesky");
}

void launch_tri_inv_lower(Ctx& c, const double* L, int a, double* Linv) {
    SLFMM_REQUIRE(a <= kMaxDesign, SLFMM_ERR_BAD_ARG, "matrix too large for the triangular inverse");
    const bool sm = a <= kMaxSmall;
    if (sm) set_smem((const void*)k_tri_inv_lower, smem_sq(a));
    k_tri_inv_lower<<<1, sm ? 128 : 256, sm ? smem_sq(a) : 0, c.stream>>>(L, a, Linv, sm ? 1 : 0);
    SLFMM_LAUNCHED(c, "k_tri_inv_lower");
}

void launch_inverse(Ctx& c, const double* A, int a, double* Ainv, int* status, double* eps_used) {
    SLFMM_REQUIRE(a <= kMaxDesign, SLFMM_ERR_BAD_ARG, "matrix too large for the small inverse");
    ProfScope ps(c, "small_inverse", 16.0 * a * a, 2.0 * a * a * a);
    if (a <= kMaxGaussJordan) {
        set_smem((const void*)k_inverse_gj, 2 * smem_sq(a));
        k_inverse_gj<<<1, 1024, 2 * smem_sq(a), c.stream>>>(A, a, Ainv, status, eps_used);
    } else if (a <= kMaxSmall) {
        set_smem((const void*)k_inverse, smem_sq(a));
        k_inverse<<<1, 256, smem_sq(a), c.stream>>>(A, a, Ainv, status, eps_used, nullptr);
    } else {
        DBuf<double> work((size_t)a * a + (size_t)(a + 1) / 2, c.stream);  // matrix, then a pivot ints
        k_inverse<<<1, 1024, 0, c.stream>>>(A, a, Ainv, status, eps_used, work.get());
    }
    SLFMM_LAUNCHED(c, "k_inverse");
}

void launch_jacobi_svd(Ctx& c, const double* A, int a, double* V, double* sig) {
    SLFMM_REQUIRE(a >= 1 && a <= kMaxDesign, SLFMM_ERR_BAD_ARG,
                  "small eigen-solve limited to " + std::to_string(kMaxDesign) + " x " + std::to_string(kMaxDesign));
    const int ap = a + (a & 1);
    const size_t sm = 2 * (size_t)ap * ap * (sizeof(double) + sizeof(float));
    ProfScope ps(c, "small_eigh", 16.0 * a * a, 0.0);
    if (a <= 64) {
        set_smem((const void*)k_jacobi_svd, sm);
        k_jacobi_svd<<<1, 1024, sm, c.stream>>>(const_cast<double*>(A), a, V, sig, nullptr);
    } else {
        DBuf<double> ws((sm + sizeof(double) - 1) / sizeof(double), c.stream);
        k_jacobi_svd<<<1, 1024, 0, c.stream>>>(const_cast<double*>(A), a, V, sig, ws.get());
    }
    SLFMM_LAUNCHED(c, "k_jacobi_svd");
}

void launch_transpose(Ctx& c, const double* A, int rows, int cols, double* At) {
    if (!rows || !cols) return;
    k_transpose<<<grid_for(c, (uint64_t)rows * cols, 256), 256, 0, c.stream>>>(A, rows, cols, At);
    SLFMM_LAUNCHED(c, "k_transpose");
}

void launch_scale_cols(Ctx& c, double* A, uint64_t m, int a, int lda, const double* f) {
    if (!m || !a) return;
    k_scale_cols<<<grid_for(c, m * a, 256), 256, 0, c.stream>>>(A, m, a, lda, f);
    SLFMM_LAUNCHED(c, "k_scale_cols");
}

void launch_build_design(Ctx& c, const double* X, int d, const double* U, int K, uint64_t n, double* C) {
    if (!n) return;
    k_build_design<<<grid_for(c, n * (1 + d + K), 256), 256, 0, c.stream>>>(X, d, U, K, n, C);
    SLFMM_LAUNCHED(c, "k_build_design");
}

void launch_normal(Ctx& c, uint64_t seed, uint64_t rows, int cols, double* out) {
    const uint64_t total = rows * cols;
    if (!total) return;
    k_normal<<<grid_for(c, total, 256), 256, 0, c.stream>>>(seed, total, out);
    SLFMM_LAUNCHED(c, "k_normal");
}

void launch_f64_to_f32_pad(Ctx& c, const double* A, uint64_t m, int a, int lda, float* out,
                           uint64_t m_pad, int ldo) {
    if (!m_pad || !ldo) return;
    k_f64_to_f32_pad<<<grid_for(c, m_pad * ldo, 256), 256, 0, c.stream>>>(A, m, a, lda, out, m_pad, ldo);
    SLFMM_LAUNCHED(c, "k_f64_to_f32_pad");
}

void launch_f32_to_f64(Ctx& c, const float* A, uint64_t m, int a, int lda, double* out, int ldo) {
    if (!m || !a) return;
    k_f32_to_f64<<<grid_for(c, m * a, 256), 256, 0, c.stream>>>(A, m, a, lda, out, ldo);
    SLFMM_LAUNCHED(c, "k_f32_to_f64");
}

}  // namespace slfmm
