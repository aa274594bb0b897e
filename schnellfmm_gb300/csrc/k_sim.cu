// Synthetic structured cohorts generated on the device (benchmark inputs).
//
// Plays the role of the reference's simulator (src/simulate.rs:49-142) for
// the benchmark shapes, which are too large to draw on the host: per SNP an
// ancestral frequency f ~ U(f_lo, f_hi), per population a drifted frequency
// (normal approximation of Balding-Nichols: f + sqrt(Fst f (1-f)) z, clamped),
// per sample the admixture-weighted frequency, genotype = two Bernoulli
// alleles (or one doubled allele with probability `inbreeding`), and MCAR
// missing calls.  Output is the device packed layout (PLINK 2-bit codes).
#include "slfmm_internal.h"

namespace slfmm {
namespace {

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ double u53(uint64_t key, uint64_t ctr) {
    return (double)(mix64(key + (ctr + 1) * 0x9E3779B97F4A7C15ull) >> 11) * 0x1.0p-53;
}

// f[j * n_pop + k]: drifted population frequencies
__global__ void k_sim_freq(uint64_t p, int n_pop, double fst, double f_lo, double f_hi, uint64_t key,
                           float* __restrict__ f) {
    for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < p;
         j += (uint64_t)gridDim.x * blockDim.x) {
        const double fa = f_lo + (f_hi - f_lo) * u53(key, j * 64);
        const double sd = sqrt(fst * fa * (1.0 - fa));
        for (int k = 0; k < n_pop; ++k) {
            const double a = u53(key, j * 64 + 1 + 2 * k) + 0x1.0p-53;
            const double b = u53(key, j * 64 + 2 + 2 * k);
            const double z = sqrt(-2.0 * log(a)) * cospi(2.0 * b);
            f[j * n_pop + k] = (float)fmin(fmax(fa + sd * z, 1e-3), 1.0 - 1e-3);
        }
    }
}

constexpr int kSimSamples = 512;  // samples per CTA (32 words of 16 samples)
constexpr int kSimSnps = 64;      // SNPs per smem batch

// One CTA per (sample block, SNP range); thread = one 32-bit word of codes.
__global__ void __launch_bounds__(256) k_sim_geno(uint64_t n, uint64_t p, int n_pop,
                                                  const float* __restrict__ admix,
                                                  const float* __restrict__ f, double miss,
                                                  double inbreeding, uint64_t key, uint64_t snps_per_cta,
                                                  uint8_t* __restrict__ out, uint64_t stride) {
    extern __shared__ float sm[];
    float* q = sm;                              // kSimSamples x n_pop
    float* fs = sm + kSimSamples * n_pop;       // kSimSnps x n_pop
    const uint64_t s0 = (uint64_t)blockIdx.x * kSimSamples;
    for (int e = threadIdx.x; e < kSimSamples * n_pop; e += blockDim.x) {
        const uint64_t i = s0 + e / n_pop;
        q[e] = i < n ? admix[i * n_pop + e % n_pop] : 0.f;
    }
    const uint64_t j0 = (uint64_t)blockIdx.y * snps_per_cta;
    const uint64_t j1 = min(p, j0 + snps_per_cta);
    const uint32_t miss16 = (uint32_t)(miss * 65536.0);
    const uint32_t inb16 = (uint32_t)(inbreeding * 65536.0);
    const int word = threadIdx.x & 31;          // 32 words per sample block
    const int sub = threadIdx.x >> 5;           // 8 SNP lanes
    for (uint64_t jb = j0; jb < j1; jb += kSimSnps) {
        __syncthreads();
        for (int e = threadIdx.x; e < kSimSnps * n_pop; e += blockDim.x) {
            const uint64_t j = jb + e / n_pop;
            fs[e] = j < j1 ? f[j * n_pop + e % n_pop] : 0.f;
        }
        __syncthreads();
        for (int jj = sub; jj < kSimSnps; jj += 8) {
            const uint64_t j = jb + jj;
            if (j >= j1) break;
            uint32_t codes = 0;
            const float* fj = fs + jj * n_pop;
#pragma unroll 4
            for (int t = 0; t < 16; ++t) {
                const int il = word * 16 + t;
                const uint64_t i = s0 + il;
                if (i >= n) break;
                float pr = 0.f;
                for (int k = 0; k < n_pop; ++k) pr = fmaf(q[il * n_pop + k], fj[k], pr);
                const uint64_t h = mix64(key ^ (j * 0x9E3779B97F4A7C15ull + i * 0xD1B54A32D192ED03ull));
                const uint32_t thr = (uint32_t)(pr * 65536.0f);
                const uint32_t u1 = (uint32_t)(h & 0xffff), u2 = (uint32_t)((h >> 16) & 0xffff);
                const uint32_t um = (uint32_t)((h >> 32) & 0xffff), ui = (uint32_t)(h >> 48);
                uint32_t g = (u1 < thr) + (u2 < thr);
                if (ui < inb16) g = (u1 < thr) ? 2u : 0u;
                uint32_t code = g == 0 ? 0u : (g == 1 ? 2u : 3u);
                if (um < miss16) code = 1u;
                codes |= code << (2 * t);
            }
            const uint64_t wbyte = (s0 / 4) + (uint64_t)word * 4;
            if (wbyte < stride) reinterpret_cast<uint32_t*>(out + j * stride)[wbyte / 4] = codes;
        }
    }
}

}  // namespace

void launch_simulate(Ctx& c, uint64_t n, uint64_t p, int n_pop, const float* admix_dev, double fst,
                     double f_lo, double f_hi, double miss, double inbreeding, uint64_t seed, uint8_t* out,
                     uint64_t stride) {
    SLFMM_REQUIRE(n_pop >= 1 && n_pop <= 32, SLFMM_ERR_BAD_ARG, "1..32 populations");
    const uint64_t key = mix64(seed + 0x9E3779B97F4A7C15ull);
    DBuf<float> f(std::max<uint64_t>(p, 1) * n_pop, c.stream);
    k_sim_freq<<<grid_for(c, p, 256), 256, 0, c.stream>>>(p, n_pop, fst, f_lo, f_hi, key, f.get());
    SLFMM_LAUNCHED(c, "k_sim_freq");
    SLFMM_CUDA(cudaMemsetAsync(out, 0, p * stride, c.stream));
    const uint64_t sblocks = ceil_div(n, kSimSamples);
    const uint64_t want = std::max<uint64_t>(1, ((uint64_t)c.sm_count * 8) / sblocks);
    const uint64_t per = round_up(ceil_div(p, want), kSimSnps);
    dim3 grid((unsigned)sblocks, (unsigned)ceil_div(p, per));
    const size_t smem = (size_t)(kSimSamples + kSimSnps) * n_pop * sizeof(float);
    raise_dynamic_smem((const void*)k_sim_geno, smem);
    k_sim_geno<<<grid, 256, smem, c.stream>>>(n, p, n_pop, admix_dev, f.get(), miss, inbreeding, key ^ 0x5bd1e995ull,
                                              per, out, stride);
    SLFMM_LAUNCHED(c, "k_sim_geno");
}

}  // namespace slfmm
