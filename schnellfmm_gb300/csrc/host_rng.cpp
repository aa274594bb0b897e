// The reference's Gaussian sketch stream, drawn on the host.
//
// src/rsvd.rs:44-46 draws Omega (n x l) as
//   Array2::from_shape_fn((n, l), |_| Normal::new(0, 1).sample(&mut ChaCha8Rng::seed_from_u64(seed)))
// in row-major order, and init_from_random_probe (src/nmf.rs:291-293) draws its
// probe the same way from seed + 1 000 000.  The crates (rand_core 0.6.4,
// rand_chacha 0.3.1, rand_distr 0.4.3 per Cargo.lock) are not available here;
// this file is written from the published algorithms they implement:
//
//  * ChaCha with 8 rounds (Bernstein, "ChaCha, a variant of Salsa20", 2008).
//    Block function as in RFC 8439 s2.3; words 12-13 hold a 64-bit block
//    counter starting at 0 and words 14-15 a 64-bit stream id (0); the key is
//    the 32-byte seed read as 8 little-endian words.  The generator returns
//    the keystream as consecutive 32-bit words, a 64-bit draw being two of
//    them, low word first.
//  * seed_from_u64 fills the 32-byte seed with 8 outputs of PCG32's XSH-RR
//    permutation (O'Neill, "PCG: a family of simple fast space-efficient
//    statistically good algorithms for random number generation", 2014) over a
//    64-bit LCG whose state is stepped before each output.
//  * Normal(0, 1) is mean + sd * z with z from the ZIGNOR ziggurat (Doornik,
//    "An improved ziggurat method to generate normal random samples", 2005)
//    with 256 strips, R = 3.6541528853610088 and strip area V =
//    0.00492867323399.  One 64-bit draw gives the strip (low 8 bits) and a
//    uniform in [-1, 1) (its top 52 bits as the mantissa of a number in
//    [2, 4), minus 3); the wedge test takes a U[0, 1) from the next draw (top
//    53 bits times 2^-53); the tail beyond R uses Marsaglia's pair of
//    exponentials from open (0, 1) uniforms (top 52 bits in [1, 2) minus
//    1 - 2^-53).
//
// The block function is pinned by the RFC 8439 test vector; the seed
// expansion, the output order and the sampler follow the crates' published
// descriptions and cannot be run against the crates here.
#include <cmath>
#include <cstring>

#include "slfmm_internal.h"

namespace slfmm {
namespace {

inline uint32_t rotl32(uint32_t x, int r) { return (x << r) | (x >> (32 - r)); }
inline uint32_t rotr32(uint32_t x, int r) { return r ? (x >> r) | (x << (32 - r)) : x; }

inline void quarter(uint32_t& a, uint32_t& b, uint32_t& c, uint32_t& d) {
    a += b; d ^= a; d = rotl32(d, 16);
    c += d; b ^= c; b = rotl32(b, 12);
    a += b; d ^= a; d = rotl32(d, 8);
    c += d; b ^= c; b = rotl32(b, 7);
}

// one keystream block: `rounds` rounds (column + diagonal = 2) and the
// feed-forward of the input state
void chacha_block(const uint32_t in[16], int rounds, uint32_t out[16]) {
    uint32_t x[16];
    std::memcpy(x, in, sizeof(x));
    for (int r = 0; r < rounds; r += 2) {
        quarter(x[0], x[4], x[8], x[12]);
        quarter(x[1], x[5], x[9], x[13]);
        quarter(x[2], x[6], x[10], x[14]);
        quarter(x[3], x[7], x[11], x[15]);
        quarter(x[0], x[5], x[10], x[15]);
        quarter(x[1], x[6], x[11], x[12]);
        quarter(x[2], x[7], x[8], x[13]);
        quarter(x[3], x[4], x[9], x[14]);
    }
    for (int i = 0; i < 16; ++i) out[i] = x[i] + in[i];
}

class ChaCha8Stream {
public:
    explicit ChaCha8Stream(uint64_t seed) {
        st_[0] = 0x61707865u;   // "expand 32-byte k"
        st_[1] = 0x3320646eu;
        st_[2] = 0x79622d32u;
        st_[3] = 0x6b206574u;
        uint64_t s = seed;
        for (int j = 0; j < 8; ++j) {
            s = s * 6364136223846793005ull + 11634580027462260723ull;
            const uint32_t xorshifted = (uint32_t)(((s >> 18) ^ s) >> 27);
            st_[4 + j] = rotr32(xorshifted, (int)(s >> 59));
        }
        st_[12] = st_[13] = st_[14] = st_[15] = 0;
    }
    uint64_t next_u64() {
        const uint64_t lo = next_u32();
        const uint64_t hi = next_u32();
        return lo | (hi << 32);
    }

private:
    uint32_t next_u32() {
        if (idx_ == 16) {
            chacha_block(st_, 8, buf_);
            if (++st_[12] == 0) ++st_[13];
            idx_ = 0;
        }
        return buf_[idx_++];
    }
    uint32_t st_[16];
    uint32_t buf_[16];
    int idx_ = 16;
};

inline double from_bits(uint64_t b) {
    double d;
    std::memcpy(&d, &b, sizeof(d));
    return d;
}

constexpr double kZigR = 3.6541528853610088;
constexpr double kZigV = 0.00492867323399;

inline double gauss_pdf(double x) { return std::exp(-x * x / 2.0); }

// strip edges x_0 > x_1 = R > ... > x_255 > x_256 = 0 (x_0 = V / f(R), the
// base strip's equivalent width) and f(x_i)
struct ZigTables {
    double x[257];
    double f[257];
    ZigTables() {
        x[0] = kZigV / gauss_pdf(kZigR);
        x[1] = kZigR;
        for (int i = 2; i < 256; ++i) x[i] = std::sqrt(-2.0 * std::log(kZigV / x[i - 1] + gauss_pdf(x[i - 1])));
        x[256] = 0.0;
        for (int i = 0; i <= 256; ++i) f[i] = gauss_pdf(x[i]);
    }
};

const ZigTables& zig_tables() {
    static const ZigTables t;
    return t;
}

inline double unit_closed_open(ChaCha8Stream& r) { return (double)(r.next_u64() >> 11) * (1.0 / 9007199254740992.0); }
inline double unit_open(ChaCha8Stream& r) {
    return from_bits((1023ull << 52) | (r.next_u64() >> 12)) - (1.0 - 1.0 / 9007199254740992.0);
}

double standard_normal(ChaCha8Stream& r, const ZigTables& t) {
    for (;;) {
        const uint64_t bits = r.next_u64();
        const int i = (int)(bits & 0xff);
        const double u = from_bits((1024ull << 52) | (bits >> 12)) - 3.0;
        const double x = u * t.x[i];
        if (std::fabs(x) < t.x[i + 1]) return x;
        if (i == 0) {
            double ex = 1.0, ey = 0.0;
            while (-2.0 * ey < ex * ex) {
                const double a = unit_open(r);
                const double b = unit_open(r);
                ex = std::log(a) / kZigR;
                ey = std::log(b);
            }
            return u < 0.0 ? ex - kZigR : kZigR - ex;
        }
        if (t.f[i + 1] + (t.f[i] - t.f[i + 1]) * unit_closed_open(r) < gauss_pdf(x)) return x;
    }
}

}  // namespace

void reference_normal(uint64_t seed, uint64_t rows, uint64_t cols, double* out) {
    const ZigTables& t = zig_tables();
    ChaCha8Stream r(seed);
    const double mean = 0.0, sd = 1.0;
    for (uint64_t e = 0; e < rows * cols; ++e) out[e] = mean + sd * standard_normal(r, t);
}

void draw_normal(Ctx& c, uint64_t seed, uint64_t rows, int cols, double* out) {
    if (c.rng != SLFMM_RNG_CHACHA8) {
        launch_normal(c, seed, rows, cols, out);
        return;
    }
    std::vector<double> h(rows * (uint64_t)cols);
    reference_normal(seed, rows, (uint64_t)cols, h.data());
    if (!h.empty()) {
        SLFMM_CUDA(cudaMemcpyAsync(out, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream));
        SLFMM_CUDA(cudaStreamSynchronize(c.stream));
    }
}

}  // namespace slfmm

extern "C" int slfmm_reference_normal(uint64_t seed, uint64_t rows, uint32_t cols, double* out) {
    if (rows && cols && rows > UINT64_MAX / cols) return SLFMM_ERR_BAD_ARG;
    if (!out && rows && cols) return SLFMM_ERR_BAD_ARG;
    slfmm::reference_normal(seed, rows, cols, out);
    return SLFMM_OK;
}
