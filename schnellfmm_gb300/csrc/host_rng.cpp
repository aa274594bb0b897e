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
#include <algorithm>
#include <cmath>
#include <cstring>
#include <future>
#include <memory>
#include <thread>
#include <vector>

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

// Input state of ChaCha8Rng::seed_from_u64(seed) at block 0.
void chacha8_key_state(uint64_t seed, uint32_t st[16]) {
    st[0] = 0x61707865u;   // "expand 32-byte k"
    st[1] = 0x3320646eu;
    st[2] = 0x79622d32u;
    st[3] = 0x6b206574u;
    uint64_t s = seed;
    for (int j = 0; j < 8; ++j) {
        s = s * 6364136223846793005ull + 11634580027462260723ull;
        const uint32_t xorshifted = (uint32_t)(((s >> 18) ^ s) >> 27);
        st[4 + j] = rotr32(xorshifted, (int)(s >> 59));
    }
    st[12] = st[13] = st[14] = st[15] = 0;
}

// 64-bit output number `pos` of the stream: block pos / 8, words 2 (pos % 8)
// (low) and 2 (pos % 8) + 1 (high); the stream is counter-addressable.
inline uint64_t chacha8_u64_at(const uint32_t key[16], uint64_t pos) {
    uint32_t in[16], out[16];
    std::memcpy(in, key, sizeof(in));
    const uint64_t b = pos / 8;
    in[12] = (uint32_t)b;
    in[13] = (uint32_t)(b >> 32);
    chacha_block(in, 8, out);
    const int w = (int)(pos % 8);
    return (uint64_t)out[2 * w] | ((uint64_t)out[2 * w + 1] << 32);
}

class ChaCha8Stream {
public:
    explicit ChaCha8Stream(uint64_t seed) { chacha8_key_state(seed, st_); }
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

template <class Stream>
inline double unit_closed_open(Stream& r) { return (double)(r.next_u64() >> 11) * (1.0 / 9007199254740992.0); }
template <class Stream>
inline double unit_open(Stream& r) {
    return from_bits((1023ull << 52) | (r.next_u64() >> 12)) - (1.0 - 1.0 / 9007199254740992.0);
}

// The ziggurat's first test on one 64-bit draw: true (and x) when the draw
// is accepted at once, without further draws.
inline bool zig_fast(uint64_t bits, const ZigTables& t, double& x) {
    const int i = (int)(bits & 0xff);
    const double u = from_bits((1024ull << 52) | (bits >> 12)) - 3.0;
    x = u * t.x[i];
    return std::fabs(x) < t.x[i + 1];
}

template <class Stream>
double standard_normal(Stream& r, const ZigTables& t) {
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

// The stream from output `pos` on, read from a precomputed run of outputs
// [0, n) and computed block by block past its end.
struct BufferedStream {
    const uint64_t* buf;
    uint64_t n;
    const uint32_t* key;
    uint64_t pos;
    uint64_t next_u64() { return pos < n ? buf[pos++] : chacha8_u64_at(key, pos++); }
};

template <class F>
void parallel_for(uint64_t n, int threads, F&& fn) {
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; ++t)
        pool.emplace_back([&, t] { fn(n * (uint64_t)t / threads, n * (uint64_t)(t + 1) / threads); });
    fn(0, n / (uint64_t)threads);
    for (auto& th : pool) th.join();
}

// The same draws as the sequential loop, on host threads.  Draw e starts at
// some 64-bit output s_e; most draws take one output (the ziggurat's first
// test accepts), so s_{e+1} = s_e + 1 except after a draw that goes on to
// the wedge or tail tests.  The outputs are generated and tested in
// parallel (the stream is counter-addressable); one thread then walks only
// the outputs whose first test fails, in order, running the full sampler
// from each one that is a draw start (an output inside an earlier draw's
// extra draws is not), which fixes every s_e; the values are copied out in
// parallel.
void reference_normal_parallel(uint64_t seed, uint64_t count, double* out, int threads) {
    const ZigTables& t = zig_tables();
    uint32_t key[16];
    chacha8_key_state(seed, key);
    uint64_t npos = count + count / 32 + 4096;
    for (;;) {
        const uint64_t nb = (npos + 7) / 8;
        npos = nb * 8;
        std::unique_ptr<uint64_t[]> bits(new uint64_t[npos]);  // no zero fill: every entry is written
        std::unique_ptr<double[]> val(new double[npos]);
        std::vector<std::vector<uint64_t>> slow(threads);
        const uint64_t per = (nb + threads - 1) / threads;
        std::vector<std::thread> pool;
        auto gen = [&](int th) {
            const uint64_t b0 = std::min(nb, per * th), b1 = std::min(nb, b0 + per);
            uint32_t in[16], o[16];
            std::memcpy(in, key, sizeof(in));
            for (uint64_t b = b0; b < b1; ++b) {
                in[12] = (uint32_t)b;
                in[13] = (uint32_t)(b >> 32);
                chacha_block(in, 8, o);
                for (int w = 0; w < 8; ++w) {
                    const uint64_t j = b * 8 + w;
                    bits[j] = (uint64_t)o[2 * w] | ((uint64_t)o[2 * w + 1] << 32);
                    double x;
                    if (zig_fast(bits[j], t, x)) val[j] = x;
                    else slow[th].push_back(j);
                }
            }
        };
        for (int th = 1; th < threads; ++th) pool.emplace_back(gen, th);
        gen(0);
        for (auto& th : pool) th.join();
        // walk: runs of one-output draws between the draw starts that need
        // more outputs
        struct Run { uint64_t pos, out, len; };
        std::vector<Run> runs;
        std::vector<std::pair<uint64_t, double>> singles;  // (output index, value)
        uint64_t cur = 0, produced = 0;
        bool done = false;
        for (int th = 0; th < threads && !done; ++th)
            for (uint64_t e : slow[th]) {
                if (e < cur) continue;                   // inside an earlier draw
                const uint64_t len = std::min(e - cur, count - produced);
                if (len) runs.push_back({cur, produced, len});
                produced += len;
                if (produced == count) { done = true; break; }
                BufferedStream bs{bits.get(), npos, key, e};
                singles.emplace_back(produced, standard_normal(bs, t));
                ++produced;
                cur = bs.pos;
                if (produced == count) { done = true; break; }
            }
        if (!done && cur < npos) {
            const uint64_t len = std::min(npos - cur, count - produced);
            runs.push_back({cur, produced, len});
            produced += len;
        }
        if (produced < count) {  // more outputs needed than generated (rare)
            npos *= 2;
            continue;
        }
        const double mean = 0.0, sd = 1.0;
        parallel_for(runs.size(), threads, [&](uint64_t r0, uint64_t r1) {
            for (uint64_t r = r0; r < r1; ++r)
                for (uint64_t k = 0; k < runs[r].len; ++k) out[runs[r].out + k] = mean + sd * val[runs[r].pos + k];
        });
        for (const auto& sv : singles) out[sv.first] = mean + sd * sv.second;
        return;
    }
}

}  // namespace

void reference_normal(uint64_t seed, uint64_t rows, uint64_t cols, double* out) {
    const uint64_t count = rows * cols;
    const int hw = (int)std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    if (count >= (1u << 16) && hw > 1) {
        reference_normal_parallel(seed, count, out, hw);
        return;
    }
    const ZigTables& t = zig_tables();
    ChaCha8Stream r(seed);
    const double mean = 0.0, sd = 1.0;
    for (uint64_t e = 0; e < count; ++e) out[e] = mean + sd * standard_normal(r, t);
}


struct Ctx::PendingNormal {
    uint64_t seed, rows;
    int cols;
    std::future<std::vector<double>> draws;
};

void prefetch_normal(Ctx& c, uint64_t seed, uint64_t rows, int cols) {
    if (c.rng != SLFMM_RNG_CHACHA8 || rows == 0 || cols <= 0 || cols > 64) return;  // the fit checks the shape
    if (c.pending_normal && c.pending_normal->seed == seed && c.pending_normal->rows == rows &&
        c.pending_normal->cols == cols)
        return;
    auto p = std::make_shared<Ctx::PendingNormal>();
    p->seed = seed;
    p->rows = rows;
    p->cols = cols;
    p->draws = std::async(std::launch::async, [seed, rows, cols] {
        std::vector<double> h(rows * (uint64_t)cols);
        reference_normal(seed, rows, (uint64_t)cols, h.data());
        return h;
    });
    c.pending_normal = std::move(p);
}

void draw_normal(Ctx& c, uint64_t seed, uint64_t rows, int cols, double* out) {
    if (c.rng != SLFMM_RNG_CHACHA8) {
        launch_normal(c, seed, rows, cols, out);
        return;
    }
    std::vector<double> h;
    auto& p = c.pending_normal;
    if (p && p->seed == seed && p->rows == rows && p->cols == cols) {
        auto mine = std::move(p);
        h = mine->draws.get();
    } else {
        h.resize(rows * (uint64_t)cols);
        reference_normal(seed, rows, (uint64_t)cols, h.data());
    }
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
