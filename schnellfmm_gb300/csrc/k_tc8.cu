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
// Every CTA streams its own W stages; a stage is reloaded only after the
// CTA's MMAs on it have completed (per-stage "B empty" barriers).  The W
// operand is stored stage-major in global memory -- each 256-sample stage one
// contiguous blob [half][row][128 B] with the 128-byte swizzle already applied
// -- so a stage lands with ONE bulk copy.  On GB300 the copies one thread
// issues complete one after another at a near-constant ~500-750 cycles each
// whatever their size (4 KB to 64 KB, L2 or HBM), so the number of copies per
// stage, not their bytes, sets how fast a single producer can feed the MMAs.
//
// Replaces the reference's per-chunk FP64 dgemms (src/rsvd.rs:61-69, :88-97,
// :117-125, :144-153; src/testing.rs:355-374) and, through the indicator
// operand, the NaN -> column-mean fill of decode_single_snp
// (src/bed.rs:349-378) inside them.
#include <cuda.h>
#include <cuda_fp8.h>

#include <cstdlib>

#include "slfmm_internal.h"
#include "tc_common.cuh"

namespace slfmm {
namespace {
using namespace tc;

constexpr int kM = 128;
constexpr int kTileK = 128;                        // samples (codes) per tile block
constexpr int kTileBytes = kM * kTileK / 4;        // 4 KiB: 128 rows x 32 B
constexpr int kHalves = 2;                         // tile blocks per pipeline stage
constexpr int kStageK = kTileK * kHalves;          // 256 samples per stage
constexpr int kStageBytes = kTileBytes * kHalves;  // packed bytes per stage
constexpr int kUnpackSets = 2;   // sets of four unpack warps taking K blocks round robin
constexpr int kThreads = 128 + 128 * kUnpackSets;  // code-copy, 2 MMA, W-copy warps + unpack sets
constexpr int kMainTerms = 4;
constexpr int kIndTerms = 3;
constexpr uint32_t kTabGeno = 0x40380000u;  // code 00,01 -> 0; 10 -> 1.0; 11 -> 2.0 (E4M3 bytes)
constexpr uint32_t kTabMiss = 0x00003800u;  // code 01 (missing) -> 1.0

struct Tc8Args {
    uint32_t rows, kb_total, kb_per_split;
    uint32_t wpad;          // output columns
    uint32_t n_main;        // kMainTerms * wpad
    uint32_t n_ind;         // kIndTerms * wpad or 0
    uint32_t n_total;       // B rows (n_main + n_ind, or n_main when ind_shared)
    uint32_t ind_shared;    // indicator MMAs read B rows [0, n_ind) of the main terms
    uint32_t d_cols;        // TMEM columns reserved for D
    uint32_t a_cols;        // TMEM columns per A stage (32, or 64 with the indicator)
    uint32_t stages, tmem_cols;  // stages: A operand ring depth (TMEM)
    uint32_t wstages;       // W operand ring depth (shared memory), >= stages
    uint32_t pstages;       // packed-code prefetch depth
    uint32_t group;         // K blocks an MMA warp waits for at once (1, 2, 4; divides stages)
    uint32_t kcopies;       // accumulator copies (2: MMA warps take alternate K groups)
    uint32_t nsplit;        // 1: MMA warp 0 issues the genotype MMAs, warp 1 the indicator MMAs
    uint32_t a_base;        // first TMEM column of the A stages
    uint32_t usets;         // unpack sets in use: at most `stages`, so that a set never waits on a stage
                            // two uses ahead (an mbarrier parity wait cannot tell those apart)
    uint32_t b_stage_bytes; // n_total * 256: one stage of the stage-major W operand
    const float* inv_scale; // n_total: 2^-(e0 + 4t) per B row
    const uint8_t* wop;     // stage-major, pre-swizzled W operand (wop_offset)
    int mode;               // 0: out = P + M; 1: out = s_r (P - mu_r (cs_c - M))
    long long expire_cycles;  // > 0: test hook, see below
    uint32_t tile0;           // matrix index of the tile of unit 0
    uint32_t units, gx;       // work units (row tiles x K splits) and row tiles
    uint32_t rotate;          // stagger the K order of the tiles (see below)
    const double* row_mean;
    const double* row_scale;
    const double* cs;
    float* out;
    uint32_t ldo;
    uint64_t split_stride;
    const uint8_t* tiles;   // tile-major packed codes
    uint64_t tile_bytes;    // kbt * 4096
    int* err;
};

// Pins 32 values in registers at this point of the program (an empty asm
// that reads them), so the compiler cannot sink their computation past a
// following wait.
__device__ __forceinline__ void keep32(const uint32_t (&v)[32]) {
    asm volatile("" ::"r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]),
                 "r"(v[8]), "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15]),
                 "r"(v[16]), "r"(v[17]), "r"(v[18]), "r"(v[19]), "r"(v[20]), "r"(v[21]), "r"(v[22]), "r"(v[23]),
                 "r"(v[24]), "r"(v[25]), "r"(v[26]), "r"(v[27]), "r"(v[28]), "r"(v[29]), "r"(v[30]), "r"(v[31]));
}

// Warp-wide bounded wait: lane 0 polls the barrier, the result is broadcast
// and __syncwarp orders the other lanes after lane 0's observation.  One
// poller per warp keeps the barrier word's traffic low.
__device__ __forceinline__ bool warp_wait(uint64_t* bar, uint32_t parity, int* err, int code) {
    int ok = 1;
    if ((threadIdx.x & 31) == 0) ok = mbar_wait(bar, parity, err, code) ? 1 : 0;
    ok = __shfl_sync(0xffffffffu, ok, 0);
    __syncwarp();
    return ok != 0;
}

// Ring position: slot index and the parity of its current use.
struct Ring {
    uint32_t slot, phase;
    __device__ __forceinline__ void advance(uint32_t by, uint32_t n) {
        slot += by;
        while (slot >= n) {
            slot -= n;
            phase ^= 1u;
        }
    }
};

// MMA issue loop of one of the two MMA warps.  Measured properties of the
// issuing thread shape it: (1) it is latency bound on operand arithmetic
// between MMAs, so descriptors / TMEM addresses are per-stage bases plus
// compile-time offsets; (2) an mbarrier wait by the issuing thread returns only
// after the MMAs it issued before have (nearly) drained from the tensor pipe,
// so a single issuing warp leaves the pipe idle at every wait.  Two MMA warps
// whose waits fall at different K blocks keep it busy: without the indicator
// they take alternate groups of G K blocks into two accumulator copies (summed
// in the epilogue); with it one issues the genotype MMAs and the other the
// indicator MMAs of every K block, their group boundaries G/2 apart.
//
// This warp's K blocks of one work unit: [start, start + len0), then groups
// of G, each followed by `skip` K blocks that belong to the other warp.  The
// unit's first K block is stage g0 of the CTA's stage sequence (the rings run
// on across the CTA's units: stage g sits in A slot g % S, W slot g % SW).
__device__ __forceinline__ Ring ring_at(uint64_t g, uint32_t n) {
    return Ring{(uint32_t)(g % n), (uint32_t)((g / n) & 1u)};
}

template <int NCH, bool MAIN, bool IND, int G>
__device__ __forceinline__ bool tc8_mma_loop(const Tc8Args& a, uint32_t tmem, uint32_t d_main, uint32_t bsm_addr,
                                             uint64_t* full_b, uint64_t* full_a, uint64_t* a_empty,
                                             uint64_t* b_empty, uint64_t g0, uint32_t nkb, uint32_t start,
                                             uint32_t len0, uint32_t skip) {
    const uint32_t S = a.stages, SW = a.wstages;
    const uint32_t chunk = a.n_main / NCH;
    const uint32_t id_main = instr_desc_e4m3(chunk);
    const uint32_t id_ind = IND ? instr_desc_e4m3(a.n_ind) : 0u;
    const uint64_t bdesc0 = smem_desc(bsm_addr);
    const uint64_t bstep = a.b_stage_bytes >> 4;          // descriptor address units per stage
    const uint64_t chstep = (uint64_t)chunk * (128 >> 4);  // per main chunk of B rows
    const uint64_t indoff = a.ind_shared ? 0ull : (uint64_t)a.n_main * (128 >> 4);
    const uint64_t hstep = (uint64_t)a.n_total * (128 >> 4);  // next 128-sample half of the stage
    const uint32_t d_ind = tmem + a.n_main;
    const uint32_t a0 = tmem + a.a_base;
    Ring st = ring_at(g0 + start, S), sw = ring_at(g0 + start, SW);  // A ring (TMEM), W ring (shared memory)
    uint32_t i = start, len = len0;
    while (i < nkb) {
        const uint32_t g = min(len, nkb - i);
        bool ok = true;
        Ring w = st, wb = sw;
        for (uint32_t j = 0; j < g && ok; ++j) {
            ok = mbar_wait(full_b + wb.slot, wb.phase, a.err, 25) && mbar_wait(full_a + w.slot, w.phase, a.err, 26);
            w.advance(1, S);
            wb.advance(1, SW);
        }
        if (!ok) return false;
        fence_after();
#pragma unroll
        for (int j = 0; j < G; ++j) {
            if ((uint32_t)j < g) {
                const uint64_t bd = bdesc0 + sw.slot * bstep;
                const uint32_t ad = a0 + st.slot * a.a_cols;
                const uint32_t acc0 = (i + j) > start ? 1u : 0u;
#pragma unroll
                for (int kk = 0; kk < kStageK / 32; ++kk) {
                    const uint32_t acc = kk > 0 ? 1u : acc0;
                    const uint64_t bk = bd + (kk >> 2) * hstep + (kk & 3) * 2;
                    if (MAIN) {
#pragma unroll
                        for (int ch = 0; ch < NCH; ++ch)
                            mma_ts_f8(d_main + ch * chunk, ad + kk * 8, bk + ch * chstep, id_main, acc);
                    }
                    if (IND) mma_ts_f8(d_ind, ad + kStageK / 4 + kk * 8, bk + indoff, id_ind, acc);
                }
                mma_commit(a_empty + st.slot);
                mma_commit(b_empty + sw.slot);
                st.advance(1, S);
                sw.advance(1, SW);
            }
        }
        i += g + skip;
        st.advance(skip, S);
        sw.advance(skip, SW);
        len = G;
    }
    return true;
}

template <int NCH, bool MAIN, bool IND>
__device__ __forceinline__ bool tc8_mma_dispatch(const Tc8Args& a, uint32_t tmem, uint32_t d_main, uint32_t bsm_addr,
                                                 uint64_t* full_b, uint64_t* full_a, uint64_t* a_empty,
                                                 uint64_t* b_empty, uint64_t g0, uint32_t nkb, uint32_t start,
                                                 uint32_t len0, uint32_t skip) {
    if (a.group == 4)
        return tc8_mma_loop<NCH, MAIN, IND, 4>(a, tmem, d_main, bsm_addr, full_b, full_a, a_empty, b_empty, g0, nkb,
                                               start, len0, skip);
    if (a.group == 2)
        return tc8_mma_loop<NCH, MAIN, IND, 2>(a, tmem, d_main, bsm_addr, full_b, full_a, a_empty, b_empty, g0, nkb,
                                               start, len0, skip);
    return tc8_mma_loop<NCH, MAIN, IND, 1>(a, tmem, d_main, bsm_addr, full_b, full_a, a_empty, b_empty, g0, nkb,
                                           start, len0, skip);
}

// One CTA per SM runs work units u = blockIdx.x, blockIdx.x + gridDim.x, ...
// (unit u: row tile u % gx, K split u / gx); a launch with one CTA per unit
// is the same code with one unit each.  The copy and MMA rings run on across
// a CTA's units (stage g of the CTA's sequence sits in slot g % depth), so the
// producers prefetch the next unit's operands while the current unit's last
// stages and epilogue run; D is reused once the epilogue has read it
// (d_empty).  A unit's accumulation order depends only on its tile and
// split, so every grid gives the same bits.
__global__ void __launch_bounds__(kThreads, 1) k_tc8_rows(const __grid_constant__ Tc8Args a) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const uint32_t S = a.stages, SW = a.wstages, P = a.pstages;
    uint8_t* bsm = smem;
    uint8_t* psm = bsm + SW * a.b_stage_bytes;
    float* scl = reinterpret_cast<float*>(psm + P * kStageBytes);             // up to 512 floats
    uint64_t* bars = reinterpret_cast<uint64_t*>(reinterpret_cast<uint8_t*>(scl) + 2048);
    uint64_t* full_b = bars;                 // [SW] W stage landed (TMA tx)
    uint64_t* b_empty = bars + SW;           // [SW] every MMA warp's MMAs on the W stage done
    uint64_t* full_a = bars + 2 * SW;        // [S] A operand written to TMEM (128 arrivals)
    uint64_t* a_empty = full_a + S;          // [S] the MMAs reading the A stage done
    uint64_t* p_full = a_empty + S;          // [P] packed codes landed (TMA tx)
    uint64_t* p_empty = p_full + P;          // [P] packed codes consumed (4 warp arrivals)
    uint64_t* tmem_full = p_empty + P;       // a unit's MMAs done (both MMA warps commit)
    uint64_t* d_empty = tmem_full + 1;       // a unit's epilogue has read D (8 unpack warps)
    uint64_t* never = d_empty + 1;           // test hook: a barrier nothing arrives at
    uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(never + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool ind = a.n_ind != 0;
    auto unit_kb0 = [&](uint32_t u) { return (u / a.gx) * a.kb_per_split; };
    auto unit_nkb = [&](uint32_t u) {
        const uint32_t kb0 = unit_kb0(u), kb1 = min(a.kb_total, kb0 + a.kb_per_split);
        return kb1 > kb0 ? kb1 - kb0 : 0u;
    };
    // K order: the tiles of a launch all read the same W stages, and with
    // every CTA at the same stage the L2 serves one 56 KB stage to ~150 SMs
    // at once.  Each tile starts at its own stage (a rotation of the K loop,
    // fixed by its index in the matrix, so the accumulation order and the
    // bits do not depend on how rows are split into launches).
    auto unit_rot = [&](uint32_t u, uint32_t nkb) {
        return (a.rotate && nkb > 1) ? (uint32_t)(((a.tile0 + u % a.gx) * 37ull) % nkb) : 0u;
    };

    if (threadIdx.x == 0) {
        for (uint32_t s = 0; s < SW; ++s) {
            mbar_init(full_b + s, 1);
            mbar_init(b_empty + s, a.nsplit ? 2 : 1);   // every MMA warp that reads the stage commits
        }
        for (uint32_t s = 0; s < S; ++s) {
            mbar_init(full_a + s, 4);     // one arrival per unpack warp
            mbar_init(a_empty + s, a.nsplit ? 2 : 1);
        }
        for (uint32_t p = 0; p < P; ++p) {
            mbar_init(p_full + p, 1);
            mbar_init(p_empty + p, 4);
        }
        mbar_init(tmem_full, 2);
        mbar_init(d_empty, 4 * kUnpackSets);
        mbar_init(never, 1);
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
    const uint32_t tmem = *tmem_holder;

    // Test hook (slfmm_debug_expire_next_wait): before any copy or MMA is
    // issued, thread 0 waits on a barrier that nothing completes, bounded by
    // expire_cycles; the wait expires, sets the error flag (site 30), and the
    // CTA skips its work and frees its TMEM.  Nothing is in flight, so the
    // context stays usable.
    if (a.expire_cycles > 0) {
        if (threadIdx.x == 0) mbar_wait_for(never, 0, a.err, 30, a.expire_cycles);
    } else if (warp == 0) {
        if (lane == 0) {
            // packed-code producer: runs up to P stages ahead of the unpackers,
            // across units; each (tile, stage) operand is one contiguous bulk copy
            uint64_t g = 0, issued = 0;
            bool ok = true;
            for (uint32_t u = blockIdx.x; u < a.units && ok; u += gridDim.x) {
                const uint32_t nkb = unit_nkb(u), rot = unit_rot(u, nkb);
                const uint8_t* src =
                    a.tiles + (uint64_t)(u % a.gx) * a.tile_bytes + (uint64_t)unit_kb0(u) * kStageBytes;
                for (uint32_t i = 0; i < nkb; ++i, ++g) {
                    const uint32_t ks = i + rot < nkb ? i + rot : i + rot - nkb;
                    const Ring pr = ring_at(g, P);
                    if (g >= P && !mbar_wait(p_empty + pr.slot, pr.phase ^ 1u, a.err, 21)) {
                        ok = false;
                        break;
                    }
                    mbar_arrive_tx(p_full + pr.slot, kStageBytes);
                    bulk_g2s(psm + pr.slot * kStageBytes, src + (uint64_t)ks * kStageBytes, kStageBytes,
                             p_full + pr.slot);
                    issued = g + 1;
                }
            }
            // never leave with copies in flight into this CTA's shared memory
            for (uint64_t q = issued > P ? issued - P : 0; q < issued; ++q) {
                const Ring pr = ring_at(q, P);
                mbar_wait(p_full + pr.slot, pr.phase, a.err, 22);
            }
        }
    } else if (warp == 2) {
        // each spinning role has a warp of its own: lanes of one warp that
        // spin in different loops starve each other
        if (lane == 0) {
            // W producer: one bulk copy per stage, across units
            uint64_t g = 0, issued = 0;
            bool ok = true;
            for (uint32_t u = blockIdx.x; u < a.units && ok; u += gridDim.x) {
                const uint32_t nkb = unit_nkb(u), rot = unit_rot(u, nkb), kb0 = unit_kb0(u);
                for (uint32_t i = 0; i < nkb; ++i, ++g) {
                    const uint32_t ks = i + rot < nkb ? i + rot : i + rot - nkb;
                    const Ring wr = ring_at(g, SW);
                    if (g >= SW && !mbar_wait(b_empty + wr.slot, wr.phase ^ 1u, a.err, 23)) {
                        ok = false;
                        break;
                    }
                    mbar_arrive_tx(full_b + wr.slot, a.b_stage_bytes);
                    bulk_g2s(bsm + wr.slot * a.b_stage_bytes, a.wop + (uint64_t)(kb0 + ks) * a.b_stage_bytes,
                             a.b_stage_bytes, full_b + wr.slot);
                    issued = g + 1;
                }
            }
            for (uint64_t q = issued > SW ? issued - SW : 0; q < issued; ++q) {
                const Ring wr = ring_at(q, SW);
                mbar_wait(full_b + wr.slot, wr.phase, a.err, 24);
            }
        }
    } else if (warp == 1 || warp == 3) {
        if (lane == 0) {
            const uint32_t m = warp == 1 ? 0u : 1u;  // MMA warp index
            const uint32_t bsm_addr = smem_u32(bsm);
            const uint32_t G = a.group;
            const int nch = a.n_main > 256 ? 2 : 1;  // host guarantees an even split into <= 256-wide MMAs
            uint64_t g0 = 0;
            uint32_t k = 0;  // this CTA's units so far
            bool ok = true;
            for (uint32_t u = blockIdx.x; u < a.units && ok; u += gridDim.x, ++k) {
                const uint32_t nkb = unit_nkb(u);
                // D is free once the previous unit's epilogue has read it
                if (k > 0) {
                    ok = mbar_wait(d_empty, (k - 1) & 1u, a.err, 31);
                    fence_after();
                }
                if (ok && a.nsplit) {
                    // genotype MMAs on warp 0, indicator MMAs on warp 1, boundaries G/2 apart
                    if (m == 0) {
                        if (nch == 1)
                            ok = tc8_mma_dispatch<1, true, false>(a, tmem, tmem, bsm_addr, full_b, full_a, a_empty,
                                                                  b_empty, g0, nkb, 0, G, 0);
                        else
                            ok = tc8_mma_dispatch<2, true, false>(a, tmem, tmem, bsm_addr, full_b, full_a, a_empty,
                                                                  b_empty, g0, nkb, 0, G, 0);
                    } else {
                        ok = tc8_mma_dispatch<1, false, true>(a, tmem, tmem, bsm_addr, full_b, full_a, a_empty,
                                                              b_empty, g0, nkb, 0, G > 1 ? G / 2 : 1, 0);
                    }
                } else if (ok && a.kcopies == 2) {
                    // alternate groups of G K blocks into accumulator copies m
                    const uint32_t d_main = tmem + m * a.d_cols;
                    if (nch == 1)
                        ok = tc8_mma_dispatch<1, true, false>(a, tmem, d_main, bsm_addr, full_b, full_a, a_empty,
                                                              b_empty, g0, nkb, m * G, G, G);
                    else
                        ok = tc8_mma_dispatch<2, true, false>(a, tmem, d_main, bsm_addr, full_b, full_a, a_empty,
                                                              b_empty, g0, nkb, m * G, G, G);
                } else if (ok && m == 0) {
                    // one MMA warp does everything
                    if (nch == 1) {
                        if (ind)
                            ok = tc8_mma_dispatch<1, true, true>(a, tmem, tmem, bsm_addr, full_b, full_a, a_empty,
                                                                 b_empty, g0, nkb, 0, G, 0);
                        else
                            ok = tc8_mma_dispatch<1, true, false>(a, tmem, tmem, bsm_addr, full_b, full_a, a_empty,
                                                                  b_empty, g0, nkb, 0, G, 0);
                    } else {
                        if (ind)
                            ok = tc8_mma_dispatch<2, true, true>(a, tmem, tmem, bsm_addr, full_b, full_a, a_empty,
                                                                 b_empty, g0, nkb, 0, G, 0);
                        else
                            ok = tc8_mma_dispatch<2, true, false>(a, tmem, tmem, bsm_addr, full_b, full_a, a_empty,
                                                                  b_empty, g0, nkb, 0, G, 0);
                    }
                }
                mma_commit(tmem_full);  // both MMA warps arrive per unit (an idle one at once)
                g0 += nkb;
            }
        }
    } else {
        // kUnpackSets sets of four unpack warps take the stages of the CTA's
        // sequence round robin; warp % 4 is the TMEM lane quarter a warp may access
        const uint32_t set = (uint32_t)(warp - 4) >> 2;
        const uint32_t q = (uint32_t)warp & 3u;
        const uint32_t row = q * 32 + lane;
        const uint32_t lane_base = tmem + ((q * 32) << 16);
        const uint32_t nsets = a.usets;
        uint64_t g0 = 0;
        uint32_t k = 0;
        bool ok = true;
        for (uint32_t u = blockIdx.x; u < a.units && ok; u += gridDim.x, ++k) {
            const uint32_t nkb = unit_nkb(u);
            for (uint32_t i = 0; i < nkb && set < nsets; ++i) {
                const uint64_t g = g0 + i;
                if (g % nsets != set) continue;
                const Ring pr = ring_at(g, P), st = ring_at(g, S);
                // one lane polls each barrier and the warp follows it (the warp
                // barrier orders the other lanes after its observation)
                if (!warp_wait(p_full + pr.slot, pr.phase, a.err, 27)) {
                    ok = false;
                    break;
                }
                // this row's 256 codes: 32 B in each of the stage's two tile blocks
                const uint8_t* rp = psm + pr.slot * kStageBytes + row * (kTileK / 4);
                const uint4 p0 = reinterpret_cast<const uint4*>(rp)[0], p1 = reinterpret_cast<const uint4*>(rp)[1];
                const uint4 p2 = reinterpret_cast<const uint4*>(rp + kTileBytes)[0];
                const uint4 p3 = reinterpret_cast<const uint4*>(rp + kTileBytes)[1];
                __syncwarp();
                if (lane == 0) mbar_arrive(p_empty + pr.slot);   // codes are in registers: release the slot
                // a 32-bit word holds 16 two-bit codes; masking the even / odd codes
                // into nibbles gives PRMT selectors directly (4 codes per PRMT), and
                // the B operand stores K in the matching even-then-odd order
                const uint32_t w16[16] = {p0.x, p0.y, p0.z, p0.w, p1.x, p1.y, p1.z, p1.w,
                                          p2.x, p2.y, p2.z, p2.w, p3.x, p3.y, p3.z, p3.w};
                uint32_t ev[16], od[16];
#pragma unroll
                for (int t = 0; t < 16; ++t) {
                    ev[t] = w16[t] & 0x33333333u;
                    od[t] = (w16[t] >> 2) & 0x33333333u;
                }
                uint32_t gv[32], h[32];
#pragma unroll
                for (int t = 0; t < 8; ++t) {
                    gv[4 * t] = __byte_perm(kTabGeno, 0u, ev[t]);
                    gv[4 * t + 1] = __byte_perm(kTabGeno, 0u, ev[t] >> 16);
                    gv[4 * t + 2] = __byte_perm(kTabGeno, 0u, od[t]);
                    gv[4 * t + 3] = __byte_perm(kTabGeno, 0u, od[t] >> 16);
                    h[4 * t] = __byte_perm(kTabGeno, 0u, ev[8 + t]);
                    h[4 * t + 1] = __byte_perm(kTabGeno, 0u, ev[8 + t] >> 16);
                    h[4 * t + 2] = __byte_perm(kTabGeno, 0u, od[8 + t]);
                    h[4 * t + 3] = __byte_perm(kTabGeno, 0u, od[8 + t] >> 16);
                }
                keep32(gv);  // expanded before the stage wait: only the stores follow it
                keep32(h);
                if (g >= S && !warp_wait(a_empty + st.slot, st.phase ^ 1u, a.err, 28)) {
                    ok = false;
                    break;
                }
                const uint32_t a_col = lane_base + a.a_base + st.slot * a.a_cols;
                tmem_st_x32(a_col, gv);
                tmem_st_x32(a_col + 32, h);
                if (ind) {
#pragma unroll
                    for (int t = 0; t < 8; ++t) {
                        gv[4 * t] = __byte_perm(kTabMiss, 0u, ev[t]);
                        gv[4 * t + 1] = __byte_perm(kTabMiss, 0u, ev[t] >> 16);
                        gv[4 * t + 2] = __byte_perm(kTabMiss, 0u, od[t]);
                        gv[4 * t + 3] = __byte_perm(kTabMiss, 0u, od[t] >> 16);
                        h[4 * t] = __byte_perm(kTabMiss, 0u, ev[8 + t]);
                        h[4 * t + 1] = __byte_perm(kTabMiss, 0u, ev[8 + t] >> 16);
                        h[4 * t + 2] = __byte_perm(kTabMiss, 0u, od[8 + t]);
                        h[4 * t + 3] = __byte_perm(kTabMiss, 0u, od[8 + t] >> 16);
                    }
                    tmem_st_x32(a_col + 64, gv);
                    tmem_st_x32(a_col + 96, h);
                }
                asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
                fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(full_a + st.slot);
            }
            if (!ok) break;
            // epilogue of unit u: the sets take 16-column groups round robin
            ok = warp_wait(tmem_full, k & 1u, a.err, 29);
            // the second accumulator copy holds data only if its first group exists
            const bool second_copy = a.kcopies == 2 && nkb > a.group;
            fence_after();
            const uint32_t grow = (u % a.gx) * kM + row;
            const bool live = ok && grow < a.rows;
            double rm = 0.0, rs = 0.0;
            if (a.mode == 1 && live) {
                rm = a.row_mean[grow];
                rs = a.row_scale[grow];
            }
            float* dst = a.out + (uint64_t)(u / a.gx) * a.split_stride + (uint64_t)grow * a.ldo;
            for (uint32_t c0 = set * 16; c0 < a.wpad && ok; c0 += 16 * kUnpackSets) {
                float pm[16], pi[16], v[16];
#pragma unroll
                for (int kk = 0; kk < 16; ++kk) pm[kk] = pi[kk] = 0.f;
                for (int t = 0; t < kMainTerms; ++t) {
                    const uint32_t col = t * a.wpad + c0;
                    tmem_ld_x16(lane_base + col, v);
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                    if (second_copy) {
                        float v2[16];
                        tmem_ld_x16(lane_base + a.d_cols + col, v2);
                        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                        for (int kk = 0; kk < 16; ++kk) v[kk] += v2[kk];
                    }
#pragma unroll
                    for (int kk = 0; kk < 16; ++kk) pm[kk] = fmaf(scl[col + kk], v[kk], pm[kk]);
                }
                if (ind) {
                    for (int t = 0; t < kIndTerms; ++t) {
                        const uint32_t col = a.n_main + t * a.wpad + c0;
                        const uint32_t scol = (a.ind_shared ? 0u : a.n_main) + t * a.wpad + c0;
                        tmem_ld_x16(lane_base + col, v);
                        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                        for (int kk = 0; kk < 16; ++kk) pi[kk] = fmaf(scl[scol + kk], v[kk], pi[kk]);
                    }
                }
                if (live) {
#pragma unroll
                    for (int kk = 0; kk < 16; ++kk) {
                        if (a.mode == 1)
                            v[kk] = (float)(rs * ((double)pm[kk] - rm * (a.cs[c0 + kk] - (double)pi[kk])));
                        else
                            v[kk] = pm[kk] + pi[kk];
                    }
                    float4* d4 = reinterpret_cast<float4*>(dst + c0);
#pragma unroll
                    for (int t = 0; t < 4; ++t) d4[t] = make_float4(v[4 * t], v[4 * t + 1], v[4 * t + 2], v[4 * t + 3]);
                }
            }
            // D may be overwritten by the next unit's MMAs
            fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(d_empty);
            g0 += nkb;
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

// per-column max |x * kscale| as float bits (non-negative floats order as
// ints); one warp per row, lanes over columns (w <= 128), the per-row scale
// converted once per row
template <typename T>
__global__ void __launch_bounds__(256) k_colmax_abs(const T* __restrict__ src, int ld, uint64_t K, int w,
                                                    const double* __restrict__ kscale, unsigned* __restrict__ colmax) {
    const int lane = threadIdx.x & 31;
    float m[4] = {0.f, 0.f, 0.f, 0.f};
    const uint64_t nw = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t k = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); k < K; k += nw) {
        float ks = 1.f;
        if (kscale) {
            if (lane == 0) ks = (float)kscale[k];
            ks = __shfl_sync(0xffffffffu, ks, 0);
        }
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int c = lane + 32 * t;
            if (c < w) m[t] = fmaxf(m[t], fabsf((float)src[k * ld + c] * ks));
        }
    }
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        const int c = lane + 32 * t;
        if (c < w) atomicMax(colmax + c, __float_as_uint(m[t]));
    }
}

__device__ __forceinline__ int term_e0(unsigned bits) {
    const float cm = __uint_as_float(bits);
    if (!(cm > 0.f)) return 0;
    int E;
    frexpf(cm, &E);
    return 8 - E;  // cm * 2^e0 in [128, 256)
}

// exact 2^ex as a float (ldexpf outside the normal exponent range)
__device__ __forceinline__ float pow2f(int ex) {
    return (ex >= -126 && ex <= 127) ? __int_as_float((127 + ex) << 23) : ldexpf(1.f, ex);
}

// Byte offset of element (row, k) of a stage-major W operand with n_rows rows:
// stage kb = k / 256 is the contiguous blob [half][row][128 B] at
// kb * n_rows * 256, and within each 128-byte row the 16-byte chunk j sits at
// chunk j ^ (row & 7) -- the 128-byte swizzle the MMA descriptors expect of a
// 1024-byte aligned shared-memory stage (n_rows % 8 == 0 keeps every half's
// rows aligned to the 8-row swizzle period).
__device__ __forceinline__ uint64_t wop_offset(uint32_t row, uint64_t k, uint32_t n_rows) {
    const uint64_t kb = k >> 8;
    const uint32_t h = (uint32_t)(k >> 7) & 1u, kk = (uint32_t)k & 127u;
    return kb * (uint64_t)n_rows * 256 + (uint64_t)(h * n_rows + row) * 128 +
           ((((kk >> 4) ^ (row & 7u)) << 4) | (kk & 15u));
}

// W (K x w) -> `terms` E4M3 rows per column at B rows row_off + t * wpad + c
// of a stage-major operand with n_rows rows (wop_offset), zero padded to
// K_pad; inv_scale[row] = 2^-(e0 + 4t).
// Term t is round_e4m3((r - terms_<t) * 2^(e0 + 4t)); the power-of-two scales
// are exact, so each step's residual is rounded once.
template <typename T>
__global__ void __launch_bounds__(256) k_fp8_terms(const T* __restrict__ src, int ld, uint64_t K, int w, int wpad,
                                                   uint64_t K_pad, const double* __restrict__ kscale, int terms,
                                                   int row_off, int n_rows, const unsigned* __restrict__ colmax,
                                                   uint8_t* __restrict__ B, float* __restrict__ inv_scale) {
    __shared__ __align__(16) uint8_t tile[kMainTerms][32][132];
    __shared__ float ks[128];
    __shared__ int e0s[32];
    const uint64_t k0 = (uint64_t)blockIdx.x * 128;
    const int c0 = blockIdx.y * 32;
    for (int i = threadIdx.x; i < 128; i += blockDim.x) {
        const uint64_t k = k0 + i;
        ks[i] = (kscale && k < K) ? (float)kscale[k] : 1.f;
    }
    for (int i = threadIdx.x; i < 32; i += blockDim.x) {
        const int c = c0 + i;
        e0s[i] = c < w ? term_e0(colmax[c]) : 0;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 128 * 32; e += blockDim.x) {
        const int kk = e / 32, cc = e % 32;
        const uint64_t k = k0 + kk;
        const int c = c0 + cc;
        float r = 0.f;
        if (k < K && c < w) r = (float)src[k * ld + c] * ks[kk];
        const int e0 = e0s[cc];
        for (int t = 0; t < terms; ++t) {
            const int ex = e0 + 4 * t;
            const __nv_fp8_storage_t qv = __nv_cvt_float_to_fp8(r * pow2f(ex), __NV_SATFINITE, __NV_E4M3);
            const __half_raw hr = __nv_cvt_fp8_to_halfraw(qv, __NV_E4M3);
            r = fmaf(-__half2float(__half(hr)), pow2f(-ex), r);
            tile[t][cc][kk] = (uint8_t)qv;
        }
    }
    __syncthreads();
    if (blockIdx.x == 0)
        for (int e = threadIdx.x; e < terms * 32; e += blockDim.x) {
            const int t = e / 32, cc = e % 32, c = c0 + cc;
            if (c < wpad) inv_scale[row_off + t * wpad + c] = c < w ? pow2f(-(e0s[cc] + 4 * t)) : 1.f;
        }
    // B position kp within each 16-group holds K index kk = perm(kp): the even
    // K indices of the group, then the odd ones (the order the unpackers emit
    // the genotypes of a 32-bit code word in); written as 32-bit words
    for (int e = threadIdx.x; e < terms * 32 * 32; e += blockDim.x) {
        const int t = e / (32 * 32), rem = e % (32 * 32), cc = rem / 32, kp0 = (rem % 32) * 4;
        const int c = c0 + cc;
        if (c >= wpad) continue;
        uint32_t word = 0;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int kp = kp0 + b;
            const int kk = (kp & ~15) | ((kp & 7) << 1) | ((kp >> 3) & 1);
            word |= (uint32_t)tile[t][cc][kk] << (8 * b);
        }
        *reinterpret_cast<uint32_t*>(B + wop_offset((uint32_t)(row_off + t * wpad + c), k0 + kp0, (uint32_t)n_rows)) =
            word;
    }
}

// The two scalings of one narrow FP32 operand that a transposed pass splits
// (diag(s) Q for the genotypes, diag(mu s) Q for the missing-call indicator).
struct TermSet {
    const double* kscale;    // per-K-row scale (null: 1)
    int terms;               // E4M3 terms (0: set absent)
    int row_off;             // first B row of the set
    const unsigned* colmax;  // per-column max |x * kscale| (float bits)
};

// Per-column max |x kscale| of both sets in one pass over a narrow operand
// (w <= ld <= 32, ld % 4 == 0, 16-byte aligned rows): a thread keeps one
// 16-byte column quad and walks rows, four rows in flight; lanes with the
// same quad are combined by shuffles before the atomics.
__global__ void __launch_bounds__(256) k_colmax_pair(const float* __restrict__ src, int ld, uint64_t K, int w,
                                                     const double* __restrict__ ksa, const double* __restrict__ ksb,
                                                     unsigned* __restrict__ cma, unsigned* __restrict__ cmb) {
    const int q = ld >> 2;  // quads per row: 1, 2, 4 or 8 (divides the thread count)
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t nthreads = (uint64_t)gridDim.x * blockDim.x;
    const int qp = (int)(tid % q);
    const uint64_t step = nthreads / q;
    const float4* s4 = reinterpret_cast<const float4*>(src);
    float ma[4] = {0.f, 0.f, 0.f, 0.f}, mb[4] = {0.f, 0.f, 0.f, 0.f};
    for (uint64_t j0 = tid / q; j0 < K; j0 += 4 * step) {
        float4 v[4];
        float fa[4], fb[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint64_t j = j0 + u * step;
            const bool ok = j < K;
            v[u] = ok ? s4[j * q + qp] : make_float4(0.f, 0.f, 0.f, 0.f);
            fa[u] = ok && ksa ? (float)ksa[j] : 1.f;
            fb[u] = ok && ksb ? (float)ksb[j] : 1.f;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const float x[4] = {v[u].x, v[u].y, v[u].z, v[u].w};
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                ma[i] = fmaxf(ma[i], fabsf(x[i] * fa[u]));
                mb[i] = fmaxf(mb[i], fabsf(x[i] * fb[u]));
            }
        }
    }
    // lanes l, l + q, l + 2q, ... of a warp hold the same quad
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        if (o < q) break;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            ma[i] = fmaxf(ma[i], __shfl_xor_sync(0xffffffffu, ma[i], o));
            mb[i] = fmaxf(mb[i], __shfl_xor_sync(0xffffffffu, mb[i], o));
        }
    }
    // then the block's warps through shared memory: one atomic per column
    // and block (non-negative floats order as their bits)
    __shared__ unsigned red[8][2][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane < q) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            red[warp][0][4 * lane + i] = __float_as_uint(ma[i]);
            red[warp][1][4 * lane + i] = __float_as_uint(mb[i]);
        }
    }
    __syncthreads();
    if (threadIdx.x < 64) {
        const int set = threadIdx.x >> 5, c = threadIdx.x & 31;
        unsigned* dst = set ? cmb : cma;
        if (c < w && c < 4 * q && dst) {
            unsigned m = 0;
            for (int wv = 0; wv < (int)(blockDim.x >> 5); ++wv) m = max(m, red[wv][set][c]);
            atomicMax(dst + c, m);
        }
    }
}

// Split-FP8 terms of both sets in one pass (the loads of the operand are
// shared): as k_fp8_terms, with two K rows per E4M3 conversion (the paired
// conversion rounds each value as the scalar one does, so the terms are the
// same) and the power-of-two scales taken from per-column tables.
__global__ void __launch_bounds__(256) k_fp8_terms_pair(const float* __restrict__ src, int ld, uint64_t K, int w,
                                                        int wpad, uint64_t K_pad, TermSet sa, TermSet sb, int n_rows,
                                                        uint8_t* __restrict__ B, float* __restrict__ inv_scale) {
    constexpr int kT = kMainTerms + kIndTerms;
    __shared__ __align__(16) uint8_t tile[kT][32][132];
    __shared__ float ksa[128], ksb[128];
    __shared__ float up[kT][32], dn[kT][32];
    const uint64_t k0 = (uint64_t)blockIdx.x * 128;
    const int c0 = blockIdx.y * 32;
    const int nt = sa.terms + sb.terms;
    for (int i = threadIdx.x; i < 128; i += blockDim.x) {
        const uint64_t k = k0 + i;
        ksa[i] = (sa.kscale && k < K) ? (float)sa.kscale[k] : 1.f;
        ksb[i] = (sb.kscale && k < K) ? (float)sb.kscale[k] : 1.f;
    }
    for (int e = threadIdx.x; e < nt * 32; e += blockDim.x) {
        const int t = e / 32, cc = e % 32, c = c0 + cc;
        const bool first = t < sa.terms;
        const int tt = first ? t : t - sa.terms;
        const int e0 = c < w ? term_e0((first ? sa.colmax : sb.colmax)[c]) : 0;
        up[t][cc] = pow2f(e0 + 4 * tt);
        dn[t][cc] = pow2f(-(e0 + 4 * tt));
        if (blockIdx.x == 0 && c < wpad)
            inv_scale[(first ? sa.row_off : sb.row_off) + tt * wpad + c] = c < w ? pow2f(-(e0 + 4 * tt)) : 1.f;
    }
    __syncthreads();
    for (int pr = threadIdx.x; pr < 64 * 32; pr += blockDim.x) {
        const int kk = 2 * (pr / 32), cc = pr % 32;
        const uint64_t k = k0 + kk;
        const int c = c0 + cc;
        float x0 = 0.f, x1 = 0.f;
        if (c < w) {
            if (k < K) x0 = (float)src[k * ld + c];
            if (k + 1 < K) x1 = (float)src[(k + 1) * ld + c];
        }
#pragma unroll
        for (int set = 0; set < 2; ++set) {
            const int terms = set ? sb.terms : sa.terms, base = set ? sa.terms : 0;
            const float* ks = set ? ksb : ksa;
            float r0 = x0 * ks[kk], r1 = x1 * ks[kk + 1];
#pragma unroll
            for (int t = 0; t < kMainTerms; ++t) {
                if (t < terms) {
                    const float u = up[base + t][cc], d = dn[base + t][cc];
                    const __nv_fp8x2_storage_t q2 =
                        __nv_cvt_float2_to_fp8x2(make_float2(r0 * u, r1 * u), __NV_SATFINITE, __NV_E4M3);
                    const float2 f = __half22float2(__half2(__nv_cvt_fp8x2_to_halfraw2(q2, __NV_E4M3)));
                    r0 = fmaf(-f.x, d, r0);
                    r1 = fmaf(-f.y, d, r1);
                    tile[base + t][cc][kk] = (uint8_t)(q2 & 0xffu);
                    tile[base + t][cc][kk + 1] = (uint8_t)(q2 >> 8);
                }
            }
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < nt * 32 * 32; e += blockDim.x) {
        const int t = e / (32 * 32), rem = e % (32 * 32), cc = rem / 32, kp0 = (rem % 32) * 4;
        const int c = c0 + cc;
        if (c >= wpad) continue;
        const int row = t < sa.terms ? sa.row_off + t * wpad + c : sb.row_off + (t - sa.terms) * wpad + c;
        uint32_t word = 0;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int kp = kp0 + b;
            const int kk = (kp & ~15) | ((kp & 7) << 1) | ((kp >> 3) & 1);
            word |= (uint32_t)tile[t][cc][kk] << (8 * b);
        }
        *reinterpret_cast<uint32_t*>(B + wop_offset((uint32_t)row, k0 + kp0, (uint32_t)n_rows)) = word;
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

}  // namespace

// Tuning overrides (autotuner / experiments): SLFMM_TC8_STAGES, _PSTAGES, _GROUP.
static int env_int(const char* name, int dflt) {
    const char* v = std::getenv(name);
    return v && *v ? std::atoi(v) : dflt;
}

// The plan with explicit caps on the packed-code ring (pmax), the W ring
// (smax) and the MMA wait group (gmax); fp8_plan takes them from the
// environment (defaults 8, 8, 4).
Fp8Plan fp8_plan_knobs(int wpad, bool ind, uint64_t tiles, int pmax_in, int smax, int gmax_in, int wmax,
                       bool ind_shared) {
    Fp8Plan p{};
    p.wpad = (uint32_t)wpad;
    p.n_main = kMainTerms * wpad;
    p.n_ind = ind ? kIndTerms * wpad : 0;
    p.ind_shared = (ind && ind_shared) ? 1u : 0u;
    p.n_total = p.ind_shared ? p.n_main : p.n_main + p.n_ind;      // B rows
    p.d_cols = (uint32_t)round_up(p.n_main + p.n_ind, 32);       // accumulator columns
    p.a_cols = (ind ? 2 : 1) * (kStageK / 4);  // TMEM columns of one stage's A operand(s)
    p.b_stage_bytes = p.n_total * 128 * kHalves;  // one bulk copy: 16-byte multiple, below the 1 MB tx limit
    // one CTA per SM: all of TMEM; the packed-code ring gives up depth (8, 4,
    // then 2 stages) until shared memory holds at least two W stages
    p.tmem_cols = 512;
    const size_t fixed = 1024 + 2048 + 128 * 8 + 64;
    // MMA warp roles: with the indicator, genotype and indicator MMAs on
    // separate warps; without it, two accumulator copies when TMEM holds them
    // next to at least three A stages
    p.nsplit = ind ? 1 : 0;
    p.kcopies = (!ind && 2 * p.d_cols + 3 * p.a_cols <= 512) ? 2 : 1;
    p.a_base = p.kcopies * p.d_cols;
    const uint32_t by_tmem = p.a_base < 512 ? (512 - p.a_base) / p.a_cols : 0;
    // A ring: as deep as TMEM allows (cap smax).  W ring: its own depth in
    // shared memory, at least one stage more than the A ring and at least 3
    // where it fits (cap wmax): a W stage is refilled only after the MMAs on
    // it complete, and the refill comes from L2 (the same W for every CTA).
    // The packed-code ring gives up depth (pmax, halving down to 2) for it.
    p.stages = std::min<uint32_t>(by_tmem, (uint32_t)std::max(1, smax));
    const uint32_t pmax = (uint32_t)std::min(16, std::max(2, pmax_in));
    const uint32_t wcap = (uint32_t)std::max(1, std::min(16, wmax));
    const uint32_t wwant = std::min(wcap, std::max(p.stages + 1, 3u));
    uint32_t by_smem = 0;
    for (p.pstages = pmax;; p.pstages /= 2) {
        const size_t budget = 225 * 1024 - fixed - (size_t)p.pstages * kStageBytes;
        by_smem = (uint32_t)(budget / p.b_stage_bytes);
        if (by_smem >= wwant || p.pstages <= 2) break;
    }
    p.wstages = std::min(by_smem, wcap);
    p.stages = std::min(p.stages, p.wstages);
    // MMA wait groups: up to 16 MMAs per wait and warp, at least two groups in the ring
    const uint32_t nch = p.n_main > 256 ? 2 : 1;
    const uint32_t per_stage = (kStageK / 32) * (p.nsplit || p.kcopies == 2 ? nch : nch + (ind ? 1 : 0));
    p.group = 1;
    const uint32_t gmax = (uint32_t)gmax_in;
    for (uint32_t gsz : {4u, 2u})
        if (gsz <= gmax && gsz * per_stage <= 16 && p.stages >= 2 * gsz) {
            p.group = gsz;
            break;
        }
    p.stages -= p.stages % p.group;
    p.smem = fixed + (size_t)p.pstages * kStageBytes + (size_t)p.wstages * p.b_stage_bytes;
    (void)tiles;
    p.ok = p.n_total % 8 == 0 && p.stages >= 2 && p.n_main % ceil_div(p.n_main, 256) == 0 && (p.n_main / ceil_div(p.n_main, 256)) % 16 == 0 &&
           p.n_ind <= 256;
    return p;
}

Fp8Plan fp8_plan(int wpad, bool ind, uint64_t tiles, bool ind_shared) {
    return fp8_plan_knobs(wpad, ind, tiles, env_int("SLFMM_TC8_PSTAGES", 8), env_int("SLFMM_TC8_STAGES", 8),
                          env_int("SLFMM_TC8_GROUP", 4), env_int("SLFMM_TC8_WSTAGES", 8),
                          ind_shared && env_int("SLFMM_TC8_SHARED_IND", 1) != 0);
}

// row-major packed rows (rows x stride) -> tile-major copy; one thread per
// 16-byte output chunk, so the writes stream and every read is one full
// 32-byte sector
__global__ void k_tile_rows(const uint8_t* __restrict__ in, uint64_t rows, uint64_t stride, uint64_t kbt,
                            uint64_t chunks, uint8_t* __restrict__ out) {
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < chunks;
         e += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t h = e & 1u, r = (e >> 1) & 127u, rest = e >> 8;
        const uint64_t kb = rest % kbt, t = rest / kbt;
        const uint64_t row = t * kM + r, col = kb * 32 + h * 16;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (row < rows && col < stride) v = *reinterpret_cast<const uint4*>(in + row * stride + col);
        reinterpret_cast<uint4*>(out)[e] = v;
    }
}

// Tile-major transpose of the 2-bit matrix.  Block (t, kb) of the output --
// 128 samples of sample tile t x the 128 SNPs of K block kb -- is the 2-bit
// transpose of block (kb, t) of the SNP-row tiles; both are contiguous 4 KiB
// runs.  One block per iteration: a coalesced 4 KiB load into shared memory,
// each thread then assembles 4 output words (16 codes each) of one sample
// from 16 SNP rows, and the 4 KiB result is stored contiguously.
__global__ void __launch_bounds__(256) k_transpose_tiles(const uint8_t* __restrict__ src, uint64_t kbt_src,
                                                         uint64_t ntiles_src, uint8_t* __restrict__ dst,
                                                         uint64_t kbt_dst, uint64_t ntiles_dst, uint64_t kb_lo,
                                                         uint64_t kb_hi) {
    __shared__ __align__(16) uint8_t in[128 * 32];
    const uint64_t nk = kb_hi - kb_lo;  // output K blocks [kb_lo, kb_hi) of every sample tile
    const uint64_t nblocks = ntiles_dst * nk;
    const int j = threadIdx.x & 127;   // sample within the tile
    const int h = threadIdx.x >> 7;    // which 64 SNPs
    for (uint64_t bb = blockIdx.x; bb < nblocks; bb += gridDim.x) {
        const uint64_t t = bb / nk, kb = kb_lo + (bb - t * nk);
        const uint64_t b = t * kbt_dst + kb;
        const bool valid = kb < ntiles_src && t < kbt_src;
        __syncthreads();
        const uint4* s4 = reinterpret_cast<const uint4*>(src + (kb * kbt_src + t) * (uint64_t)kTileBytes);
        reinterpret_cast<uint4*>(in)[threadIdx.x] = valid ? s4[threadIdx.x] : make_uint4(0, 0, 0, 0);
        __syncthreads();
        const int byte = j >> 2, shift = 2 * (j & 3);
        uint32_t wv[4];
#pragma unroll
        for (int w = 0; w < 4; ++w) {
            uint32_t v = 0;
#pragma unroll
            for (int ii = 0; ii < 16; ++ii) {
                const int i = h * 64 + w * 16 + ii;  // SNP within the K block
                v |= (uint32_t)((in[i * 32 + byte] >> shift) & 3u) << (2 * ii);
            }
            wv[w] = v;
        }
        *reinterpret_cast<uint4*>(dst + b * (uint64_t)kTileBytes + j * 32 + h * 16) = make_uint4(wv[0], wv[1], wv[2], wv[3]);
    }
}

// Sample-major tiles of a sample subset: row rr of output sample tile ts
// (output sample s = 128 ts + rr) is row i % 128 of source tile i / 128, i =
// keep[s], in every K block; samples past n_keep are zero codes.  One thread
// per 16 bytes (two per 32-byte tile row).
__global__ void k_gather_tile_rows(const uint8_t* __restrict__ src, uint64_t kbt, const uint32_t* __restrict__ keep,
                                   uint64_t n_keep, uint64_t ntiles_dst, uint8_t* __restrict__ dst) {
    const uint64_t total = ntiles_dst * kbt * 256;
    const uint4* s4 = reinterpret_cast<const uint4*>(src);
    uint4* d4 = reinterpret_cast<uint4*>(dst);
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t h = e & 1u, rr = (e >> 1) & 127u, rest = e >> 8;
        const uint64_t kb = rest % kbt, ts = rest / kbt;
        const uint64_t sidx = ts * kM + rr;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (sidx < n_keep) {
            const uint64_t i = keep[sidx];
            v = s4[((i / kM) * kbt + kb) * 256 + (i % kM) * 2 + h];
        }
        d4[e] = v;
    }
}

// Allele and missing counts of every SNP from the SNP-major tiles (the
// codes of samples past n are 00 there): one warp per SNP, lanes over the
// K blocks of its tile row; counts as k_snp_counts (c0 = n - c1 - c2 - cm).
__global__ void k_snp_counts_tiles(const uint8_t* __restrict__ tiles, uint64_t kbt, uint64_t p, uint64_t n,
                                   int32_t* __restrict__ counts) {
    constexpr uint32_t kLo2 = 0x55555555u;
    const uint64_t j = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32;
    const int lane = threadIdx.x & 31;
    if (j >= p) return;
    const uint64_t t = j / kM, r = j % kM;
    uint32_t c1 = 0, c2 = 0, cm = 0;
    for (uint64_t kb = lane; kb < kbt; kb += 32) {
        const uint4* q = reinterpret_cast<const uint4*>(tiles + (t * kbt + kb) * kTileBytes + r * 32);
        const uint4 a = q[0], b = q[1];
        const uint32_t ws[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const uint32_t lo = ws[k] & kLo2, hi = (ws[k] >> 1) & kLo2;
            c1 += __popc(hi & ~lo);
            c2 += __popc(hi & lo);
            cm += __popc(~hi & lo);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        c1 += __shfl_xor_sync(0xffffffffu, c1, o);
        c2 += __shfl_xor_sync(0xffffffffu, c2, o);
        cm += __shfl_xor_sync(0xffffffffu, cm, o);
    }
    if (lane == 0) {
        counts[j * 4 + 0] = (int32_t)(n - c1 - c2 - cm);
        counts[j * 4 + 1] = (int32_t)c1;
        counts[j * 4 + 2] = (int32_t)c2;
        counts[j * 4 + 3] = (int32_t)cm;
    }
}

// Missing-call lists (CSR by SNP, ascending sample indices) of a matrix held
// only as SNP-major tiles: one warp per SNP, lanes over 32 K blocks at a
// time; a lane's missing calls (code 01) are placed after those of the lower
// lanes by a warp scan of the per-lane counts.
__global__ void k_miss_fill_tiles(const uint8_t* __restrict__ tiles, uint64_t kbt, uint64_t p,
                                  const uint64_t* __restrict__ ptr, uint32_t* __restrict__ idx) {
    constexpr uint32_t kLo2 = 0x55555555u;
    const uint64_t j = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32;
    const int lane = threadIdx.x & 31;
    if (j >= p) return;
    const uint64_t t = j / kM, r = j % kM;
    uint64_t base = ptr[j];
    for (uint64_t kb0 = 0; kb0 < kbt; kb0 += 32) {
        const uint64_t kb = kb0 + lane;
        uint32_t m[8];
        int cnt = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) m[k] = 0u;
        if (kb < kbt) {
            const uint4* q = reinterpret_cast<const uint4*>(tiles + (t * kbt + kb) * kTileBytes + r * 32);
            const uint4 a = q[0], b = q[1];
            const uint32_t ws[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                m[k] = ws[k] & kLo2 & ~((ws[k] >> 1) & kLo2);
                cnt += __popc(m[k]);
            }
        }
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        uint64_t pos = base + (uint64_t)(incl - cnt);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            uint32_t mm = m[k];
            while (mm) {
                const int bit = __ffs(mm) - 1;
                idx[pos++] = (uint32_t)(kb * 128 + k * 16 + bit / 2);
                mm &= mm - 1;
            }
        }
        base += (uint64_t)__shfl_sync(0xffffffffu, incl, 31);
    }
}

__global__ void k_miss_counts_of(const int32_t* __restrict__ counts, uint64_t p, uint64_t* __restrict__ mc) {
    for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < p; j += (uint64_t)gridDim.x * blockDim.x)
        mc[j] = (uint64_t)counts[j * 4 + 3];
}

void launch_miss_counts_of(Ctx& c, const Geno& g, uint64_t* mc) {
    if (!g.p) return;
    k_miss_counts_of<<<grid_for(c, g.p, 256), 256, 0, c.stream>>>(g.counts.get(), g.p, mc);
    SLFMM_LAUNCHED(c, "k_miss_counts_of");
}

void launch_miss_fill_tiles(Ctx& c, const Geno& g) {
    SLFMM_REQUIRE(g.have_tiles, SLFMM_ERR_BAD_ARG, "this matrix has neither a row-major copy nor SNP-major tiles");
    if (!g.p) return;
    k_miss_fill_tiles<<<(unsigned)ceil_div(g.p * 32, 256), 256, 0, c.stream>>>(g.tiles.get(), g.kbt, g.p,
                                                                               g.miss_ptr.get(), g.miss_idx.get());
    SLFMM_LAUNCHED(c, "k_miss_fill_tiles");
}

static void tile_rows(Ctx& c, const uint8_t* in, uint64_t rows, uint64_t stride, DBuf<uint8_t>& out, uint64_t& kbt,
                      uint64_t& ntiles) {
    SLFMM_REQUIRE(stride % 32 == 0, SLFMM_ERR_BAD_ARG, "packed stride must be a multiple of 32 bytes");
    kbt = stride / 32;
    ntiles = round_up(std::max<uint64_t>(ceil_div(rows, kM), 1), 8);
    const uint64_t bytes = ntiles * kbt * kTileBytes;
    out.alloc(bytes, c.stream);
    const uint64_t chunks = bytes / 16;
    k_tile_rows<<<grid_for(c, chunks, 256), 256, 0, c.stream>>>(in, rows, stride, kbt, chunks, out.get());
    SLFMM_LAUNCHED(c, "k_tile_rows");
}

// Tile-major copies built chunk by chunk while a matrix is uploaded: rows
// [r0, r1) of the SNP-major matrix (r0 a multiple of 128) are tiled and
// transposed as soon as they land.  `last` also writes the padding tiles.
void tile_chunk(Ctx& c, const Geno& g, uint64_t r0, uint64_t r1, bool last) {
    SLFMM_REQUIRE(r0 % kM == 0, SLFMM_ERR_BAD_ARG, "upload chunks must start on a 128-row tile");
    if (r0 == 0) {
        SLFMM_REQUIRE(g.stride % 32 == 0, SLFMM_ERR_BAD_ARG, "packed stride must be a multiple of 32 bytes");
        g.kbt = g.stride / 32;
        g.ntiles = round_up(std::max<uint64_t>(ceil_div(g.p, kM), 1), 8);
        g.tiles.alloc(g.ntiles * g.kbt * kTileBytes, c.stream);
        g.kbtT = round_up(std::max<uint64_t>(ceil_div(g.p, kM), 1), kHalves);
        g.ntilesT = round_up(std::max<uint64_t>(ceil_div(g.n, kM), 1), 8);
        g.tilesT.alloc(g.ntilesT * g.kbtT * kTileBytes, c.stream);
    }
    const uint64_t t0 = r0 / kM, t1 = last ? g.ntiles : ceil_div(r1, kM);
    const uint64_t chunks = (t1 - t0) * g.kbt * (kTileBytes / 16);
    k_tile_rows<<<grid_for(c, chunks, 256), 256, 0, c.stream>>>(packed_rows(g) + r0 * g.stride, r1 - r0, g.stride,
                                                                 g.kbt, chunks,
                                                                 g.tiles.get() + t0 * g.kbt * kTileBytes);
    SLFMM_LAUNCHED(c, "k_tile_rows");
    const uint64_t k1 = last ? g.kbtT : std::min(g.kbtT, ceil_div(r1, kM));
    if (k1 > t0) {
        const uint64_t blocks = std::min<uint64_t>(g.ntilesT * (k1 - t0), (uint64_t)c.sm_count * 16);
        k_transpose_tiles<<<(unsigned)blocks, 256, 0, c.stream>>>(g.tiles.get(), g.kbt, g.ntiles, g.tilesT.get(),
                                                                   g.kbtT, g.ntilesT, t0, k1);
        SLFMM_LAUNCHED(c, "k_transpose_tiles");
    }
    if (last) g.have_tiles = g.have_tilesT = true;
}

void tiles_subset_samples(Ctx& c, const Geno& full, const uint32_t* keep_dev, uint64_t n_keep, Geno& sub) {
    SLFMM_REQUIRE(n_keep > 0 && n_keep <= full.n, SLFMM_ERR_BAD_ARG, "bad sample subset");
    build_tiles(c, full, true);
    sub.n = n_keep;
    sub.p = full.p;
    sub.stride = round_up(ceil_div(n_keep, 4), 128);
    // sample-major: the kept samples' rows of the full matrix's tiles
    sub.kbtT = full.kbtT;
    sub.ntilesT = round_up(std::max<uint64_t>(ceil_div(n_keep, kM), 1), 8);
    sub.tilesT.alloc(sub.ntilesT * sub.kbtT * kTileBytes, c.stream);
    const uint64_t rows16 = sub.ntilesT * sub.kbtT * 256;
    k_gather_tile_rows<<<grid_for(c, rows16, 256), 256, 0, c.stream>>>(full.tilesT.get(), full.kbtT, keep_dev, n_keep,
                                                                       sub.ntilesT, sub.tilesT.get());
    SLFMM_LAUNCHED(c, "k_gather_tile_rows");
    // SNP-major: the 2-bit transpose of those blocks
    sub.kbt = sub.stride / 32;
    sub.ntiles = round_up(std::max<uint64_t>(ceil_div(sub.p, kM), 1), 8);
    sub.tiles.alloc(sub.ntiles * sub.kbt * kTileBytes, c.stream);
    const uint64_t blocks = std::min<uint64_t>(sub.ntiles * sub.kbt, (uint64_t)c.sm_count * 16);
    k_transpose_tiles<<<(unsigned)blocks, 256, 0, c.stream>>>(sub.tilesT.get(), sub.kbtT, sub.ntilesT, sub.tiles.get(),
                                                               sub.kbt, sub.ntiles, 0, sub.kbt);
    SLFMM_LAUNCHED(c, "k_transpose_tiles");
    sub.have_tiles = sub.have_tilesT = true;
    sub.counts.alloc(std::max<uint64_t>(sub.p, 1) * 4, c.stream);
    if (sub.p) {
        k_snp_counts_tiles<<<(unsigned)ceil_div(sub.p * 32, 256), 256, 0, c.stream>>>(sub.tiles.get(), sub.kbt, sub.p,
                                                                                      sub.n, sub.counts.get());
        SLFMM_LAUNCHED(c, "k_snp_counts_tiles");
    }
}

TileView build_tiles(Ctx& c, const Geno& g, bool transposed) {
    if (!transposed) {
        if (!g.have_tiles) {
            tile_rows(c, packed_rows(g), g.p, g.stride, g.tiles, g.kbt, g.ntiles);
            g.have_tiles = true;
        }
        return TileView{g.tiles.get(), g.kbt, g.ntiles};
    }
    if (!g.have_tilesT) {
        // straight from the SNP-row tiles: sample tiles x K blocks of 128 SNPs
        build_tiles(c, g, false);
        g.kbtT = round_up(std::max<uint64_t>(ceil_div(g.p, kM), 1), kHalves);  // whole stages
        g.ntilesT = round_up(std::max<uint64_t>(ceil_div(g.n, kM), 1), 8);
        g.tilesT.alloc(g.ntilesT * g.kbtT * kTileBytes, c.stream);
        const uint64_t blocks = std::min<uint64_t>(g.ntilesT * g.kbtT, (uint64_t)c.sm_count * 16);
        k_transpose_tiles<<<(unsigned)blocks, 256, 0, c.stream>>>(g.tiles.get(), g.kbt, g.ntiles, g.tilesT.get(),
                                                                   g.kbtT, g.ntilesT, 0, g.kbtT);
        SLFMM_LAUNCHED(c, "k_transpose_tiles");
        g.have_tilesT = true;
    }
    return TileView{g.tilesT.get(), g.kbtT, g.ntilesT};
}

void launch_fp8_terms_f64(Ctx& c, const double* src, int ld, uint64_t K, int w, int wpad, uint64_t K_pad,
                          const double* kscale, int terms, int row_off, int n_rows, uint8_t* B, float* inv_scale) {
    DBuf<unsigned> cm(wpad, c.stream);
    cm.zero();
    SLFMM_REQUIRE(w >= 1 && w <= 128 && wpad <= 128, SLFMM_ERR_BAD_ARG, "operand wider than 128 columns");
    SLFMM_REQUIRE(n_rows % 8 == 0 && row_off + terms * wpad <= n_rows && K_pad % kStageK == 0, SLFMM_ERR_BAD_ARG,
                  "bad stage-major operand shape");
    k_colmax_abs<double><<<grid_for(c, K, 8), 256, 0, c.stream>>>(src, ld, K, w, kscale, cm.get());
    SLFMM_LAUNCHED(c, "k_colmax_abs");
    dim3 grid((unsigned)ceil_div(K_pad, 128), (unsigned)ceil_div(wpad, 32));
    k_fp8_terms<double><<<grid, 256, 0, c.stream>>>(src, ld, K, w, wpad, K_pad, kscale, terms, row_off, n_rows,
                                                    cm.get(), B, inv_scale);
    SLFMM_LAUNCHED(c, "k_fp8_terms");
}

void launch_fp8_terms_f32_pair(Ctx& c, const float* src, int ld, uint64_t K, int w, int wpad, uint64_t K_pad,
                               const double* ks_main, const double* ks_ind, int ind_row_off, int n_rows, uint8_t* B,
                               float* inv_scale) {
    SLFMM_REQUIRE(w >= 1 && w <= 128 && wpad <= 128, SLFMM_ERR_BAD_ARG, "operand wider than 128 columns");
    SLFMM_REQUIRE(n_rows % 8 == 0 && kMainTerms * wpad <= n_rows &&
                      (!ks_ind || ind_row_off + kIndTerms * wpad <= n_rows) && K_pad % kStageK == 0,
                  SLFMM_ERR_BAD_ARG, "bad stage-major operand shape");
    DBuf<unsigned> cm(2 * (uint64_t)wpad, c.stream);
    cm.zero();
    unsigned* cma = cm.get();
    unsigned* cmb = ks_ind ? cm.get() + wpad : nullptr;
    const bool quads = ld % 4 == 0 && ld <= 32 && reinterpret_cast<uintptr_t>(src) % 16 == 0;
    if (quads) {
        const unsigned blocks = (unsigned)std::max<uint64_t>(
            1, std::min<uint64_t>(ceil_div(K * (uint64_t)(ld / 4), 1024), (uint64_t)c.sm_count * 4));
        k_colmax_pair<<<blocks, 256, 0, c.stream>>>(src, ld, K, w, ks_main, ks_ind, cma, cmb);
        SLFMM_LAUNCHED(c, "k_colmax_pair");
    } else {
        k_colmax_abs<float><<<grid_for(c, K, 8), 256, 0, c.stream>>>(src, ld, K, w, ks_main, cma);
        SLFMM_LAUNCHED(c, "k_colmax_abs");
        if (ks_ind) {
            k_colmax_abs<float><<<grid_for(c, K, 8), 256, 0, c.stream>>>(src, ld, K, w, ks_ind, cmb);
            SLFMM_LAUNCHED(c, "k_colmax_abs");
        }
    }
    const TermSet sa{ks_main, kMainTerms, 0, cma};
    const TermSet sb{ks_ind, ks_ind ? kIndTerms : 0, ind_row_off, cmb};
    dim3 grid((unsigned)ceil_div(K_pad, 128), (unsigned)ceil_div(wpad, 32));
    k_fp8_terms_pair<<<grid, 256, 0, c.stream>>>(src, ld, K, w, wpad, K_pad, sa, sb, n_rows, B, inv_scale);
    SLFMM_LAUNCHED(c, "k_fp8_terms_pair");
}

void throw_tc8_timeout(int site) {
    throw Error(SLFMM_ERR_DEVICE_TIMEOUT,
                "split-FP8 contraction: a bounded device wait expired (site " + std::to_string(site) + ")");
}

static int tc8_launch(Ctx& c, const Fp8Plan& pl, const TileView& tv, uint64_t rows, uint64_t K, const uint8_t* B,
                      const float* inv_scale, uint64_t K_pad, int mode, const double* row_mean,
                      const double* row_scale, const double* cs, float* out, int ldo, int splits,
                      uint64_t split_stride, int* err_dev);

// Autotuner: the ring depths (packed codes, W stages) of a plan, timed on
// two waves of the real pass and cached per context and shape.  Only knobs
// that leave the arithmetic alone are tuned: the candidates keep the default
// plan's MMA wait group and accumulator layout, so every choice gives the
// same bits.
static Fp8Plan tc8_tuned_plan(Ctx& c, const Fp8Plan& pl, const TileView& tv, uint64_t rows, uint64_t K,
                              const uint8_t* B, const float* inv_scale, uint64_t K_pad, int mode,
                              const double* row_mean, const double* row_scale, const double* cs, int ldo, int splits,
                              uint64_t split_stride) {
    const std::string key = std::to_string(pl.wpad) + "/" + std::to_string(pl.n_ind) + "/" + std::to_string(K) +
                            "/" + std::to_string(splits) + "/" + std::to_string(mode) + "/" +
                            std::to_string(pl.ind_shared);
    auto rebuild = [&](int pmax, int smax) {
        return fp8_plan_knobs((int)pl.wpad, pl.n_ind != 0, ceil_div(rows, (uint64_t)kM), pmax, smax, (int)pl.group,
                              env_int("SLFMM_TC8_WSTAGES", 8), pl.ind_shared != 0);
    };
    auto it = c.tuned.find(key);
    if (it != c.tuned.end()) return rebuild(it->second.first, it->second.second);
    const uint64_t trial_rows = std::min<uint64_t>(rows, (uint64_t)c.sm_count * 2 * kM);
    DBuf<float> scratch(std::max<uint64_t>(trial_rows, 1) * (uint64_t)ldo * std::max(splits, 1), c.stream);
    cudaEvent_t e0, e1;
    SLFMM_CUDA(cudaEventCreate(&e0));
    SLFMM_CUDA(cudaEventCreate(&e1));
    struct EvGuard {
        cudaEvent_t a, b;
        ~EvGuard() { cudaEventDestroy(a); cudaEventDestroy(b); }
    } guard{e0, e1};
    DBuf<int> err(1, c.stream);
    err.zero();
    float best = 1e30f;
    std::pair<int, int> pick{8, 8};
    for (int pmax : {2, 4, 8, 16})
        for (int smax : {2, 3, 4, 8}) {
            const Fp8Plan q = rebuild(pmax, smax);
            if (!q.ok || q.group != pl.group || q.kcopies != pl.kcopies || q.nsplit != pl.nsplit) continue;
            float ms = 1e30f;
            for (int rep = 0; rep < 2; ++rep) {
                SLFMM_CUDA(cudaEventRecord(e0, c.stream));
                tc8_launch(c, q, tv, trial_rows, K, B, inv_scale, K_pad, mode, row_mean, row_scale, cs,
                           scratch.get(), ldo, splits, trial_rows * (uint64_t)ldo, err.get());
                SLFMM_CUDA(cudaEventRecord(e1, c.stream));
                SLFMM_CUDA(cudaEventSynchronize(e1));
                float t = 0.f;
                SLFMM_CUDA(cudaEventElapsedTime(&t, e0, e1));
                ms = std::min(ms, t);
            }
            if (ms < best) {
                best = ms;
                pick = {pmax, smax};
            }
        }
    int h = 0;
    SLFMM_CUDA(cudaMemcpyAsync(&h, err.get(), sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    SLFMM_CUDA(cudaStreamSynchronize(c.stream));
    if (h != 0) throw_tc8_timeout(h);
    c.tuned[key] = pick;
    if (c.verbose)
        fprintf(stderr, "[schnelgpu] autotune %s: packed ring cap %d, W ring cap %d (%.3f ms on %llu rows)\n",
                key.c_str(), pick.first, pick.second, best, (unsigned long long)trial_rows);
    return rebuild(pick.first, pick.second);
}

int launch_tc8_rows(Ctx& c, const Fp8Plan& pl, const TileView& tv, uint64_t rows, uint64_t K,
                    const uint8_t* B, const float* inv_scale, uint64_t K_pad, int mode, const double* row_mean,
                    const double* row_scale, const double* cs, float* out, int ldo, int splits,
                    uint64_t split_stride, int* err_dev) {
    if (c.autotune && pl.ok && rows > 0) {
        const Fp8Plan tp = tc8_tuned_plan(c, pl, tv, rows, K, B, inv_scale, K_pad, mode, row_mean, row_scale, cs, ldo,
                                          splits, split_stride);
        if (tp.ok) return tc8_launch(c, tp, tv, rows, K, B, inv_scale, K_pad, mode, row_mean, row_scale, cs, out, ldo,
                                     splits, split_stride, err_dev);
    }
    return tc8_launch(c, pl, tv, rows, K, B, inv_scale, K_pad, mode, row_mean, row_scale, cs, out, ldo, splits,
                      split_stride, err_dev);
}

static int tc8_launch(Ctx& c, const Fp8Plan& pl, const TileView& tv, uint64_t rows, uint64_t K, const uint8_t* B,
                      const float* inv_scale, uint64_t K_pad, int mode, const double* row_mean,
                      const double* row_scale, const double* cs, float* out, int ldo, int splits,
                      uint64_t split_stride, int* err_dev) {
    SLFMM_REQUIRE(pl.ok, SLFMM_ERR_BAD_ARG, "no feasible split-FP8 tile plan for this width");
    SLFMM_REQUIRE(K_pad % kStageK == 0 && K_pad >= ceil_div(K, kStageK) * kStageK, SLFMM_ERR_BAD_ARG,
                  "bad K padding");
    SLFMM_REQUIRE(tv.base && tv.kbt % kHalves == 0 && tv.kbt >= ceil_div(K, kStageK) * kHalves, SLFMM_ERR_BAD_ARG,
                  "tile-major operand too short in K");
    SLFMM_REQUIRE(tv.ntiles >= ceil_div(rows, kM), SLFMM_ERR_BAD_ARG,
                  "tile-major operand has too few tiles");
    SLFMM_REQUIRE(mode == 0 || pl.n_ind != 0, SLFMM_ERR_BAD_ARG, "row correction needs the indicator operand");
    SLFMM_REQUIRE(reinterpret_cast<uintptr_t>(B) % 16 == 0 && pl.b_stage_bytes % 16 == 0, SLFMM_ERR_BAD_ARG,
                  "W operand not 16-byte aligned");
    raise_dynamic_smem((const void*)k_tc8_rows, pl.smem);
    DBuf<int> err;
    if (!err_dev) {
        err.alloc(1, c.stream);
        err.zero();
    }
    Tc8Args a{};
    a.rows = (uint32_t)rows;
    a.kb_total = (uint32_t)ceil_div(K, kStageK);
    a.kb_per_split = (uint32_t)ceil_div(a.kb_total, (uint64_t)std::max(splits, 1));
    a.wpad = pl.wpad;
    a.n_main = pl.n_main;
    a.n_ind = pl.n_ind;
    a.n_total = pl.n_total;
    a.ind_shared = pl.ind_shared;
    a.d_cols = pl.d_cols;
    a.a_cols = pl.a_cols;
    a.stages = pl.stages;
    a.wstages = pl.wstages;
    a.pstages = pl.pstages;
    a.group = pl.group;
    a.kcopies = pl.kcopies;
    a.nsplit = pl.nsplit;
    a.a_base = pl.a_base;
    a.usets = std::min<uint32_t>(kUnpackSets, std::min(pl.stages, pl.pstages));
    a.tmem_cols = pl.tmem_cols;
    a.b_stage_bytes = pl.b_stage_bytes;
    a.inv_scale = inv_scale;
    a.wop = B;
    a.expire_cycles = c.expire_next_wait;
    a.tile0 = (uint32_t)tv.tile0;
    a.rotate = (uint32_t)env_int("SLFMM_TC8_ROTATE", 1);  // tuning override
    c.expire_next_wait = 0;
    a.mode = mode;
    a.row_mean = row_mean;
    a.row_scale = row_scale;
    a.cs = cs;
    a.out = out;
    a.ldo = (uint32_t)ldo;
    a.split_stride = split_stride;
    a.tiles = tv.base;
    a.tile_bytes = tv.kbt * (uint64_t)kTileBytes;
    a.err = err_dev ? err_dev : err.get();
    const unsigned gy = (unsigned)ceil_div(a.kb_total, a.kb_per_split);
    const unsigned gx = (unsigned)ceil_div(rows, kM);
    a.gx = gx;
    a.units = gx * gy;
    // one CTA per SM working through the units (SLFMM_TC8_PERSIST=0: one CTA
    // per unit; the same code and bits either way)
    const unsigned ctas = env_int("SLFMM_TC8_PERSIST", 1) != 0
                              ? std::min<unsigned>(a.units, (unsigned)std::max(c.sm_count, 1))
                              : a.units;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(std::max(ctas, 1u), 1, 1);
    cfg.blockDim = dim3(kThreads, 1, 1);
    cfg.dynamicSmemBytes = pl.smem;
    cfg.stream = c.stream;
    const cudaError_t le = cudaLaunchKernelEx(&cfg, k_tc8_rows, a);
    if (le != cudaSuccess) {
        cudaGetLastError();
        char buf[320];
        snprintf(buf, sizeof buf,
                 "split-FP8 contraction launch failed (%s): units %u x %u, smem %zu, stages %u/%u, pstages %u, "
                 "group %u, n_total %u, rows %llu, K %llu",
                 cudaGetErrorString(le), gx, gy, pl.smem, pl.stages, pl.wstages, pl.pstages, pl.group, pl.n_total,
                 (unsigned long long)rows, (unsigned long long)K);
        throw Error(SLFMM_ERR_CUDA, buf);
    }
    SLFMM_LAUNCHED(c, "k_tc8_rows");
    if (err_dev) return (int)gy;
    int h = 0;
    SLFMM_CUDA(cudaMemcpyAsync(&h, err.get(), sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    SLFMM_CUDA(cudaStreamSynchronize(c.stream));
    if (h != 0) throw_tc8_timeout(h);
    return (int)gy;
}

void launch_sub_colterm(Ctx& c, double* S, int lds, uint64_t n, int w, const double* colterm) {
    if (!n || !w) return;
    k_sub_colterm<<<grid_for(c, n * w, 256), 256, 0, c.stream>>>(S, lds, n, w, colterm);
    SLFMM_LAUNCHED(c, "k_sub_colterm");
}

}  // namespace slfmm
