// C ABI and host orchestration of the GB300 streaming LFMM2 engine.
//
// Mirrors the library surface of schnelLFMM (src/lib.rs:102-263) and the
// stage functions estimate_factors_streaming (src/rsvd.rs:26-177) and
// test_associations_fused (src/testing.rs:252-528).  The reference streams
// the memory-mapped .bed through a thread pool for every pass; here the
// packed matrix is uploaded once (pinned staging ring, double-buffered) and
// every pass is a kernel over the resident copy.
#include <algorithm>
#include <mutex>
#include <chrono>
#include <atomic>
#include <cmath>
#include <cstring>
#include <fstream>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "slfmm_internal.h"

struct slfmm_ctx : slfmm::Ctx {};
struct slfmm_geno : slfmm::Geno {};

namespace slfmm {

void profile_collect(Ctx& c) {
    for (auto& kv : c.prof) {
        for (auto& ev : kv.second.pending) {
            float ms = 0.f;
            if (cudaEventSynchronize(ev.second) == cudaSuccess && cudaEventElapsedTime(&ms, ev.first, ev.second) == cudaSuccess)
                kv.second.ms += ms;
            cudaEventDestroy(ev.first);
            cudaEventDestroy(ev.second);
        }
        kv.second.pending.clear();
    }
}

void raise_dynamic_smem(const void* fn, size_t bytes) {
    if (bytes <= 48 * 1024) return;
    static std::mutex mu;
    static std::map<std::pair<int, const void*>, size_t> raised;
    int dev = 0;
    SLFMM_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    size_t& cur = raised[{dev, fn}];
    if (bytes <= cur) return;
    SLFMM_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    cur = bytes;
}

void after_launch(Ctx& c, const char* name) {
    ++c.launches;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        throw Error(SLFMM_ERR_CUDA, std::string("launch of ") + name + " failed: " + cudaGetErrorString(e));
}

namespace {

// ---------------------------------------------------------------------------
// small host <-> device helpers
// ---------------------------------------------------------------------------
template <typename T>
void h2d(Ctx& c, T* dst, const T* src, size_t count) {
    if (count) SLFMM_CUDA(cudaMemcpyAsync(dst, src, count * sizeof(T), cudaMemcpyHostToDevice, c.stream));
}
template <typename T>
void d2h(Ctx& c, T* dst, const T* src, size_t count) {
    if (count) SLFMM_CUDA(cudaMemcpyAsync(dst, src, count * sizeof(T), cudaMemcpyDeviceToHost, c.stream));
}
void sync(Ctx& c) { SLFMM_CUDA(cudaStreamSynchronize(c.stream)); }

template <typename T>
std::vector<T> fetch(Ctx& c, const T* src, size_t count) {
    std::vector<T> v(count);
    d2h(c, v.data(), src, count);
    sync(c);
    return v;
}
template <typename T>
DBuf<T> upload(Ctx& c, const T* src, size_t count) {
    DBuf<T> b(count, c.stream);
    h2d(c, b.get(), src, count);
    return b;
}

void log(Ctx& c, const std::string& s) {
    if (c.verbose) fprintf(stderr, "[schnelgpu] %s\n", s.c_str());
}

// Rust "{:.Ne}" of a finite double: C's %.*e without the exponent's sign
// and zero padding (1.00e-8, not 1.00e-08).
std::string rust_exp(double v, int prec) {
    char tmp[64];
    snprintf(tmp, sizeof tmp, "%.*e", prec, v);
    char* e = std::strchr(tmp, 'e');
    if (!e) return tmp;
    *e = '\0';
    return std::string(tmp) + "e" + std::to_string(std::atoi(e + 1));
}

// The outcome of a safe_inv-style inversion (k_inverse status: 0 inverted,
// 1 inverted after adding eps to the diagonal, 2 failed even then), reported
// with the reference's stderr warning and error texts (src/testing.rs:996-1024).
void safe_inv_report(int status, double eps, const char* name) {
    if (status == 2)
        throw Error(SLFMM_ERR_SINGULAR,
                    std::string(name) + " inversion failed even with epsilon=" + rust_exp(eps, 2) + " regularization");
    if (status == 1)
        fprintf(stderr, "Warning: %s is singular, adding epsilon=%s diagonal regularization\n", name,
                rust_exp(eps, 2).c_str());
}

double host_now_ms() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

void clear_phase_marks(Ctx& c) {
    for (auto& m : c.phase_marks) cudaEventDestroy(m.ev);
    c.phase_marks.clear();
}

// Phase marks of a fit.  With profiling on, each mark records an event on
// the stream and the host clock (no synchronisation; slfmm_phase_read gives
// both per phase).  Verbose mode logs the wall time of each phase, with the
// stream synchronised at every mark so that a phase's time covers its
// device work.
void phase(Ctx& c, const char* what, bool start = false) {
    if (c.profiling) {
        if (start) clear_phase_marks(c);
        cudaEvent_t e = nullptr;
        if (cudaEventCreate(&e) == cudaSuccess) {
            if (cudaEventRecord(e, c.stream) == cudaSuccess)
                c.phase_marks.push_back({start ? std::string() : std::string(what), e, host_now_ms()});
            else
                cudaEventDestroy(e);
        }
    }
    if (!c.verbose) return;
    sync(c);
    const double t = host_now_ms();
    if (!start) {
        char buf[160];
        snprintf(buf, sizeof buf, "%-36s %9.2f ms", what, t - c.phase_t0);
        log(c, buf);
    }
    c.phase_t0 = t;
}

// ---------------------------------------------------------------------------
// SNP subset expansion (src/parallel.rs:113-122, src/bed.rs:162-171)
// ---------------------------------------------------------------------------
std::vector<uint64_t> subset_indices(const slfmm_subset* s, uint64_t n_snps) {
    std::vector<uint64_t> idx;
    if (s == nullptr || s->kind == SLFMM_SUBSET_ALL) {
        idx.resize(n_snps);
        for (uint64_t i = 0; i < n_snps; ++i) idx[i] = i;
    } else if (s->kind == SLFMM_SUBSET_RATE) {
        SLFMM_REQUIRE(s->rate > 0.0 && s->rate <= 1.0, SLFMM_ERR_BAD_ARG,
                      "--est-rate must be in (0.0, 1.0], got " + std::to_string(s->rate));
        const uint64_t step = (uint64_t)std::ceil(1.0 / s->rate);
        for (uint64_t i = 0; i < n_snps; i += step) idx.push_back(i);
    } else if (s->kind == SLFMM_SUBSET_INDICES) {
        SLFMM_REQUIRE(s->indices != nullptr || s->n_indices == 0, SLFMM_ERR_BAD_ARG, "null index list");
        idx.assign(s->indices, s->indices + s->n_indices);
        for (uint64_t v : idx)
            SLFMM_REQUIRE(v < n_snps, SLFMM_ERR_BAD_ARG, "SNP index out of range: " + std::to_string(v));
    } else {
        throw Error(SLFMM_ERR_BAD_ARG, "unknown subset kind");
    }
    return idx;
}

bool is_pinned(const void* p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// ---------------------------------------------------------------------------
// ingest: host payload -> resident packed matrix
// ---------------------------------------------------------------------------
// Work run on each chunk of rows [r0, r1) right after it lands (tiles,
// counts and missing-call offsets of the chunk are ready).
struct ChunkHook {
    // device setup, run once while the first chunks are being copied
    virtual void begin(Ctx& c) {}
    virtual void rows(Ctx& c, const Geno& g, uint64_t r0, uint64_t r1) = 0;
    virtual ~ChunkHook() = default;
};

// snps: the payload rows to take, in order (nullptr: all n_snps rows)
void upload_geno(Ctx& c, Geno& g, const uint8_t* packed, uint64_t n_phys, uint64_t n_snps,
                 const uint64_t* keep, uint64_t n_keep, const std::vector<uint64_t>* snps,
                 ChunkHook* hook = nullptr) {
    SLFMM_REQUIRE(packed != nullptr || n_snps == 0, SLFMM_ERR_BAD_ARG, "null genotype payload");
    SLFMM_REQUIRE(n_phys > 0, SLFMM_ERR_BAD_ARG, "no samples");
    const uint64_t bps = ceil_div(n_phys, 4);
    g.n = keep ? n_keep : n_phys;
    g.p = snps ? snps->size() : n_snps;
    auto row_of = [snps](uint64_t r) { return snps ? (*snps)[r] : r; };
    SLFMM_REQUIRE(g.n > 0, SLFMM_ERR_BAD_ARG, "empty sample subset");
    SLFMM_REQUIRE(g.n < (1ull << 31), SLFMM_ERR_BAD_ARG, "too many samples");
    g.stride = round_up(ceil_div(g.n, 4), 128);
    g.packed.alloc(std::max<uint64_t>(g.p, 1) * g.stride, c.stream);
    g.counts.alloc(std::max<uint64_t>(g.p, 1) * 4, c.stream);
    DBuf<uint32_t> keep_d;
    if (keep) {
        std::vector<uint32_t> k32(n_keep);
        for (uint64_t i = 0; i < n_keep; ++i) {
            SLFMM_REQUIRE(keep[i] < n_phys, SLFMM_ERR_BAD_ARG, "sample index out of range");
            k32[i] = (uint32_t)keep[i];
        }
        keep_d = upload(c, k32.data(), n_keep);
        sync(c);
    }
    if (g.p) {
        // staging: ~96 MiB (at most 256 Ki rows) per chunk, two device
        // buffers, two pinned buffers.  Split-FP8 contexts build the
        // tile-major copies chunk by chunk as the rows land (chunks then start
        // on 128-row tiles, whole waves of one tile per SM where the chunk
        // holds one); every context builds the per-SNP missing-call lists the
        // same way.  The copies are bound by the host link, so this work
        // hides behind them.
        const bool tiles = c.precision == SLFMM_PREC_SPLIT_FP8;
        uint64_t rows_per = std::max<uint64_t>(1, std::min<uint64_t>({g.p, (96ull << 20) / bps, 1ull << 18}));
        if (tiles) {
            const uint64_t wave = 128ull * (uint64_t)std::max(c.sm_count, 1);
            rows_per = rows_per >= wave ? rows_per / wave * wave : std::max<uint64_t>(128, rows_per / 128 * 128);
        }
        g.miss_ptr.alloc(g.p + 1, c.stream);
        SLFMM_CUDA(cudaMemsetAsync(g.miss_ptr.get(), 0, sizeof(uint64_t), c.stream));
        uint64_t cap = 0;  // index capacity, sized from the first chunk's density
        uint64_t first_end = 0;
        const bool direct = is_pinned(packed);
        const uint64_t nchunks = ceil_div(g.p, rows_per);
        // staging depth: two buffers (measured on GB300: deeper staging of a
        // page-locked payload neither shortens the upload nor hides the hook's
        // setup better); a pageable payload goes through two pinned buffers
        const char* ns_env = std::getenv("SLFMM_UPLOAD_STAGES");  // tuning override
        const uint64_t ns_direct = ns_env && *ns_env ? (uint64_t)std::max(2, std::atoi(ns_env)) : 2;
        const int NS = (int)std::max<uint64_t>(1, std::min<uint64_t>(direct ? ns_direct : 2, nchunks));
        std::vector<DBuf<uint8_t>> dstage(NS);
        for (auto& d : dstage) d.alloc(rows_per * bps, c.stream);
        std::vector<uint8_t*> hstage(NS, nullptr);
        std::vector<cudaEvent_t> copied(NS, nullptr), consumed(NS, nullptr);
        struct Cleanup {
            std::vector<uint8_t*>& h;
            std::vector<cudaEvent_t>& a;
            std::vector<cudaEvent_t>& b;
            ~Cleanup() {
                for (size_t i = 0; i < h.size(); ++i) {
                    if (h[i]) cudaFreeHost(h[i]);
                    if (a[i]) cudaEventDestroy(a[i]);
                    if (b[i]) cudaEventDestroy(b[i]);
                }
            }
        } cleanup{hstage, copied, consumed};
        for (int b = 0; b < NS; ++b) {
            SLFMM_CUDA(cudaEventCreateWithFlags(&copied[b], cudaEventDisableTiming));
            SLFMM_CUDA(cudaEventCreateWithFlags(&consumed[b], cudaEventDisableTiming));
            SLFMM_CUDA(cudaEventRecord(consumed[b], c.stream));
        }
        if (!direct)
            for (int b = 0; b < NS; ++b) SLFMM_CUDA(cudaMallocHost(&hstage[b], rows_per * bps));
        SLFMM_CUDA(cudaStreamSynchronize(c.stream));
        // copy chunk ch into staging buffer ch % NS once the repack that last
        // used the buffer is done
        auto issue = [&](uint64_t ch) {
            const int b = (int)(ch % NS);
            const uint64_t r0 = ch * rows_per, r1 = std::min(g.p, r0 + rows_per), rows = r1 - r0;
            bool contiguous = true;  // one copy when the rows are consecutive (src/parallel.rs:129-146)
            if (snps)
                for (uint64_t r = r0 + 1; r < r1 && contiguous; ++r) contiguous = (*snps)[r] == (*snps)[r - 1] + 1;
            SLFMM_CUDA(cudaStreamWaitEvent(c.copy_stream, consumed[b], 0));
            if (direct && contiguous) {
                SLFMM_CUDA(cudaMemcpyAsync(dstage[b].get(), packed + row_of(r0) * bps, rows * bps,
                                           cudaMemcpyHostToDevice, c.copy_stream));
            } else if (direct) {
                for (uint64_t r = r0; r < r1; ++r)
                    SLFMM_CUDA(cudaMemcpyAsync(dstage[b].get() + (r - r0) * bps, packed + row_of(r) * bps, bps,
                                               cudaMemcpyHostToDevice, c.copy_stream));
            } else {
                // the pinned buffer b is reused only after its previous H2D finished
                SLFMM_CUDA(cudaEventSynchronize(copied[b]));
                if (contiguous) {
                    std::memcpy(hstage[b], packed + row_of(r0) * bps, rows * bps);
                } else {
                    for (uint64_t r = r0; r < r1; ++r)
                        std::memcpy(hstage[b] + (r - r0) * bps, packed + row_of(r) * bps, bps);
                }
                SLFMM_CUDA(cudaMemcpyAsync(dstage[b].get(), hstage[b], rows * bps, cudaMemcpyHostToDevice,
                                           c.copy_stream));
            }
            SLFMM_CUDA(cudaEventRecord(copied[b], c.copy_stream));
        };
        for (uint64_t ch = 0; ch + 1 < (uint64_t)NS; ++ch) issue(ch);
        if (hook) hook->begin(c);
        for (uint64_t ch = 0; ch < nchunks; ++ch) {
            if (ch + NS - 1 < nchunks) issue(ch + NS - 1);
            const int b = (int)(ch % NS);
            const uint64_t r0 = ch * rows_per, r1 = std::min(g.p, r0 + rows_per), rows = r1 - r0;
            if (ch == 1) {
                // the first chunk's list length sizes the index array (later
                // chunks' copies are already in flight); 1.5x its density
                // plus slack, and a chunk that overruns it leaves the lists
                // to be rebuilt after the upload
                const uint64_t nnz0 = fetch(c, g.miss_ptr.get() + first_end, 1)[0];
                const double est = (double)nnz0 * (double)g.p / (double)first_end;
                cap = (uint64_t)(1.5 * est) + g.p + 4096;
                g.miss_idx.alloc(cap, c.stream);
                csr_chunk_fill(c, g, 0, first_end, cap);
            }
            SLFMM_CUDA(cudaStreamWaitEvent(c.stream, copied[b], 0));
            launch_repack(c, dstage[b].get(), rows, bps, n_phys, keep_d.get(), g.n,
                          g.packed.get() + r0 * g.stride, g.stride);
            SLFMM_CUDA(cudaEventRecord(consumed[b], c.stream));
            launch_snp_counts_range(c, g, r0, rows);
            if (tiles) tile_chunk(c, g, r0, r1, ch + 1 == nchunks);
            csr_chunk_offsets(c, g, r0, rows);
            if (ch == 0) first_end = r1;
            else csr_chunk_fill(c, g, r0, rows, cap);
            if (hook) hook->rows(c, g, r0, r1);
        }
        const uint64_t nnz = fetch(c, g.miss_ptr.get() + g.p, 1)[0];
        if (nchunks == 1) {
            cap = std::max<uint64_t>(nnz, 1);
            g.miss_idx.alloc(cap, c.stream);
            csr_chunk_fill(c, g, 0, g.p, cap);
        }
        if (nnz <= cap) {
            g.nnz = nnz;
            g.have_csr = true;
        } else {
            g.miss_idx.release();  // rebuilt on first use
        }
        SLFMM_CUDA(cudaStreamSynchronize(c.stream));
        SLFMM_CUDA(cudaStreamSynchronize(c.copy_stream));
    }
    sync(c);
}

// ---------------------------------------------------------------------------
// per-SNP standardisation state of one genotype matrix
// ---------------------------------------------------------------------------
// NMF values at the missing calls: f_ir = W_i . H_r (W n x k, H one row of k
// per SNP, FP32); k = 0 means mean imputation
struct NmfFill {
    int k = 0;
    const float* W = nullptr;
    const float* H = nullptr;
};

struct SnpStd {
    DBuf<double> mean, scale, tss;
    DBuf<uint8_t> zero_var;
    DBuf<float> lut;  // p x 4
    NmfFill fill;
};

void std_mean(Ctx& c, const Geno& g, int norm, SnpStd& s) {
    const uint64_t p = std::max<uint64_t>(g.p, 1);
    s.mean.alloc(p, c.stream);
    s.scale.alloc(p, c.stream);
    s.tss.alloc(p, c.stream);
    s.zero_var.alloc(p, c.stream);
    s.lut.alloc(p * 4, c.stream);
    launch_stats_mean(c, g, norm, s.mean.get(), s.scale.get(), s.tss.get(), s.zero_var.get());
    launch_lut_std(c, g.p, s.mean.get(), s.scale.get(), s.lut.get());
}

// ---------------------------------------------------------------------------
// contractions over the resident genotypes
// ---------------------------------------------------------------------------
int pad16(int w) { return (int)round_up((uint64_t)w, 16); }

// Split-FP8 operand of a SNP-row pass with the missing-call indicator: 4 + 3
// scaled E4M3 terms of W (n x w FP64) and its column sums.  The epilogue then
// applies out = s_j (P - mu_j (cs - M)) in the same kernel.  ok is false when
// the width leaves no indicator plan (too wide for TMEM) or it is switched off.
struct Fp8RowOperand {
    bool ok = false;
    Fp8Plan pl{};
    int wp = 0;
    uint64_t n_pad = 0;
    DBuf<uint8_t> B;
    DBuf<float> isc;
    DBuf<double> cs;
};

// whether a width-w row pass has the indicator plan (SLFMM_TC8_ROW_IND=0 turns
// it off)
bool fp8_row_indicator_plan(int w, uint64_t tiles) {
    const int wp = pad16(w);
    const char* ind_env = std::getenv("SLFMM_TC8_ROW_IND");
    if (wp > kMaxW || (ind_env && ind_env[0] == '0')) return false;
    const Fp8Plan pl = fp8_plan(wp, true, tiles, true);
    return pl.ok && pl.n_ind != 0;
}

bool fp8_row_operand(Ctx& c, uint64_t n, uint64_t tiles, const double* W, int w, int ldw, Fp8RowOperand& op) {
    op.wp = pad16(w);
    op.n_pad = round_up(n, 256);  // whole split-FP8 stages (256 codes)
    if (!fp8_row_indicator_plan(w, tiles)) return false;
    // genotype and indicator MMAs multiply the same W: the indicator's three
    // terms are the leading three of the main four (ind_shared plan)
    op.pl = fp8_plan(op.wp, true, tiles, true);
    op.cs.alloc(op.wp, c.stream);
    op.cs.zero();
    launch_colsums(c, W, n, w, ldw, op.cs.get());
    op.B.alloc((uint64_t)op.pl.n_total * op.n_pad, c.stream);
    op.isc.alloc(op.pl.n_total, c.stream);
    const int nr = (int)op.pl.n_total;
    launch_fp8_terms_f64(c, W, ldw, n, w, op.wp, op.n_pad, nullptr, 4, 0, nr, op.B.get(), op.isc.get());
    if (!op.pl.ind_shared)
        launch_fp8_terms_f64(c, W, ldw, n, w, op.wp, op.n_pad, nullptr, 3, (int)op.pl.n_main, nr, op.B.get(),
                             op.isc.get());
    op.ok = true;
    return true;
}

// out rows [r0, r0 + rows) of a row pass with an indicator operand; err_dev
// non-null defers the bounded-wait check to the caller
void fp8_row_launch(Ctx& c, const Geno& g, const SnpStd& s, const Fp8RowOperand& op, uint64_t r0, uint64_t rows,
                    float* out, int* err_dev) {
    const uint64_t t0 = r0 / 128;
    const TileView tv{g.tiles.get() + t0 * g.kbt * 4096, g.kbt, g.ntiles - t0, t0};
    launch_tc8_rows(c, op.pl, tv, rows, g.n, op.B.get(), op.isc.get(), op.n_pad, 1, s.mean.get() + r0,
                    s.scale.get() + r0, op.cs.get(), out + r0 * op.wp, op.wp, 1, 0, err_dev);
}

// A split-FP8 SNP-row pass prepared once and run over row ranges (r0 a
// multiple of 128): either the indicator form, or column blocks without the
// indicator followed by the per-SNP fix over the missing-call lists
// (operands too wide for TMEM).  The association pass runs it chunk by chunk
// so that finished rows can be copied out while later ones compute.
struct Fp8RowPass {
    int w = 0, wp = 0;
    uint64_t n_pad = 0;
    Fp8RowOperand op;  // indicator form when op.ok
    std::vector<Fp8Plan> plans;
    std::vector<DBuf<uint8_t>> Bs;
    std::vector<DBuf<float>> iscs;
    std::vector<int> c0s;
    DBuf<float> W32;  // the fix's W rows (FP32)
    DBuf<double> cs;
};

// Whether a row pass over g takes the missing-call indicator operand rather
// than the sparse per-SNP fix over the missing-call lists.  The indicator adds
// three E4M3 terms of tensor work and 96 + 64 TMEM columns that shorten the
// operand ring; the fix gathers one W row per missing call from L2, so its
// cost grows with the missing calls.  Measured on GB300 (n = 20 000, w = 30,
// 0.5 % missing): 4.18 ms for the ring without the indicator plus 3.43 ms for
// the fix, against 8.2 ms with the indicator (which also measured 15 ms on
// some boxes, where the other forms did not change); at 7 % missing (n =
// 5 000) the fix costs more than the indicator, and below a few thousand
// samples (a few stages per tile, n = 100-3 000 measured) the indicator ring
// is not the limiter while the fix is one more launch per pass.  So the fix
// is taken for n >= 8192 samples when at most 1 % of the calls are missing,
// and for the sketch pass of the randomized SVD (`sketch`) whenever
// n >= 8192: that pass also runs chunk by chunk under an upload, before the
// missing-call count is known, and both must take the same form.
// SLFMM_TC8_ROW_IND=1 / =0 force the indicator on / off.
constexpr uint64_t kSparseFixMinSamples = 8192;

bool fp8_row_indicator_forced() {
    const char* env = std::getenv("SLFMM_TC8_ROW_IND");
    return env && env[0] == '1';
}

// the form of a sketch pass over n samples, known before any data lands
bool fp8_sketch_takes_indicator(uint64_t n) {
    const char* env = std::getenv("SLFMM_TC8_ROW_IND");
    if (env && env[0] == '0') return false;
    return fp8_row_indicator_forced() || n < kSparseFixMinSamples;
}

bool fp8_row_take_indicator(Ctx& c, const Geno& g, bool sketch) {
    if (sketch) return fp8_sketch_takes_indicator(g.n);
    if (fp8_row_indicator_forced()) return true;
    if (g.n < kSparseFixMinSamples) {
        const char* env = std::getenv("SLFMM_TC8_ROW_IND");
        return !(env && env[0] == '0');
    }
    const char* env = std::getenv("SLFMM_TC8_ROW_IND");
    if (env && env[0] == '0') return false;
    build_missing_lists(c, g);
    const double cells = (double)g.n * (double)g.p;
    return cells > 0 && (double)g.nnz > 0.01 * cells;
}

// The operand of a row pass over n samples and `tiles` row tiles: the
// indicator form when `indicator` and it has a plan, else column blocks
// without it (needs nothing of the matrix itself).
void fp8_row_operand_prepare(Ctx& c, uint64_t n, uint64_t tiles, const double* W, int w, int ldw, bool indicator,
                             Fp8RowPass& rp) {
    rp.w = w;
    rp.wp = pad16(w);
    rp.n_pad = round_up(n, 256);  // whole split-FP8 stages (256 codes)
    if (indicator && fp8_row_operand(c, n, tiles, W, w, ldw, rp.op)) return;
    rp.W32.alloc(rp.n_pad * rp.wp, c.stream);
    launch_f64_to_f32_pad(c, W, n, w, ldw, rp.W32.get(), rp.n_pad, rp.wp);
    const Fp8Plan pl = fp8_plan(rp.wp, false, tiles);
    const int cb = pl.ok ? rp.wp : 64;
    rp.cs.alloc(rp.wp, c.stream);
    rp.cs.zero();
    launch_colsums(c, W, n, w, ldw, rp.cs.get());
    for (int c0 = 0; c0 < w; c0 += cb) {
        // the epilogue writes pb.wpad columns: the last block is padded only to 16
        const int wb = std::min(cb, w - c0), bp = std::min(cb, pad16(wb));
        const Fp8Plan pb = bp == rp.wp ? pl : fp8_plan(bp, false, tiles);
        DBuf<uint8_t> B((uint64_t)pb.n_total * rp.n_pad, c.stream);
        DBuf<float> isc(pb.n_total, c.stream);
        launch_fp8_terms_f64(c, W + c0, ldw, n, wb, bp, rp.n_pad, nullptr, 4, 0, (int)pb.n_total, B.get(),
                             isc.get());
        rp.plans.push_back(pb);
        rp.Bs.push_back(std::move(B));
        rp.iscs.push_back(std::move(isc));
        rp.c0s.push_back(c0);
    }
}

void fp8_row_prepare(Ctx& c, const Geno& g, const double* W, int w, int ldw, Fp8RowPass& rp, bool sketch = false) {
    build_tiles(c, g, false);
    const bool ind = fp8_row_take_indicator(c, g, sketch);
    fp8_row_operand_prepare(c, g.n, ceil_div(g.p, 128), W, w, ldw, ind, rp);
    if (!rp.op.ok) build_missing_lists(c, g);
}

// the per-SNP missing-call fix of rows [r0, r0 + rows) of a pass without
// the indicator: out = s_j (P - mu_j (cs - sum over the SNP's missing calls of W))
void fp8_row_fix(Ctx& c, const Geno& g, const SnpStd& s, const Fp8RowPass& rp, uint64_t r0, uint64_t rows,
                 float* out) {
    if (rp.op.ok) return;
    build_missing_lists(c, g);
    // algorithmic bytes: the lists' indices and one W row per missing call
    const uint64_t nnz_rows = rows == g.p ? g.nnz : (uint64_t)((double)g.nnz * rows / std::max<uint64_t>(g.p, 1));
    ProfScope ps(c, "row_fix", (double)nnz_rows * (4.0 + 4.0 * rp.w) + (double)rows * rp.w * 8, 1.0 * nnz_rows * rp.w);
    launch_rowfix_mean(c, out + r0 * rp.wp, rp.wp, rows, rp.w, g.miss_ptr.get() + r0, g.miss_idx.get(),
                       rp.W32.get(), rp.wp, g.n, rp.cs.get(), s.mean.get() + r0, s.scale.get() + r0);
}

// rows [r0, r0 + rows) of out (ld wp); err_dev as in launch_tc8_rows.  The
// tensor-core launches are profiled as "row_contract" (algorithmic bytes:
// the rows' packed codes, their outputs and the operand).  Without the
// indicator, `fix` false leaves the raw products P in out and the per-SNP fix
// to fp8_row_fix (an upload that has not finished its missing-call lists).
void fp8_row_run(Ctx& c, const Geno& g, const SnpStd& s, const Fp8RowPass& rp, uint64_t r0, uint64_t rows,
                 float* out, int* err_dev, bool fix = true) {
    const double bytes = (double)rows * ceil_div(g.n, 4) + (double)rows * rp.w * 4 + (double)g.n * rp.w * 4;
    const double flops = 2.0 * g.n * rows * rp.w;
    if (rp.op.ok) {
        ProfScope ps(c, "row_contract", bytes, flops);
        fp8_row_launch(c, g, s, rp.op, r0, rows, out, err_dev);
        return;
    }
    const uint64_t t0 = r0 / 128;
    const TileView tv{g.tiles.get() + t0 * g.kbt * 4096, g.kbt, g.ntiles - t0, t0};
    for (size_t b = 0; b < rp.plans.size(); ++b) {
        const double share = (double)rp.plans[b].wpad / rp.wp;
        ProfScope ps(c, "row_contract", bytes * share, flops * share);
        launch_tc8_rows(c, rp.plans[b], tv, rows, g.n, rp.Bs[b].get(), rp.iscs[b].get(), rp.n_pad, 0,
                        s.mean.get() + r0, s.scale.get() + r0, rp.cs.get(), out + r0 * rp.wp + rp.c0s[b], rp.wp, 1,
                        0, err_dev);
    }
    if (fix) fp8_row_fix(c, g, s, rp, r0, rows, out);
}

// out (p x wp, FP32) = Y_hat^T W, W = n x w FP64 (leading dim ldw)
void row_contract_base(Ctx& c, const Geno& g, const SnpStd& s, const double* W, int w, int ldw,
                       DBuf<float>& out, int& wp, bool sketch = false) {
    wp = pad16(w);
    if (wp > kMaxW) {
        // wider operands (association designs with many covariates): blocks
        // of 128 columns, each contracted as above and placed in its columns
        out.alloc(std::max<uint64_t>(g.p, 1) * wp, c.stream);
        for (int c0 = 0; c0 < w; c0 += kMaxW) {
            const int wb = std::min(kMaxW, w - c0);
            DBuf<float> part;
            int wpb = 0;
            row_contract_base(c, g, s, W + c0, wb, ldw, part, wpb, sketch);
            if (g.p)
                SLFMM_CUDA(cudaMemcpy2DAsync(out.get() + c0, (size_t)wp * sizeof(float), part.get(),
                                             (size_t)wpb * sizeof(float), (size_t)wpb * sizeof(float), g.p,
                                             cudaMemcpyDeviceToDevice, c.stream));
        }
        return;
    }
    const uint64_t n_pad = round_up(g.n, 256);  // whole split-FP8 stages (256 codes)
    out.alloc(std::max<uint64_t>(g.p, 1) * wp, c.stream);
    const double bytes = (double)g.p * ceil_div(g.n, 4) + (double)g.p * w * 4 + (double)g.n * w * 4;
    if (c.precision == SLFMM_PREC_SPLIT_FP8) {
        // exact E4M3 genotypes x 4 scaled E4M3 terms of W; with the missing-call
        // indicator operand the epilogue applies out = s_j (P - mu_j (cs - M))
        Fp8RowPass rp;
        fp8_row_prepare(c, g, W, w, ldw, rp, sketch);
        fp8_row_run(c, g, s, rp, 0, g.p, out.get(), nullptr);
        return;
    }
    DBuf<float> W32(n_pad * wp, c.stream);
    launch_f64_to_f32_pad(c, W, g.n, w, ldw, W32.get(), n_pad, wp);
    if (tc_available(c)) {
        // exact genotypes x (hi + lo) BF16 split of W on the tensor cores, then
        // out = s_j (P - mu_j (colsum(W) - sum_{missing} W))
        DBuf<__nv_bfloat16> bs(2 * (uint64_t)wp * n_pad, c.stream);
        launch_split_bf16_f64(c, W, ldw, g.n, w, wp, n_pad, nullptr, bs.get());
        build_missing_lists(c, g);
        DBuf<double> cs(wp, c.stream);
        cs.zero();
        launch_colsums(c, W, g.n, w, ldw, cs.get());
        {
            ProfScope ps(c, "row_contract", bytes, 2.0 * g.n * g.p * w);
            launch_tc_rows(c, packed_rows(g), g.stride, g.p, g.n, bs.get(), n_pad, wp, out.get(), wp, 1, 0);
        }
        launch_rowfix_mean(c, out.get(), wp, g.p, w, g.miss_ptr.get(), g.miss_idx.get(), W32.get(), wp, g.n,
                           cs.get(), s.mean.get(), s.scale.get());
        return;
    }
    ProfScope ps(c, "row_contract", bytes, 2.0 * g.n * g.p * w);
    launch_row_lut(c, g, s.lut.get(), W32.get(), wp, out.get());
}

// S (n x wp, FP64) = Y_hat Q, Q = p x wp FP32 (w real columns)
void col_contract_base(Ctx& c, const Geno& g, const SnpStd& s, const float* Q, int w, int wp, DBuf<double>& S) {
    S.alloc(g.n * wp, c.stream);
    const double bytes = (double)g.p * ceil_div(g.n, 4) + (double)g.p * w * 4 + (double)g.n * w * 8;
    if (c.precision == SLFMM_PREC_SPLIT_FP8) {
        // forward pass on the transposed matrix: terms of diag(s) Q against the
        // genotypes plus terms of diag(mu s) Q against the missing-call
        // indicator, then S -= (mu s)^T Q
        const TileView tv = build_tiles(c, g, true);
        const uint64_t p_pad = round_up(g.p, 256);  // whole split-FP8 stages (256 codes)
        const uint64_t tiles = ceil_div(g.n, 128);
        Fp8Plan pl = fp8_plan(wp, true, tiles);
        const bool ind = pl.ok;
        if (!ind) pl = fp8_plan(wp, false, tiles);
        DBuf<uint8_t> B((uint64_t)pl.n_total * p_pad, c.stream);
        DBuf<float> isc(pl.n_total, c.stream);
        DBuf<double> coef(std::max<uint64_t>(g.p, 1), c.stream), colterm(wp, c.stream);
        launch_scale_product(c, s.mean.get(), s.scale.get(), g.p, coef.get());
        launch_fp8_terms_f32_pair(c, Q, wp, g.p, w, wp, p_pad, s.scale.get(), ind ? coef.get() : nullptr,
                                  (int)pl.n_main, (int)pl.n_total, B.get(), isc.get());
        const int splits = tc_split_count(c, g.n, g.p);
        DBuf<float> part((uint64_t)splits * g.n * wp, c.stream);
        int used = 0;
        {
            ProfScope ps(c, "col_contract", bytes, 2.0 * g.n * g.p * w);
            used = launch_tc8_rows(c, pl, tv, g.n, g.p, B.get(), isc.get(), p_pad, 0, nullptr,
                                   nullptr, nullptr, part.get(), wp, splits, g.n * wp);
        }
        launch_reduce_splits(c, part.get(), used, g.n, wp, g.n, S.get());
        launch_weighted_colsum(c, Q, wp, g.p, w, coef.get(), colterm.get());
        if (ind) {
            launch_sub_colterm(c, S.get(), wp, g.n, w, colterm.get());
        } else {
            build_missing_csc(c, g);
            launch_colfix_mean(c, S.get(), wp, g.n, w, g.missT_ptr.get(), g.missT_idx.get(), Q, wp, coef.get(),
                               colterm.get());
        }
        return;
    }
    if (tc_available(c)) {
        // forward pass on the transposed matrix (rows = samples, K = SNPs):
        // S = G~ (diag(s) Q) - 1 (mu s)^T Q + missing-call corrections
        build_transposed(c, g);
        build_missing_csc(c, g);
        const uint64_t p_pad = round_up(g.p, 128);
        DBuf<__nv_bfloat16> bs(2 * (uint64_t)wp * p_pad, c.stream);
        launch_split_bf16_f32(c, Q, wp, g.p, w, wp, p_pad, s.scale.get(), bs.get());
        const int splits = tc_split_count(c, g.n, g.p);
        DBuf<float> part((uint64_t)splits * g.n * wp, c.stream);
        int used = 0;
        {
            ProfScope ps(c, "col_contract", bytes, 2.0 * g.n * g.p * w);
            used = launch_tc_rows(c, g.packedT.get(), g.strideT, g.n, g.p, bs.get(), p_pad, wp, part.get(), wp, splits,
                                  g.n * wp);
        }
        launch_reduce_splits(c, part.get(), used, g.n, wp, g.n, S.get());
        DBuf<double> coef(std::max<uint64_t>(g.p, 1), c.stream), colterm(wp, c.stream);
        launch_scale_product(c, s.mean.get(), s.scale.get(), g.p, coef.get());
        launch_weighted_colsum(c, Q, wp, g.p, w, coef.get(), colterm.get());
        launch_colfix_mean(c, S.get(), wp, g.n, w, g.missT_ptr.get(), g.missT_idx.get(), Q, wp, coef.get(),
                           colterm.get());
        return;
    }
    ProfScope ps(c, "col_contract", bytes, 2.0 * g.n * g.p * w);
    launch_col_lut(c, g, s.lut.get(), Q, wp, S.get());
}

// ---------------------------------------------------------------------------
// Step 0 (src/precompute.rs:30-88) in thin form
// ---------------------------------------------------------------------------
// The passes with NMF values at the missing calls: the base pass counts a
// missing call at the SNP mean (standardised 0); the correction adds
// s_r (f_ir - mu_r) times the operand row.
void row_contract(Ctx& c, const Geno& g, const SnpStd& s, const double* W, int w, int ldw, DBuf<float>& out,
                  int& wp, bool sketch = false) {
    row_contract_base(c, g, s, W, w, ldw, out, wp, sketch);
    if (s.fill.k) {
        build_missing_lists(c, g);
        DBuf<float> W32(std::max<uint64_t>(g.n, 1) * wp, c.stream);
        launch_f64_to_f32_pad(c, W, g.n, w, ldw, W32.get(), g.n, wp);
        launch_fill_row_correct(c, g, out.get(), wp, w, W32.get(), wp, s.fill.W, s.fill.H, s.fill.k, s.mean.get(),
                                s.scale.get());
    }
}

void col_contract(Ctx& c, const Geno& g, const SnpStd& s, const float* Q, int w, int wp, DBuf<double>& S) {
    col_contract_base(c, g, s, Q, w, wp, S);
    if (s.fill.k) {
        build_missing_csc(c, g);
        launch_fill_col_correct(c, g, S.get(), wp, w, Q, wp, s.fill.W, s.fill.H, s.fill.k, s.mean.get(),
                                s.scale.get());
    }
}

// statistics with NMF values at the missing calls
void std_fill(Ctx& c, const Geno& g, int norm, const NmfFill& f, SnpStd& s) {
    const uint64_t p = std::max<uint64_t>(g.p, 1);
    s.mean.alloc(p, c.stream);
    s.scale.alloc(p, c.stream);
    s.tss.alloc(p, c.stream);
    s.zero_var.alloc(p, c.stream);
    s.lut.alloc(p * 4, c.stream);
    build_missing_lists(c, g);
    launch_fill_stats(c, g, norm, f.W, f.H, f.k, s.mean.get(), s.scale.get(), s.tss.get(), s.zero_var.get());
    launch_lut_std(c, g.p, s.mean.get(), s.scale.get(), s.lut.get());
    s.fill = f;
}

// raw products: mean = mean_src (or 0), scale = 1 -- the base passes then
// give the raw mean-filled product minus mean_r colsum(W) (or, with mean 0,
// the product with missing calls at 0)
void std_raw(Ctx& c, const Geno& g, const double* mean_src, SnpStd& s) {
    const uint64_t p = std::max<uint64_t>(g.p, 1);
    s.mean.alloc(p, c.stream);
    s.scale.alloc(p, c.stream);
    s.tss.alloc(p, c.stream);
    s.zero_var.alloc(p, c.stream);
    s.lut.alloc(p * 4, c.stream);
    if (mean_src) SLFMM_CUDA(cudaMemcpyAsync(s.mean.get(), mean_src, g.p * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
    else s.mean.zero();
    std::vector<double> ones(p, 1.0);
    h2d(c, s.scale.get(), ones.data(), p);
    s.tss.zero();
    s.zero_var.zero();
    launch_lut_std(c, g.p, s.mean.get(), s.scale.get(), s.lut.get());
    sync(c);
}

struct Step0 {
    uint64_t n = 0;
    int d = 0, r = 0;
    DBuf<double> xs;         // n x d centred covariates
    DBuf<double> qd;         // n x r left singular vectors of X
    DBuf<double> qd_omd;     // n x r: Q_d diag(1 - d_j)
    DBuf<double> qd_omdinv;  // n x r: Q_d diag(1 - 1/d_j)
    DBuf<double> ridge_inv;  // d x d
};

void center_covariates_dev(Ctx& c, double* xs, uint64_t n, int d, bool scale) {
    DBuf<double> means(std::max(d, 1), c.stream);
    launch_colmeans(c, xs, n, d, d, means.get());
    launch_center_cols(c, xs, n, d, d, means.get());
    if (scale) launch_scale_cols_sd(c, xs, n, d, d);
}

void step0(Ctx& c, const double* x_host, uint64_t n, int d, double lambda, bool scale_cov, Step0& s) {
    SLFMM_REQUIRE(lambda > 0.0, SLFMM_ERR_BAD_ARG,
                  "Ridge penalty lambda must be positive, got " + std::to_string(lambda) +
                      ". lambda=0 makes the D_lambda diagonal singular. Use a small positive value like 1e-10.");
    SLFMM_REQUIRE(d >= 1 && d <= kMaxDesign, SLFMM_ERR_BAD_ARG,
                  "number of covariates must be in 1.." + std::to_string(kMaxDesign));
    s.n = n;
    s.d = d;
    s.xs = upload(c, x_host, n * d);
    center_covariates_dev(c, s.xs.get(), n, d, scale_cov);
    DBuf<double> gx(d * d, c.stream), gtmp(d * d, c.stream), V(d * d, c.stream), sig(d, c.stream);
    launch_atb(c, s.xs.get(), d, s.xs.get(), d, n, d, d, gx.get());
    SLFMM_CUDA(cudaMemcpyAsync(gtmp.get(), gx.get(), d * d * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
    launch_jacobi_svd(c, gtmp.get(), d, V.get(), sig.get());
    // ridge: (X^T X + lambda I)^-1 with safe_inv semantics
    std::vector<double> gxh = fetch(c, gx.get(), (size_t)d * d);
    for (int j = 0; j < d; ++j) gxh[j * d + j] += lambda;
    DBuf<double> gl = upload(c, gxh.data(), gxh.size());
    s.ridge_inv.alloc(d * d, c.stream);
    DBuf<int> st(1, c.stream);
    DBuf<double> eps(1, c.stream);
    launch_inverse(c, gl.get(), d, s.ridge_inv.get(), st.get(), eps.get());
    std::vector<double> Vh = fetch(c, V.get(), (size_t)d * d);
    std::vector<double> ev = fetch(c, sig.get(), (size_t)d);
    safe_inv_report(fetch(c, st.get(), 1)[0], fetch(c, eps.get(), 1)[0], "X^T X + \u03bbI (ridge)");
    // kept directions: sigma_j^2 = eigenvalue of X^T X
    std::vector<int> keep;
    const double emax = ev.empty() ? 0.0 : ev[0];
    for (int j = 0; j < d; ++j)
        if (ev[j] > 0.0 && ev[j] > emax * 1e-24) keep.push_back(j);
    s.r = (int)keep.size();
    std::vector<double> Vs(d * std::max(s.r, 1)), Vo(Vs.size()), Vi(Vs.size());
    for (int k = 0; k < s.r; ++k) {
        const int j = keep[k];
        const double sigma = std::sqrt(ev[j]);
        const double dl = std::sqrt(lambda / (lambda + ev[j]));  // src/precompute.rs:55-59
        for (int i = 0; i < d; ++i) {
            const double v = Vh[i * d + j] / sigma;
            Vs[i * s.r + k] = v;
            Vo[i * s.r + k] = v * (1.0 - dl);
            Vi[i * s.r + k] = v * (1.0 - 1.0 / dl);
        }
    }
    s.qd.alloc(n * std::max(s.r, 1), c.stream);
    s.qd_omd.alloc(n * std::max(s.r, 1), c.stream);
    s.qd_omdinv.alloc(n * std::max(s.r, 1), c.stream);
    if (s.r) {
        DBuf<double> a = upload(c, Vs.data(), Vs.size()), b = upload(c, Vo.data(), Vo.size()),
                     e = upload(c, Vi.data(), Vi.size());
        launch_gemm_small(c, s.xs.get(), d, n, d, a.get(), s.r, s.r, 1.0, 0.0, s.qd.get(), s.r);
        launch_gemm_small(c, s.xs.get(), d, n, d, b.get(), s.r, s.r, 1.0, 0.0, s.qd_omd.get(), s.r);
        launch_gemm_small(c, s.xs.get(), d, n, d, e.get(), s.r, s.r, 1.0, 0.0, s.qd_omdinv.get(), s.r);
        sync(c);
    }
}

// A (n x b, lda) <- P A  or P^-1 A, P = I - Q_d (1 - D_d) Q_d^T
void apply_p(Ctx& c, const Step0& s, double* A, int b, int lda, bool inverse) {
    if (s.r == 0 || b == 0) return;
    DBuf<double> T(s.r * b, c.stream);
    launch_atb(c, s.qd.get(), s.r, A, lda, s.n, s.r, b, T.get());
    launch_gemm_small(c, inverse ? s.qd_omdinv.get() : s.qd_omd.get(), s.r, s.n, s.r, T.get(), b, b, -1.0,
                      1.0, A, lda);
}

void center_columns(Ctx& c, double* A, uint64_t m, int b, int lda) {
    DBuf<double> means(std::max(b, 1), c.stream);
    launch_colmeans(c, A, m, b, lda, means.get());
    launch_center_cols(c, A, m, b, lda, means.get());
}

// ---------------------------------------------------------------------------
// orthonormalisation (Cholesky-QR2, FP64 Gram + Cholesky)
// ---------------------------------------------------------------------------
void cholqr2_f32(Ctx& c, float* Z, uint64_t m, int a, int ld) {
    ProfScope ps(c, "cholqr2", 2.0 * m * a * 4, 4.0 * m * a * a);
    DBuf<double> G(a * a, c.stream), Linv(a * a, c.stream);
    DBuf<int> st(1, c.stream);
    for (int round = 0; round < 2; ++round) {
        launch_gram_f32(c, Z, ld, m, a, G.get());
        launch_cholesky(c, G.get(), a, st.get());
        launch_tri_inv_lower(c, G.get(), a, Linv.get());
        launch_trmul_f32(c, Z, ld, m, a, Linv.get());
    }
}

void cholqr2_f64(Ctx& c, double* A, uint64_t m, int a, int ld) {
    ProfScope ps(c, "cholqr2", 2.0 * m * a * 8, 4.0 * m * a * a);
    DBuf<double> G(a * a, c.stream), Linv(a * a, c.stream), LinvT(a * a, c.stream), tmp(m * a, c.stream);
    DBuf<int> st(1, c.stream);
    for (int round = 0; round < 2; ++round) {
        launch_atb(c, A, ld, A, ld, m, a, a, G.get());
        launch_cholesky(c, G.get(), a, st.get());
        launch_tri_inv_lower(c, G.get(), a, Linv.get());
        launch_transpose(c, Linv.get(), a, a, LinvT.get());
        launch_gemm_small(c, A, ld, m, a, LinvT.get(), a, a, 1.0, 0.0, tmp.get(), a);
        SLFMM_CUDA(cudaMemcpy2DAsync(A, ld * sizeof(double), tmp.get(), a * sizeof(double), a * sizeof(double), m,
                                     cudaMemcpyDeviceToDevice, c.stream));
    }
}

// ---------------------------------------------------------------------------
// randomized SVD (src/rsvd.rs:26-177), thin form: sketch P Omega, forward
// passes P (Y Q_z), U_hat = P^-1 U(P Y Q_z)[:, :K]
// ---------------------------------------------------------------------------
// the sketch operand P Omega (n x l), centred
void sketch_operand(Ctx& c, const Step0& s0, uint64_t n, int l, uint64_t seed, const double* omega_host,
                    DBuf<double>& W) {
    W.alloc(n * l, c.stream);
    if (omega_host) h2d(c, W.get(), omega_host, n * l);
    else draw_normal(c, seed, n, l, W.get());
    apply_p(c, s0, W.get(), l, l, false);                    // M^T Omega analogue (:51)
    center_columns(c, W.get(), n, l, l);
}

void rsvd_checks(uint64_t n, uint64_t p, int l) {
    SLFMM_REQUIRE(l <= 64, SLFMM_ERR_BAD_ARG, "K + oversampling must be <= 64");
    SLFMM_REQUIRE(p >= (uint64_t)l, SLFMM_ERR_BAD_ARG, "fewer estimation SNPs than K + oversampling");
    SLFMM_REQUIRE(n >= (uint64_t)l, SLFMM_ERR_BAD_ARG, "fewer samples than K + oversampling");
}

// Z_pre: the sketch Y_hat^T P Omega already computed (p x pad16(l), FP32)
void rsvd(Ctx& c, const Geno& g, const SnpStd& st, const Step0& s0, int K, int l, int q,
          uint64_t seed, const double* omega_host, DBuf<double>& u_hat, DBuf<float>* Z_pre = nullptr) {
    const uint64_t n = g.n;
    rsvd_checks(n, g.p, l);
    DBuf<float> Z;
    int wp = 0;
    if (Z_pre) {
        Z = std::move(*Z_pre);
        wp = pad16(l);
    } else {
        DBuf<double> W;
        sketch_operand(c, s0, n, l, seed, omega_host, W);
        row_contract(c, g, st, W.get(), l, l, Z, wp, true);  // sketch (:56-72)
    }
    cholqr2_f32(c, Z.get(), g.p, l, wp);                     // QR (:75)
    for (int it = 0; it < q; ++it) {
        DBuf<double> S;
        col_contract(c, g, st, Z.get(), l, wp, S);              // fwd (:88-97)
        apply_p(c, s0, S.get(), l, wp, false);
        cholqr2_f64(c, S.get(), n, l, wp);                   // QR(a_qz) (:104-105)
        apply_p(c, s0, S.get(), l, wp, false);               // M^T Q (:106)
        center_columns(c, S.get(), n, l, wp);
        row_contract(c, g, st, S.get(), l, wp, Z, wp);       // bwd (:111-128)
        cholqr2_f32(c, Z.get(), g.p, l, wp);                 // QR (:131)
    }
    DBuf<double> B;
    col_contract(c, g, st, Z.get(), l, wp, B);                  // projection (:138-157)
    apply_p(c, s0, B.get(), l, wp, false);
    // small SVD (:160-173): eigen-decomposition of the l x l Gram (FP64)
    DBuf<double> G(l * l, c.stream), V(l * l, c.stream), sig(l, c.stream);
    launch_atb(c, B.get(), wp, B.get(), wp, n, l, l, G.get());
    launch_jacobi_svd(c, G.get(), l, V.get(), sig.get());
    std::vector<double> Vh = fetch(c, V.get(), (size_t)l * l);
    std::vector<double> ev = fetch(c, sig.get(), (size_t)l);
    std::vector<double> Vk((size_t)l * K);
    for (int k = 0; k < K; ++k) {
        const double sg = std::sqrt(std::max(ev[k], 0.0));
        for (int i = 0; i < l; ++i) Vk[i * K + k] = sg > 0 ? Vh[i * l + k] / sg : 0.0;
    }
    DBuf<double> Vkd = upload(c, Vk.data(), Vk.size());
    u_hat.alloc(n * K, c.stream);
    launch_gemm_small(c, B.get(), wp, n, l, Vkd.get(), K, K, 1.0, 0.0, u_hat.get(), K);
    apply_p(c, s0, u_hat.get(), K, K, true);                 // U_hat = Q D^-1 U_small
    sync(c);
}

// ---------------------------------------------------------------------------
// association pass (src/testing.rs:252-528)
// ---------------------------------------------------------------------------
struct AssocOut {
    double* beta;
    double* tstat;
    double* pvalue;
    double* r2;
    double* gif_per_trait;
    double gif;
};

void assoc(Ctx& c, const Geno& g, const SnpStd& st, const Step0& s0, const double* u_hat_dev, int K,
           AssocOut& out) {
    const uint64_t n = g.n, p = g.p;
    const int d = s0.d, w = 1 + d + K;
    if (n <= (uint64_t)(1 + d + K))
        throw Error(SLFMM_ERR_DF_NONPOSITIVE,
                    "Insufficient degrees of freedom: n=" + std::to_string(n) + " samples but 1+d+K=1+" +
                        std::to_string(d) + "+" + std::to_string(K) + "=" + std::to_string(1 + d + K) +
                        ". Need n > 1 + d + K for valid t-tests. Reduce K or add more samples.");
    SLFMM_REQUIRE(w <= kMaxDesign, SLFMM_ERR_BAD_ARG,
                  "1 + d + K must be <= " + std::to_string(kMaxDesign) + " (got " + std::to_string(w) + ")");
    const double df = (double)(n - 1 - d - K);
    // design C = [1 | X | U_hat], unit-norm columns
    DBuf<double> C(n * w, c.stream), G(w * w, c.stream);
    launch_build_design(c, s0.xs.get(), d, u_hat_dev, K, n, C.get());
    launch_atb(c, C.get(), w, C.get(), w, n, w, w, G.get());
    // safe_inv of C^T C and X^T X (src/testing.rs:306, :316): an exactly
    // singular matrix (a zero LU pivot, e.g. a duplicated covariate) gets
    // eps = 1e-8 max|diag| on its diagonal, with the reference's warning.
    // The reference then uses (C^T C + eps I)^-1.  Its limit for small eps,
    // with N an orthonormal basis of the null space of C, is theta = the
    // minimum-norm least-squares solution (I - N N^T) theta_any and c_jj =
    // [(C^T C)^+]_jj + (N N^T)_jj / eps; that form is used below (applying
    // (C^T C + eps I)^-1 directly would multiply the contraction's rounding
    // by 1/sqrt(eps)).  RSS, SS_cov and beta depend only on span(C), which
    // the column-dropping factorisation spans exactly.
    double ctc_eps = 0.0;
    {
        DBuf<double> inv((size_t)w * w, c.stream), epsd(1, c.stream);
        DBuf<int> sti(1, c.stream);
        if (d > 0) {
            DBuf<double> xtx((size_t)d * d, c.stream);
            launch_atb(c, s0.xs.get(), d, s0.xs.get(), d, n, d, d, xtx.get());
            launch_inverse(c, xtx.get(), d, inv.get(), sti.get(), epsd.get());
            safe_inv_report(fetch(c, sti.get(), 1)[0], fetch(c, epsd.get(), 1)[0], "X^T X for sequential R^2");
        }
        launch_inverse(c, G.get(), w, inv.get(), sti.get(), epsd.get());
        const int status = fetch(c, sti.get(), 1)[0];
        const double eps = fetch(c, epsd.get(), 1)[0];
        safe_inv_report(status, eps, "C^T C  where C = [1 | X | U_hat]");
        if (status == 1) ctc_eps = eps;
    }
    std::vector<double> Gh = fetch(c, G.get(), (size_t)w * w);
    const std::vector<double> Graw = Gh;  // unnormalised C^T C
    std::vector<double> f(w);
    for (int k = 0; k < w; ++k) f[k] = Gh[k * w + k] > 0 ? 1.0 / std::sqrt(Gh[k * w + k]) : 0.0;
    DBuf<double> fd = upload(c, f.data(), w);
    launch_scale_cols(c, C.get(), n, w, w, fd.get());
    for (int i = 0; i < w; ++i)
        for (int j = 0; j < w; ++j) Gh[i * w + j] *= f[i] * f[j];
    for (int k = 0; k < w; ++k)
        if (f[k] == 0.0) Gh[k * w + k] = 0.0;
    DBuf<double> L = upload(c, Gh.data(), Gh.size());
    DBuf<int> st1(1, c.stream), dropped(w, c.stream);
    launch_cholesky(c, L.get(), w, st1.get(), 1e-10, dropped.get());
    DBuf<double> Linv(w * w, c.stream);
    launch_tri_inv_lower(c, L.get(), w, Linv.get());
    std::vector<double> Li = fetch(c, Linv.get(), (size_t)w * w);
    std::vector<int> dr = fetch(c, dropped.get(), (size_t)w);
    for (int k = 0; k < w; ++k)
        if (dr[k])
            for (int m = 0; m < w; ++m) Li[k * w + m] = 0.0;
    // Q_C = C Linv^T (dropped columns zero)
    std::vector<double> LiT((size_t)w * w);
    for (int i = 0; i < w; ++i)
        for (int j = 0; j < w; ++j) LiT[j * w + i] = Li[i * w + j];
    DBuf<double> LiTd = upload(c, LiT.data(), LiT.size());
    DBuf<double> QC(n * w, c.stream);
    launch_gemm_small(c, C.get(), w, n, w, LiTd.get(), w, w, 1.0, 0.0, QC.get(), w);
    // theta rows and c_jj (coefficients of the X columns, src/testing.rs:1036-1048)
    const int wu = w - 1;
    std::vector<float> th((size_t)d * wu, 0.f), bt((size_t)d * wu, 0.f);
    std::vector<double> cjj(d, 0.0);
    std::vector<uint8_t> drop_x(d, 0);
    bool any_dropped = false;
    for (int k = 0; k < w; ++k) any_dropped = any_dropped || dr[k] != 0;
    if (any_dropped) {
        // C^T C singular (a zero LU pivot) or so close to it that the
        // factorisation dropped a column: the limit of the regularised solve,
        // in unnormalised coordinates (theta_i = f_i theta~_i).  Without a
        // zero pivot the reference inverts the ill-conditioned matrix as it
        // is, which also gives every column of the null space a near-zero t;
        // eps = 1e-8 max|diag| stands for its effective regulariser then.
        if (!(ctc_eps > 0.0)) {
            double dmax = 0.0;
            for (int k = 0; k < w; ++k) dmax = std::max(dmax, std::fabs(Graw[k * w + k]));
            ctc_eps = 1e-8 * std::max(dmax, 1e-300);
        }
        std::vector<double> Ginv((size_t)w * w, 0.0);  // generalised inverse on the kept columns
        for (int i = 0; i < w; ++i)
            for (int j = 0; j < w; ++j) {
                double acc = 0.0;
                for (int k = std::max(i, j); k < w; ++k) acc += Li[k * w + i] * Li[k * w + j];
                Ginv[i * w + j] = f[i] * acc * f[j];
            }
        // null vectors n_b = e_b - alpha, alpha = (C_K^T C_K)^-1 C_K^T c_b, one
        // per dropped column b, orthonormalised (modified Gram-Schmidt)
        std::vector<std::vector<double>> nv;
        for (int b = 0; b < w; ++b) {
            if (!dr[b]) continue;
            std::vector<double> v(w, 0.0);
            v[b] = 1.0;
            for (int i = 0; i < w; ++i) {
                if (dr[i]) continue;
                double a = 0.0;
                for (int j = 0; j < w; ++j)
                    if (!dr[j]) a += Ginv[i * w + j] * Graw[j * w + b];
                v[i] -= a;
            }
            for (const auto& q : nv) {
                double dot = 0.0;
                for (int i = 0; i < w; ++i) dot += q[i] * v[i];
                for (int i = 0; i < w; ++i) v[i] -= dot * q[i];
            }
            double nn = 0.0;
            for (int i = 0; i < w; ++i) nn += v[i] * v[i];
            if (nn > 0.0) {
                nn = 1.0 / std::sqrt(nn);
                for (int i = 0; i < w; ++i) v[i] *= nn;
                nv.push_back(std::move(v));
            }
        }
        // theta = M u with M_jk = sum_i (I - N N^T)_ji f_i Li_ki
        for (int jj = 0; jj < d; ++jj) {
            const int j = 1 + jj;
            std::vector<double> pj(w);
            for (int i = 0; i < w; ++i) {
                double nn = 0.0;
                for (const auto& q : nv) nn += q[j] * q[i];
                pj[i] = (i == j ? 1.0 : 0.0) - nn;
            }
            double s = 0.0;
            for (int k = 0; k < w; ++k) {
                double m = 0.0;
                for (int i = 0; i <= k; ++i) m += pj[i] * f[i] * Li[k * w + i];
                if (k > 0) th[jj * wu + (k - 1)] = (float)m;
                s += m * m;
            }
            double njj = 0.0;
            for (const auto& q : nv) njj += q[j] * q[j];
            cjj[jj] = s + njj / ctc_eps;
            drop_x[jj] = 0;
        }
    } else {
        for (int jj = 0; jj < d; ++jj) {
            const int col = 1 + jj;
            drop_x[jj] = (uint8_t)(dr[col] != 0);
            double s = 0.0;
            for (int k = col; k < w; ++k) {
                th[jj * wu + (k - 1)] = (float)Li[k * w + col];
                s += Li[k * w + col] * Li[k * w + col];
            }
            cjj[jj] = s;
        }
    }
    // beta rows: R ((I - P_U) X)^T Q_C  (src/testing.rs:285-296, 360-362)
    {
        DBuf<double> UtU(K * K, c.stream), UtUi(K * K, c.stream), M1(K * d, c.stream), M2(K * d, c.stream),
            F(n * d, c.stream), FtQ(d * w, c.stream), Bpp(d * w, c.stream);
        DBuf<int> sti(1, c.stream);
        DBuf<double> epsd(1, c.stream);
        launch_atb(c, u_hat_dev, K, u_hat_dev, K, n, K, K, UtU.get());
        launch_inverse(c, UtU.get(), K, UtUi.get(), sti.get(), epsd.get());
        launch_atb(c, u_hat_dev, K, s0.xs.get(), d, n, K, d, M1.get());
        launch_gemm_small(c, UtUi.get(), K, K, K, M1.get(), d, d, 1.0, 0.0, M2.get(), d);
        SLFMM_CUDA(cudaMemcpyAsync(F.get(), s0.xs.get(), n * d * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
        launch_gemm_small(c, u_hat_dev, K, n, K, M2.get(), d, d, -1.0, 1.0, F.get(), d);
        launch_atb(c, F.get(), d, QC.get(), w, n, d, w, FtQ.get());
        launch_gemm_small(c, s0.ridge_inv.get(), d, d, d, FtQ.get(), w, w, 1.0, 0.0, Bpp.get(), w);
        safe_inv_report(fetch(c, sti.get(), 1)[0], fetch(c, epsd.get(), 1)[0], "U_hat^T U_hat");
        std::vector<double> Bh = fetch(c, Bpp.get(), (size_t)d * w);
        for (int jj = 0; jj < d; ++jj)
            for (int k = 1; k < w; ++k) bt[jj * wu + (k - 1)] = (float)Bh[jj * w + k];
    }
    DBuf<float> thd = upload(c, th.data(), th.size()), btd = upload(c, bt.data(), bt.size());
    DBuf<double> cjjd = upload(c, cjj.data(), cjj.size());
    DBuf<uint8_t> dxd = upload(c, drop_x.data(), drop_x.size());
    AssocConsts k{d, wu, df, thd.get(), btd.get(), cjjd.get(), dxd.get(), st.zero_var.get()};
    const uint64_t pp = std::max<uint64_t>(p, 1);
    DBuf<double> beta(pp * d, c.stream), r2(pp * 3, c.stream), t64(pp * d, c.stream), pv(pp * d, c.stream);
    DBuf<float> t32(pp * d, c.stream);
    DBuf<uint32_t> hist((size_t)d * kHistBins, c.stream);
    hist.zero();
    phase(c, "association design");
    // u = Q_C[:, 1:]^T y for every SNP, then the statistics.  With page-locked
    // host outputs the split-FP8 pass runs in chunks of SNPs: each chunk's
    // beta, r2 and t are final after its epilogue and copy out on the copy
    // stream while later chunks compute (only the p-values wait for the GIF).
    DBuf<float> U;
    int wp = 0;
    const uint64_t chunk = round_up(ceil_div(p, 8), 128);
    const bool chunked = c.precision == SLFMM_PREC_SPLIT_FP8 && st.fill.k == 0 && p >= 2 * chunk &&
                         (out.beta || out.r2 || out.tstat) && (!out.beta || is_pinned(out.beta)) &&
                         (!out.r2 || is_pinned(out.r2)) && (!out.tstat || is_pinned(out.tstat));
    bool copied = false;
    if (chunked) {
        Fp8RowPass rp;
        fp8_row_prepare(c, g, QC.get() + 1, wu, w, rp);
        wp = rp.wp;
        U.alloc(pp * wp, c.stream);
        DBuf<int> err(1, c.stream);
        err.zero();
        cudaEvent_t ev;
        SLFMM_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        struct EvGuard {
            cudaEvent_t e;
            ~EvGuard() { cudaEventDestroy(e); }
        } evg{ev};
        for (uint64_t r0 = 0; r0 < p; r0 += chunk) {
            const uint64_t rows = std::min(chunk, p - r0);
            fp8_row_run(c, g, st, rp, r0, rows, U.get(), err.get());
            AssocConsts kc = k;
            kc.zero_var = k.zero_var ? k.zero_var + r0 : nullptr;
            {
                ProfScope ps(c, "assoc_epilogue", (double)rows * (wu * 4 + 8 + d * 12 + 24), 4.0 * rows * d * wu);
                launch_assoc_epilogue(c, rows, U.get() + r0 * wp, wp, st.tss.get() + r0, kc, beta.get() + r0 * d,
                                      t32.get() + r0 * d, r2.get() + r0 * 3, hist.get());
            }
            // t reaches the host as the widened FP32 statistic (what the
            // calibration writes), so it is final here too
            if (out.tstat) launch_f32_to_f64(c, t32.get() + r0 * d, rows, d, d, t64.get() + r0 * d, d);
            SLFMM_CUDA(cudaEventRecord(ev, c.stream));
            SLFMM_CUDA(cudaStreamWaitEvent(c.copy_stream, ev, 0));
            if (out.tstat)
                SLFMM_CUDA(cudaMemcpyAsync(out.tstat + r0 * d, t64.get() + r0 * d, rows * d * sizeof(double),
                                           cudaMemcpyDeviceToHost, c.copy_stream));
            if (out.beta)
                SLFMM_CUDA(cudaMemcpyAsync(out.beta + r0 * d, beta.get() + r0 * d, rows * d * sizeof(double),
                                           cudaMemcpyDeviceToHost, c.copy_stream));
            if (out.r2)
                SLFMM_CUDA(cudaMemcpyAsync(out.r2 + r0 * 3, r2.get() + r0 * 3, rows * 3 * sizeof(double),
                                           cudaMemcpyDeviceToHost, c.copy_stream));
        }
        const int e = fetch(c, err.get(), 1)[0];
        if (e) {
            SLFMM_CUDA(cudaStreamSynchronize(c.copy_stream));
            throw_tc8_timeout(e);
        }
        copied = true;
        phase(c, "association row pass and statistics");
    } else {
        row_contract(c, g, st, QC.get() + 1, wu, w, U, wp);
        phase(c, "association row pass");
        ProfScope ps(c, "assoc_epilogue", (double)p * (wu * 4 + 8 + d * 12 + 24), 4.0 * p * d * wu);
        launch_assoc_epilogue(c, p, U.get(), wp, st.tss.get(), k, beta.get(), t32.get(), r2.get(), hist.get());
    }
    DBuf<double> graw(d, c.stream);
    launch_gif(c, hist.get(), d, graw.get());
    std::vector<double> gr = fetch(c, graw.get(), (size_t)d);
    std::vector<double> gpt(d);
    double gsum = 0.0;
    for (int jj = 0; jj < d; ++jj) {
        gpt[jj] = std::max(gr[jj], 1.0);
        gsum += gr[jj];
    }
    out.gif = gsum / d;
    if (out.gif_per_trait) std::copy(gpt.begin(), gpt.end(), out.gif_per_trait);
    DBuf<double> gptd = upload(c, gpt.data(), gpt.size());
    // t64 is already widened (and being copied out) when the pass ran in chunks
    launch_calibrate(c, p, d, t32.get(), gptd.get(), copied && out.tstat ? nullptr : t64.get(), pv.get());
    phase(c, "association statistics, GIF");
    if (out.beta && !copied) d2h(c, out.beta, beta.get(), p * d);
    if (out.tstat && !copied) d2h(c, out.tstat, t64.get(), p * d);
    if (out.pvalue) d2h(c, out.pvalue, pv.get(), p * d);
    if (out.r2 && !copied) d2h(c, out.r2, r2.get(), p * 3);
    sync(c);
    SLFMM_CUDA(cudaStreamSynchronize(c.copy_stream));
    phase(c, "results to host");
}

// ---------------------------------------------------------------------------
// NMF imputation (src/nmf.rs:80-455, src/parallel.rs:219-321,
// src/testing.rs:423-487)
// ---------------------------------------------------------------------------
struct NmfModel {
    int k = 0;
    DBuf<double> W;   // n x k
    DBuf<double> Ht;  // p x k: H transposed, one row per SNP
    std::vector<double> cv;
    double cv_mean = 0.0;
    uint64_t total = 0;
};

// out (n x k) = W (W^T W)^-1, i.e. (W^+)^T, with safe_inv semantics
void nmf_pinv_t(Ctx& c, const double* W, uint64_t n, int k, DBuf<double>& out, const char* what) {
    DBuf<double> wtw(k * k, c.stream), inv(k * k, c.stream), eps(1, c.stream);
    DBuf<int> st(1, c.stream);
    launch_atb(c, W, k, W, k, n, k, k, wtw.get());
    launch_inverse(c, wtw.get(), k, inv.get(), st.get(), eps.get());
    safe_inv_report(fetch(c, st.get(), 1)[0], fetch(c, eps.get(), 1)[0], what);
    out.alloc(std::max<uint64_t>(n, 1) * k, c.stream);
    launch_gemm_small(c, W, k, n, k, inv.get(), k, k, 1.0, 0.0, out.get(), k);
}

void nmf_normalize(Ctx& c, NmfModel& m, uint64_t n, uint64_t p, double eps) {
    DBuf<double> cs(m.k, c.stream);
    cs.zero();
    launch_colsums(c, m.W.get(), n, m.k, m.k, cs.get());
    launch_nmf_normalize(c, m.W.get(), n, m.Ht.get(), p, m.k, cs.get(), eps);
}

// H rows max(0, W^+ y~) for every SNP of g, y~ = raw calls, missing at the
// SNP's observed mean (the on-the-fly fill, src/parallel.rs:249-282)
void nmf_h_meanfill(Ctx& c, const Geno& g, const SnpStd& rawm, const double* Wpt, int k, DBuf<double>& Ht) {
    DBuf<float> U;
    int up = 0;
    row_contract(c, g, rawm, Wpt, k, k, U, up);
    DBuf<double> cs(k, c.stream);
    cs.zero();
    launch_colsums(c, Wpt, g.n, k, k, cs.get());
    launch_add_mean_colsum(c, U.get(), up, g.p, k, rawm.mean.get(), cs.get());
    Ht.alloc(std::max<uint64_t>(g.p, 1) * k, c.stream);
    launch_nmf_clamp0_f32(c, U.get(), up, Ht.get(), g.p, k);
}

void to_f32(Ctx& c, const double* A, uint64_t m, int a, DBuf<float>& out, int ld) {
    out.alloc(std::max<uint64_t>(m, 1) * ld, c.stream);
    launch_f64_to_f32_pad(c, A, m, a, a, out.get(), m, ld);
}

// (sum |g - pred|, sum |g - mean|, count) over a p x 3 partials array
std::vector<double> sum3(Ctx& c, const DBuf<double>& part, uint64_t p) {
    DBuf<double> tot(3, c.stream);
    tot.zero();
    launch_colsums(c, part.get(), p, 3, 3, tot.get());
    return fetch(c, tot.get(), 3);
}

void nmf_estimate(Ctx& c, const Geno& g, const slfmm_config* cfg, NmfModel& m) {
    const int k = cfg->nmf_k ? (int)cfg->nmf_k : (int)cfg->k;
    SLFMM_REQUIRE(k >= 1 && k <= kMaxNmfK, SLFMM_ERR_BAD_ARG,
                  "NMF rank must be in 1.." + std::to_string(kMaxNmfK) + ", got " + std::to_string(k));
    const double eps = cfg->nmf_eps > 0 ? cfg->nmf_eps : 1e-16;
    const uint64_t chunk = cfg->chunk_size ? cfg->chunk_size : 10000;
    const uint64_t n = g.n, p = g.p;
    const int l = k + 10;
    SLFMM_REQUIRE(p >= (uint64_t)l && n >= (uint64_t)l, SLFMM_ERR_BAD_ARG, "too few SNPs or samples for the NMF probe");
    m.k = k;
    SnpStd sm, raw0, rawm;
    std_mean(c, g, SLFMM_NORM_EIGENSTRAT, sm);
    std_raw(c, g, nullptr, raw0);
    std_raw(c, g, sm.mean.get(), rawm);
    build_missing_lists(c, g);
    build_missing_csc(c, g);
    // init_from_random_probe (src/nmf.rs:279-362): Z = Y_meanraw^T Omega',
    // W = |Omega' V_k| with V the right singular vectors of Z, H = max(0, W^+ Y)
    DBuf<double> Om(n * l, c.stream);
    draw_normal(c, cfg->seed + 1000000ull, n, l, Om.get());
    DBuf<float> Z;
    int zp = 0;
    row_contract(c, g, rawm, Om.get(), l, l, Z, zp);
    DBuf<double> csO(l, c.stream);
    csO.zero();
    launch_colsums(c, Om.get(), n, l, l, csO.get());
    launch_add_mean_colsum(c, Z.get(), zp, p, l, sm.mean.get(), csO.get());
    DBuf<double> G(l * l, c.stream), V(l * l, c.stream), sig(l, c.stream), Wr(n * k, c.stream);
    launch_gram_f32(c, Z.get(), zp, p, l, G.get());
    launch_jacobi_svd(c, G.get(), l, V.get(), sig.get());
    launch_gemm_small(c, Om.get(), l, n, l, V.get(), l, k, 1.0, 0.0, Wr.get(), k);
    m.W.alloc(n * k, c.stream);
    launch_nmf_abs_f64(c, Wr.get(), k, m.W.get(), n, k);
    {
        DBuf<double> Wpt;
        nmf_pinv_t(c, m.W.get(), n, k, Wpt, "W_init^T W_init");
        nmf_h_meanfill(c, g, rawm, Wpt.get(), k, m.Ht);
    }
    // W, H >= eps, normalise (src/nmf.rs:118-126)
    DBuf<double> zeros(std::max<uint64_t>(n, p) * k, c.stream);
    zeros.zero();
    launch_nmf_update_f64(c, m.W.get(), n, k, m.W.get(), k, zeros.get(), eps);
    launch_nmf_update_f64(c, m.Ht.get(), p, k, m.Ht.get(), k, zeros.get(), eps);
    nmf_normalize(c, m, n, p, eps);
    const int kp = pad16(k);
    DBuf<double> hh(k * k, c.stream), wtw(k * k, c.stream), denW(n * k, c.stream), denH(p * k, c.stream);
    DBuf<double> part(std::max<uint64_t>(p, 1) * 3, c.stream);
    m.cv.clear();
    m.total = 0;
    for (int it = 0; it < (int)cfg->nmf_iter; ++it) {
        // W step: N_W = Y~ H^T, HH = H H^T, W <- W N_W / (W HH)   (src/nmf.rs:140-190)
        DBuf<float> W32, H32, H32p;
        to_f32(c, m.W.get(), n, k, W32, k);
        to_f32(c, m.Ht.get(), p, k, H32, k);
        to_f32(c, m.Ht.get(), p, k, H32p, kp);
        DBuf<double> NW;
        col_contract(c, g, raw0, H32p.get(), k, kp, NW);
        launch_fill_col_correct(c, g, NW.get(), kp, k, H32p.get(), kp, W32.get(), H32.get(), k, raw0.mean.get(),
                                raw0.scale.get());
        launch_atb(c, m.Ht.get(), k, m.Ht.get(), k, p, k, k, hh.get());
        launch_gemm_small(c, m.W.get(), k, n, k, hh.get(), k, k, 1.0, 0.0, denW.get(), k);
        launch_nmf_update_f64(c, m.W.get(), n, k, NW.get(), kp, denW.get(), eps);
        nmf_normalize(c, m, n, p, eps);
        // H step with the new W: N_H = W^T Y~, H <- H N_H / (W^T W H)   (:192-240)
        launch_atb(c, m.W.get(), k, m.W.get(), k, n, k, k, wtw.get());
        to_f32(c, m.W.get(), n, k, W32, k);
        to_f32(c, m.Ht.get(), p, k, H32, k);
        DBuf<float> NH;
        int np_ = 0;
        row_contract(c, g, raw0, m.W.get(), k, k, NH, np_);
        launch_fill_row_correct(c, g, NH.get(), np_, k, W32.get(), k, W32.get(), H32.get(), k, raw0.mean.get(),
                                raw0.scale.get());
        launch_gemm_small(c, m.Ht.get(), k, p, k, wtw.get(), k, k, 1.0, 0.0, denH.get(), k);
        launch_nmf_update_f32(c, m.Ht.get(), p, k, NH.get(), np_, denH.get(), eps);
        nmf_normalize(c, m, n, p, eps);
        // CV on held-out calls (src/nmf.rs:379-455), mask stream seed + it
        to_f32(c, m.W.get(), n, k, W32, k);
        to_f32(c, m.Ht.get(), p, k, H32, k);
        launch_nmf_cv(c, g, chunk, cfg->seed + (uint64_t)it, cfg->nmf_cv_rate, W32.get(), H32.get(), k, part.get());
        const std::vector<double> t = sum3(c, part, p);
        const uint64_t cnt = (uint64_t)(t[2] + 0.5);
        m.cv.push_back(cnt ? t[0] / (double)cnt : 0.0);
        m.cv_mean = cnt ? t[1] / (double)cnt : 0.0;
        m.total += cnt;
        if (c.verbose)
            fprintf(stderr, "NMF iteration %d: CV MAE %.6f (mean imputation %.6f, %llu held out)\n", it + 1,
                    m.cv.back(), m.cv_mean, (unsigned long long)cnt);
    }
}

void check_cfg(const slfmm_config* cfg) {
    SLFMM_REQUIRE(cfg != nullptr, SLFMM_ERR_BAD_ARG, "null config");
    SLFMM_REQUIRE(cfg->k >= 1, SLFMM_ERR_BAD_ARG, "K must be >= 1");
    SLFMM_REQUIRE(cfg->norm == SLFMM_NORM_CENTER_ONLY || cfg->norm == SLFMM_NORM_EIGENSTRAT, SLFMM_ERR_BAD_ARG,
                  "unknown normalisation");
    SLFMM_REQUIRE(cfg->impute == SLFMM_IMPUTE_MEAN || cfg->impute == SLFMM_IMPUTE_NMF, SLFMM_ERR_BAD_ARG,
                  "unknown imputation strategy");
}

// The sketch pass of the randomized SVD run on each chunk of an upload as it
// lands: the chunk's SNP statistics, then Y_hat^T (P Omega) for its rows.
// The operands and kernels are those of the pass after the upload, so the
// sketch is identical; it only moves under the host-link-bound copies.
struct Presketch : ChunkHook {
    // inputs of the setup
    uint64_t n = 0, p = 0;
    const double* x = nullptr;
    int d = 0;
    const slfmm_config* cfg = nullptr;
    const double* omega = nullptr;
    // state
    Step0 s0;
    SnpStd se;
    int norm = 0, l = 0;
    Fp8RowPass rp;
    DBuf<float> Z;
    DBuf<int> err;
    // covariates (Step 0), P Omega and its split-FP8 operand, while the first
    // chunks are being copied
    void begin(Ctx& c) override {
        step0(c, x, n, d, cfg->lambda, cfg->scale_cov != 0, s0);
        DBuf<double> W;
        sketch_operand(c, s0, n, l, cfg->seed, omega, W);
        // the form the pass over the resident matrix takes (fp8_row_prepare)
        fp8_row_operand_prepare(c, n, ceil_div(p, 128), W.get(), l, l, fp8_sketch_takes_indicator(n), rp);
        se.mean.alloc(p, c.stream);
        se.scale.alloc(p, c.stream);
        se.tss.alloc(p, c.stream);
        se.zero_var.alloc(p, c.stream);
        Z.alloc(p * rp.wp, c.stream);
        err.alloc(1, c.stream);
        err.zero();
    }
    void rows(Ctx& c, const Geno& g, uint64_t r0, uint64_t r1) override {
        launch_stats_mean_range(c, g, r0, r1 - r0, norm, se.mean.get(), se.scale.get(), se.tss.get(),
                                se.zero_var.get());
        fp8_row_run(c, g, se, rp, r0, r1 - r0, Z.get(), err.get(), false);
    }
    // after the upload, once the missing-call lists are complete: the per-SNP
    // fix of the pass without the indicator, over every row at once
    void finish(Ctx& c, const Geno& g) {
        fp8_row_fix(c, g, se, rp, 0, g.p, Z.get());
    }
};

// true when the estimation and testing matrices are the same upload of p SNPs
// with mean imputation (host-side checks only; the device setup runs in
// begin())
bool presketch_eligible(Ctx& c, uint64_t n, uint64_t p, const double* x, int d, const slfmm_config* cfg,
                        const double* omega, Presketch& ps) {
    if (c.precision != SLFMM_PREC_SPLIT_FP8 || cfg->impute != SLFMM_IMPUTE_MEAN || p == 0) return false;
    const char* env = std::getenv("SLFMM_PRESKETCH");  // tuning override: 0 runs the sketch after the upload
    if (env && env[0] == '0') return false;
    check_cfg(cfg);
    ps.l = (int)cfg->k + (int)cfg->oversampling;
    if (ps.l > 64 || p < (uint64_t)ps.l || n < (uint64_t)ps.l) return false;  // the fit reports these
    ps.n = n;
    ps.p = p;
    ps.x = x;
    ps.d = d;
    ps.cfg = cfg;
    ps.omega = omega;
    ps.norm = cfg->norm;
    return true;
}

void fit_impl(Ctx& c, const Geno& ge, const Geno& gf, const double* x, int d, const slfmm_config* cfg,
              const double* omega, slfmm_results* res, Presketch* pre = nullptr) {
    if (!pre) phase(c, "", true);
    check_cfg(cfg);
    SLFMM_REQUIRE(ge.n == gf.n, SLFMM_ERR_BAD_ARG, "estimation and testing genotypes have different sample counts");
    // the reference's sketch stream is drawn on host threads while Step 0 and
    // the SNP statistics run on the device
    if (!omega && cfg->impute == SLFMM_IMPUTE_MEAN)
        prefetch_normal(c, cfg->seed, gf.n, (int)(cfg->k + cfg->oversampling));
    Step0 s0_own;
    Step0& s0 = pre ? pre->s0 : s0_own;
    if (!pre) step0(c, x, gf.n, d, cfg->lambda, cfg->scale_cov != 0, s0);
    SnpStd se_own, sf;
    SnpStd& se = pre ? pre->se : se_own;
    const SnpStd* sfp = &se;
    // NMF state kept alive for the passes that read its fills
    NmfModel nmf;
    DBuf<float> W32, He32, Hf32, Wpt32;
    if (cfg->impute == SLFMM_IMPUTE_NMF) {
        // NmfInRam on the estimation SNPs, NmfOnTheFly on the tested SNPs,
        // then the GWAS-phase CV (src/lib.rs:190-250)
        nmf_estimate(c, ge, cfg, nmf);
        const int k = nmf.k;
        DBuf<double> Wpt, Hf;
        nmf_pinv_t(c, nmf.W.get(), gf.n, k, Wpt, "W^T W for NMF pinv");
        to_f32(c, nmf.W.get(), gf.n, k, W32, k);
        to_f32(c, nmf.Ht.get(), ge.p, k, He32, k);
        to_f32(c, Wpt.get(), gf.n, k, Wpt32, k);
        std_fill(c, ge, cfg->norm, NmfFill{k, W32.get(), He32.get()}, se);
        SnpStd sm, rawm;
        std_mean(c, gf, SLFMM_NORM_EIGENSTRAT, sm);
        std_raw(c, gf, sm.mean.get(), rawm);
        nmf_h_meanfill(c, gf, rawm, Wpt.get(), k, Hf);
        to_f32(c, Hf.get(), gf.p, k, Hf32, k);
        std_fill(c, gf, cfg->norm, NmfFill{k, W32.get(), Hf32.get()}, sf);
        sfp = &sf;
        DBuf<double> part(std::max<uint64_t>(gf.p, 1) * 3, c.stream);
        launch_nmf_gwas_cv(c, gf, cfg->chunk_size ? cfg->chunk_size : 10000, cfg->seed, cfg->nmf_cv_rate, W32.get(),
                           Wpt32.get(), k, part.get());
        const std::vector<double> t = sum3(c, part, gf.p);
        const uint64_t cnt = (uint64_t)(t[2] + 0.5);
        if (res) {
            if (res->nmf_cv)
                for (size_t i = 0; i < nmf.cv.size(); ++i) res->nmf_cv[i] = nmf.cv[i];
            res->nmf_cv_mean = nmf.cv_mean;
            res->nmf_gwas_cv_mae = cnt ? t[0] / (double)cnt : 0.0;
            res->nmf_gwas_cv_mean_mae = cnt ? t[1] / (double)cnt : 0.0;
            res->nmf_gwas_cv_count = cnt;
        }
    } else {
        if (pre) {
            se.lut.alloc(ge.p * 4, c.stream);
            launch_lut_std(c, ge.p, se.mean.get(), se.scale.get(), se.lut.get());
        } else {
            std_mean(c, ge, cfg->norm, se);
        }
        if (&ge != &gf) {
            std_mean(c, gf, cfg->norm, sf);
            sfp = &sf;
        }
    }
    phase(c, "covariates, SNP statistics");
    DBuf<double> u_hat;
    const int K = (int)cfg->k, l = K + (int)cfg->oversampling;
    rsvd(c, ge, se, s0, K, l, (int)cfg->n_power_iter, cfg->seed, omega, u_hat, pre ? &pre->Z : nullptr);
    phase(c, "randomized SVD");
    if (res && res->u_hat) d2h(c, res->u_hat, u_hat.get(), gf.n * K);
    AssocOut out{res ? res->beta : nullptr, res ? res->tstat : nullptr, res ? res->pvalue : nullptr,
                 res ? res->r2 : nullptr, res ? res->gif_per_trait : nullptr, 0.0};
    assoc(c, gf, *sfp, s0, u_hat.get(), K, out);
    if (res) res->gif = out.gif;
}

// ---------------------------------------------------------------------------
// Rust "{:.6e}" formatting (src/testing.rs:780-797)
// ---------------------------------------------------------------------------
// C's %.6e re-spelt: exponent without '+' or zero padding (the slow path).
int format_exp6_printf(double v, char* buf, size_t len) {
    char tmp[48];
    snprintf(tmp, sizeof tmp, "%.6e", v);
    char* e = std::strchr(tmp, 'e');
    if (!e) return snprintf(buf, len, "%s", tmp);
    *e = '\0';
    const int ex = std::atoi(e + 1);
    return snprintf(buf, len, "%se%d", tmp, ex);
}

// Seven significant digits of |v| = m 2^e, correctly rounded (ties to even,
// like Rust's exact formatting, glibc's printf and Python's %): q =
// round(m 2^e 10^(6 - e10)) in exact 128-bit integer arithmetic, for decimal
// exponents whose power of five fits in 64 bits (|6 - e10| <= 27, which
// covers |v| in about [1e-21, 1e33]).  Returns false outside that range.
bool exp6_digits(uint64_t m, int e, int e10, uint64_t& q) {
    using u128 = unsigned __int128;
    static const uint64_t kPow5[28] = {
        1ull, 5ull, 25ull, 125ull, 625ull, 3125ull, 15625ull, 78125ull, 390625ull, 1953125ull, 9765625ull,
        48828125ull, 244140625ull, 1220703125ull, 6103515625ull, 30517578125ull, 152587890625ull,
        762939453125ull, 3814697265625ull, 19073486328125ull, 95367431640625ull, 476837158203125ull,
        2384185791015625ull, 11920928955078125ull, 59604644775390625ull, 298023223876953125ull,
        1490116119384765625ull, 7450580596923828125ull};
    const int sdec = 6 - e10;
    if (sdec > 27 || sdec < -27) return false;
    auto round_div = [](u128 num, u128 den, uint64_t& out) {
        u128 qq = num / den, rem = num - qq * den;
        const u128 twice = rem << 1;   // rem < den < 2^127
        if (twice > den || (twice == den && (qq & 1))) ++qq;
        if (qq > (u128)UINT64_MAX) return false;
        out = (uint64_t)qq;
        return true;
    };
    if (sdec >= 0) {
        const u128 x = (u128)m * kPow5[sdec];  // < 2^53 * 5^27 < 2^116
        const int k2 = e + sdec;               // value = x 2^k2
        if (k2 >= 0) {
            if (k2 > 40 || (x >> (127 - k2)) != 0) return false;
            const u128 r = x << k2;
            if (r > (u128)UINT64_MAX) return false;
            q = (uint64_t)r;
            return true;
        }
        const int sh = -k2;
        if (sh >= 127) {
            q = 0;
            return true;
        }
        u128 qq = x >> sh;
        const u128 rem = x - (qq << sh), half = (u128)1 << (sh - 1);
        if (rem > half || (rem == half && (qq & 1))) ++qq;
        if (qq > (u128)UINT64_MAX) return false;
        q = (uint64_t)qq;
        return true;
    }
    const uint64_t d5 = kPow5[-sdec];          // value = m 2^(e + sdec) / 5^-sdec
    const int k2 = e + sdec;
    if (k2 >= 0) {
        if (k2 > 70) return false;
        return round_div((u128)m << k2, d5, q);
    }
    if (-k2 > 64) {
        q = 0;
        return true;
    }
    return round_div(m, (u128)d5 << (-k2), q);
}

// Rust "{:.6e}": NaN, inf, -inf; otherwise d.dddddde<exp> with the sign of
// negative values (and of -0.0), no '+' and no zero padding in the exponent.
int format_exp6(double v, char* buf, size_t len) {
    if (std::isnan(v)) return snprintf(buf, len, "NaN");
    if (std::isinf(v)) return snprintf(buf, len, v > 0 ? "inf" : "-inf");
    if (len < 32) return format_exp6_printf(v, buf, len);
    uint64_t bits;
    std::memcpy(&bits, &v, sizeof bits);
    const bool neg = (bits >> 63) != 0;
    const int bexp = (int)((bits >> 52) & 0x7ff);
    uint64_t m = bits & ((1ull << 52) - 1);
    int e;
    if (bexp == 0) {
        e = -1074;
    } else {
        m |= 1ull << 52;
        e = bexp - 1075;
    }
    char* o = buf;
    if (neg) *o++ = '-';
    if (m == 0) {
        std::memcpy(o, "0.000000e0", 10);
        return (int)(o - buf) + 10;
    }
    // floor(log10 |v|) is floor(log10(2) floor(log2 |v|)) or one more: start
    // at the lower estimate and step up while the rounded digits reach 10^7
    const int l2 = e + 63 - __builtin_clzll(m);           // floor(log2 |v|)
    int e10 = (int)std::floor(l2 * 0.30102999566398120);
    uint64_t q = 0;
    for (int attempt = 0;; ++attempt) {
        if (attempt > 3 || !exp6_digits(m, e, e10, q)) return format_exp6_printf(v, buf, len);
        if (q >= 10000000ull) {
            ++e10;
            continue;
        }
        if (q < 1000000ull) return format_exp6_printf(v, buf, len);
        break;
    }
    char dig[7];
    for (int i = 6; i >= 0; --i) {
        dig[i] = (char)('0' + q % 10);
        q /= 10;
    }
    *o++ = dig[0];
    *o++ = '.';
    std::memcpy(o, dig + 1, 6);
    o += 6;
    *o++ = 'e';
    int x = e10;
    if (x < 0) {
        *o++ = '-';
        x = -x;
    }
    char eb[8];
    int n = 0;
    do {
        eb[n++] = (char)('0' + x % 10);
        x /= 10;
    } while (x);
    while (n) *o++ = eb[--n];
    return (int)(o - buf);
}

}  // namespace

bool write_tsv_body(FILE* f, uint64_t p, uint32_t d, const char* const* chrom, const uint64_t* pos,
                    const char* const* snp_id, const char* const* cov_names, const slfmm_results* res,
                    int n_threads);
}  // namespace slfmm

// ===========================================================================
// C ABI
// ===========================================================================
using namespace slfmm;

#define API_TRY try {
#define API_CATCH(ctxp)                                                        \
    }                                                                          \
    catch (const slfmm::Error& e) {                                            \
        if (ctxp) (ctxp)->last_error = e.what();                               \
        return e.code;                                                         \
    }                                                                          \
    catch (const std::bad_alloc&) {                                            \
        if (ctxp) (ctxp)->last_error = "host allocation failed";               \
        return SLFMM_ERR_NOMEM;                                                \
    }                                                                          \
    catch (const std::exception& e) {                                          \
        if (ctxp) (ctxp)->last_error = e.what();                               \
        return SLFMM_ERR_CUDA;                                                 \
    }                                                                          \
    return SLFMM_OK;

extern "C" {

namespace slfmm {
namespace {
// device checks, streams and the memory pool of a context
void ctx_open(Ctx& c, int device, int precision, int verbose, cudaStream_t stream) {
    int ndev = 0;
    SLFMM_CUDA(cudaGetDeviceCount(&ndev));
    SLFMM_REQUIRE(device >= 0 && device < ndev, SLFMM_ERR_CUDA, "no such CUDA device");
    SLFMM_CUDA(cudaSetDevice(device));
    cudaDeviceProp prop{};
    SLFMM_CUDA(cudaGetDeviceProperties(&prop, device));
    SLFMM_REQUIRE(prop.major == 10 && prop.minor == 3, SLFMM_ERR_CUDA,
                  std::string("schnelgpu is built for sm_103a (GB300); device is ") + prop.name);
    c.device = device;
    c.sm_count = prop.multiProcessorCount;
    c.precision = precision;
    c.verbose = verbose;
    if (stream) {
        c.stream = stream;
    } else {
        SLFMM_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
        c.own_stream = true;
    }
    SLFMM_CUDA(cudaStreamCreateWithFlags(&c.copy_stream, cudaStreamNonBlocking));
    cudaMemPool_t pool;
    SLFMM_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
    uint64_t thr = UINT64_MAX;
    SLFMM_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
    c.dev_flags.alloc(4, c.stream);
    c.dev_flags.zero();
    // slfmm_gif_noalloc allocates nothing after this point on this device
    gif_noalloc_prepare(device);
    SLFMM_CUDA(cudaStreamSynchronize(c.stream));
}

void ctx_close(Ctx& c) {
    cudaSetDevice(c.device);
    clear_phase_marks(c);
    c.dev_flags.release();
    if (c.stream) cudaStreamSynchronize(c.stream);
    if (c.copy_stream) cudaStreamDestroy(c.copy_stream);
    if (c.own_stream && c.stream) cudaStreamDestroy(c.stream);
    c.copy_stream = nullptr;
    c.stream = nullptr;
}
}  // namespace
}  // namespace slfmm

int slfmm_create(int device, const slfmm_opts* opts, slfmm_ctx** out) {
    if (!out) return SLFMM_ERR_BAD_ARG;
    *out = nullptr;
    if (opts && opts->rng != SLFMM_RNG_COUNTER && opts->rng != SLFMM_RNG_CHACHA8) return SLFMM_ERR_BAD_ARG;
    slfmm_ctx* c = new (std::nothrow) slfmm_ctx();
    if (!c) return SLFMM_ERR_NOMEM;
    try {
        ctx_open(*c, device, opts ? opts->precision : SLFMM_PREC_SPLIT_FP8, opts ? opts->verbose : 0,
                 opts ? (cudaStream_t)opts->stream : nullptr);
        const char* at = std::getenv("SLFMM_AUTOTUNE");
        c->autotune = (opts && opts->autotune) || (at && at[0] == '1');
        c->rng = opts ? opts->rng : SLFMM_RNG_CHACHA8;
    } catch (const slfmm::Error& e) {
        fprintf(stderr, "schnelgpu: %s\n", e.what());
        const int code = e.code;
        delete c;
        return code;
    }
    *out = c;
    return SLFMM_OK;
}

void slfmm_destroy(slfmm_ctx* c) {
    if (!c) return;
    ctx_close(*c);
    delete c;
}

const char* slfmm_last_error(const slfmm_ctx* c) { return c ? c->last_error.c_str() : "null context"; }
uint64_t slfmm_launch_count(const slfmm_ctx* c) { return c ? c->launches : 0; }
void* slfmm_stream(const slfmm_ctx* c) { return c ? (void*)c->stream : nullptr; }

int slfmm_bed_validate(const char* bed_path, uint64_t n_samples, uint64_t n_snps, uint8_t* payload_out,
                       char* err, size_t err_len) {
    auto fail = [&](int code, const std::string& m) {
        if (err && err_len) snprintf(err, err_len, "%s", m.c_str());
        return code;
    };
    if (!bed_path) return fail(SLFMM_ERR_BAD_ARG, "null path");
    std::ifstream f(bed_path, std::ios::binary | std::ios::ate);
    if (!f) return fail(SLFMM_ERR_IO, std::string("Failed to open ") + bed_path);
    const uint64_t size = (uint64_t)f.tellg();
    f.seekg(0);
    unsigned char magic[3] = {0, 0, 0};
    if (size >= 3) f.read((char*)magic, 3);
    if (size < 3 || magic[0] != 0x6C || magic[1] != 0x1B || magic[2] != 0x01)
        return fail(SLFMM_ERR_BAD_BED, std::string("Invalid .bed file (bad magic bytes): ") + bed_path);
    const uint64_t bps = (n_samples + 3) / 4;
    const uint64_t expected = 3 + bps * n_snps;
    if (size != expected)
        return fail(SLFMM_ERR_BAD_BED, "BED file size mismatch: expected " + std::to_string(expected) + " bytes (" +
                                           std::to_string(n_samples) + " samples x " + std::to_string(n_snps) +
                                           " SNPs), got " + std::to_string(size));
    if (payload_out) {
        f.read((char*)payload_out, (std::streamsize)(bps * n_snps));
        if (!f) return fail(SLFMM_ERR_IO, std::string("short read from ") + bed_path);
    }
    return SLFMM_OK;
}

int slfmm_geno_upload(slfmm_ctx* c, const uint8_t* packed, uint64_t n_physical, uint64_t n_snps,
                      const uint64_t* sample_keep, uint64_t n_keep, const slfmm_subset* snps, slfmm_geno** out) {
    if (!c || !out) return SLFMM_ERR_BAD_ARG;
    *out = nullptr;
    API_TRY
    SLFMM_CUDA(cudaSetDevice(c->device));
    std::unique_ptr<slfmm_geno> g(new slfmm_geno());
    if (!snps || snps->kind == SLFMM_SUBSET_ALL) {
        upload_geno(*c, *g, packed, n_physical, n_snps, sample_keep, n_keep, nullptr);
    } else {
        const std::vector<uint64_t> idx = subset_indices(snps, n_snps);
        upload_geno(*c, *g, packed, n_physical, n_snps, sample_keep, n_keep, &idx);
    }
    *out = g.release();
    API_CATCH(c)
}

int slfmm_geno_free(slfmm_ctx* c, slfmm_geno* g) {
    if (!g) return SLFMM_OK;
    if (c) cudaSetDevice(c->device);
    // the context that allocated the buffers may already be destroyed: free on
    // the given context's stream, or on the legacy default stream
    g->rebind(c ? c->stream : (cudaStream_t)0);
    delete g;
    if (!c) cudaDeviceSynchronize();
    return SLFMM_OK;
}

uint64_t slfmm_geno_n_samples(const slfmm_geno* g) { return g ? g->n : 0; }
uint64_t slfmm_geno_n_snps(const slfmm_geno* g) { return g ? g->p : 0; }

int slfmm_decode_stats(slfmm_ctx* c, const slfmm_geno* g, int norm, int32_t* counts4, double* mean,
                       double* scale, double* tss) {
    if (!c || !g) return SLFMM_ERR_BAD_ARG;
    API_TRY
    SLFMM_CUDA(cudaSetDevice(c->device));
    SLFMM_REQUIRE(norm == SLFMM_NORM_CENTER_ONLY || norm == SLFMM_NORM_EIGENSTRAT, SLFMM_ERR_BAD_ARG,
                  "unknown normalisation");
    SnpStd s;
    std_mean(*c, *g, norm, s);
    if (counts4) d2h(*c, counts4, g->counts.get(), g->p * 4);
    if (mean) d2h(*c, mean, s.mean.get(), g->p);
    if (scale) d2h(*c, scale, s.scale.get(), g->p);
    if (tss) d2h(*c, tss, s.tss.get(), g->p);
    sync(*c);
    API_CATCH(c)
}

int slfmm_decode_chunk(slfmm_ctx* c, const slfmm_geno* g, uint64_t snp0, uint64_t ncols, int norm, double* out) {
    if (!c || !g || !out) return SLFMM_ERR_BAD_ARG;
    API_TRY
    SLFMM_CUDA(cudaSetDevice(c->device));
    SLFMM_REQUIRE(snp0 <= g->p && ncols <= g->p - snp0, SLFMM_ERR_BAD_ARG, "SNP range out of bounds");
    SLFMM_REQUIRE(norm == SLFMM_NORM_CENTER_ONLY || norm == SLFMM_NORM_EIGENSTRAT, SLFMM_ERR_BAD_ARG,
                  "unknown normalisation");
    SnpStd s;
    std_mean(*c, *g, norm, s);
    DBuf<double> o(std::max<uint64_t>(g->n * ncols, 1), c->stream);
    launch_decode_chunk(*c, *g, snp0, ncols, s.mean.get(), s.scale.get(), o.get());
    d2h(*c, out, o.get(), g->n * ncols);
    sync(*c);
    API_CATCH(c)
}

int slfmm_center_covariates(slfmm_ctx* c, const double* x, uint64_t n, uint32_t d, int scale, double* out) {
    if (!c || !x || !out) return SLFMM_ERR_BAD_ARG;
    API_TRY
    SLFMM_CUDA(cudaSetDevice(c->device));
    DBuf<double> xs = upload(*c, x, n * d);
    center_covariates_dev(*c, xs.get(), n, (int)d, scale != 0);
    d2h(*c, out, xs.get(), n * d);
    sync(*c);
    API_CATCH(c)
}

int slfmm_generate_omega(slfmm_ctx* c, uint64_t seed, uint64_t n, uint32_t l, double* out) {
    if (!c || !out) return SLFMM_ERR_BAD_ARG;
    API_TRY
    SLFMM_CUDA(cudaSetDevice(c->device));
    SLFMM_REQUIRE(l <= 4096, SLFMM_ERR_BAD_ARG, "sketch width above 4096");
    DBuf<double> o(std::max<uint64_t>(n * l, 1), c->stream);
    draw_normal(*c, seed, n, (int)l, o.get());
    d2h(*c, out, o.get(), n * l);
    sync(*c);
    API_CATCH(c)
}

int slfmm_small_eigh(slfmm_ctx* c, const double* a_host, uint32_t a, double* v_out, double* sig_out) {
    if (!c || !a_host || !v_out || !sig_out || a == 0) return SLFMM_ERR_BAD_ARG;
    API_TRY
    SLFMM_CUDA(cudaSetDevice(c->device));
    SLFMM_REQUIRE(a <= (uint32_t)kMaxDesign, SLFMM_ERR_BAD_ARG,
                  "matrix wider than " + std::to_string(kMaxDesign));
    DBuf<double> A = upload(*c, a_host, (size_t)a * a), V((size_t)a * a, c->stream), sig(a, c->stream);
    launch_jacobi_svd(*c, A.get(), (int)a, V.get(), sig.get());
    d2h(*c, v_out, V.get(), (size_t)a * a);
    d2h(*c, sig_out, sig.get(), a);
    sync(*c);
    API_CATCH(c)
}

int slfmm_estimate_factors(slfmm_ctx* c, const slfmm_geno* y_est, const double* x, uint32_t d,
                           const slfmm_config* cfg, const double* omega, double* u_hat) {
    if (!c || !y_est || !x || !u_hat) return SLFMM_ERR_BAD_ARG;
    API_TRY
    SLFMM_CUDA(cudaSetDevice(c->device));
    check_cfg(cfg);
    SLFMM_REQUIRE(cfg->impute == SLFMM_IMPUTE_MEAN, SLFMM_ERR_BAD_ARG, "estimate_factors uses mean imputation");
    Step0 s0;
    step0(*c, x, y_est->n, (int)d, cfg->lambda, cfg->scale_cov != 0, s0);
    SnpStd st;
    std_mean(*c, *y_est, cfg->norm, st);
    DBuf<double> u;
    const int K = (int)cfg->k;
    rsvd(*c, *y_est, st, s0, K, K + (int)cfg->oversampling, (int)cfg->n_power_iter, cfg->seed, omega, u);
    d2h(*c, u_hat, u.get(), y_est->n * K);
    sync(*c);
    API_CATCH(c)
}

int slfmm_test_associations(slfmm_ctx* c, const slfmm_geno* y_full, const double* x, uint32_t d,
                            const double* u_hat, const slfmm_config* cfg, slfmm_results* res) {
    if (!c || !y_full || !x || !u_hat || !res) return SLFMM_ERR_BAD_ARG;
    API_TRY
    SLFMM_CUDA(cudaSetDevice(c->device));
    check_cfg(cfg);
    SLFMM_REQUIRE(cfg->impute == SLFMM_IMPUTE_MEAN, SLFMM_ERR_BAD_ARG, "test_associations uses mean imputation");
    Step0 s0;
    step0(*c, x, y_full->n, (int)d, cfg->lambda, cfg->scale_cov != 0, s0);
    SnpStd st;
    std_mean(*c, *y_full, cfg->norm, st);
    const int K = (int)cfg->k;
    DBuf<double> u = upload(*c, u_hat, y_full->n * K);
    AssocOut out{res->beta, res->tstat, res->pvalue, res->r2, res->gif_per_trait, 0.0};
    assoc(*c, *y_full, st, s0, u.get(), K, out);
    res->gif = out.gif;
    if (res->u_hat && res->u_hat != u_hat) std::memcpy(res->u_hat, u_hat, y_full->n * K * sizeof(double));
    API_CATCH(c)
}

int slfmm_fit(slfmm_ctx* c, const slfmm_geno* y_est, const slfmm_geno* y_full, const double* x, uint32_t d,
              const slfmm_config* cfg, const double* omega, slfmm_results* res) {
    if (!c || !y_full || !x) return SLFMM_ERR_BAD_ARG;
    API_TRY
    SLFMM_CUDA(cudaSetDevice(c->device));
    fit_impl(*c, y_est ? *y_est : *y_full, *y_full, x, (int)d, cfg, omega, res);
    API_CATCH(c)
}

int slfmm_fit_host(slfmm_ctx* c, const uint8_t* packed, uint64_t n_physical, uint64_t n_snps,
                   const uint64_t* sample_keep, uint64_t n_keep, const slfmm_subset* est, const double* x,
                   uint32_t d, const slfmm_config* cfg, const double* omega, slfmm_results* res) {
    if (!c || !packed || !x) return SLFMM_ERR_BAD_ARG;
    API_TRY
    SLFMM_CUDA(cudaSetDevice(c->device));
    Geno full, sub;
    const bool all = !est || est->kind == SLFMM_SUBSET_ALL;
    // with every SNP in the estimation, the sketch pass runs under the upload
    Presketch ps;
    phase(*c, "", true);
    if (cfg && !omega && cfg->impute == SLFMM_IMPUTE_MEAN)
        prefetch_normal(*c, cfg->seed, sample_keep ? n_keep : n_physical, (int)(cfg->k + cfg->oversampling));
    const bool pre = all && cfg && presketch_eligible(*c, sample_keep ? n_keep : n_physical, n_snps, x, (int)d,
                                                      cfg, omega, ps);
    upload_geno(*c, full, packed, n_physical, n_snps, sample_keep, n_keep, nullptr,
                pre ? &ps : nullptr);
    if (pre) {
        const int e = fetch(*c, ps.err.get(), 1)[0];
        if (e) throw_tc8_timeout(e);
        ps.finish(*c, full);
    }
    phase(*c, pre ? "covariates; upload with the sketch pass" : "upload");
    const Geno* ge = &full;
    if (!all) {
        const std::vector<uint64_t> est_idx = subset_indices(est, n_snps);
        upload_geno(*c, sub, packed, n_physical, n_snps, sample_keep, n_keep, &est_idx);
        ge = &sub;
    }
    fit_impl(*c, *ge, full, x, (int)d, cfg, omega, res, pre ? &ps : nullptr);
    API_CATCH(c)
}

namespace slfmm {
namespace {
// The samples `keep` (ascending or not, each < src.n) of a resident matrix as
// a new resident matrix: the padded rows are re-packed on the device from the
// resident copy (BedFile::subset_samples, src/bed.rs:155-159), then counted.
// Tile-major copies and missing-call lists are built on first use.
void geno_subset_samples(Ctx& c, const Geno& src, const std::vector<uint64_t>& keep, Geno& dst) {
    SLFMM_REQUIRE(!keep.empty(), SLFMM_ERR_BAD_ARG, "empty sample subset");
    std::vector<uint32_t> k32(keep.size());
    for (size_t i = 0; i < keep.size(); ++i) {
        SLFMM_REQUIRE(keep[i] < src.n, SLFMM_ERR_BAD_ARG, "sample index out of range");
        k32[i] = (uint32_t)keep[i];
    }
    DBuf<uint32_t> keep_d = upload(c, k32.data(), k32.size());
    dst.n = keep.size();
    dst.p = src.p;
    dst.stride = round_up(ceil_div(dst.n, 4), 128);
    dst.packed.alloc(std::max<uint64_t>(dst.p, 1) * dst.stride, c.stream);
    dst.counts.alloc(std::max<uint64_t>(dst.p, 1) * 4, c.stream);
    launch_repack(c, src.packed.get(), src.p, src.stride, src.n, keep_d.get(), dst.n, dst.packed.get(), dst.stride);
    launch_snp_counts(c, dst, nullptr);
    sync(c);
}

// Whether a split-FP8 mean-imputation fit of an n x p matrix with one
// covariate runs on the tile-major copies alone: every column pass (the RSVD
// sketch width) has an indicator plan, and the row passes take their
// missing-call lists from the SNP-major tiles, so no pass needs the
// row-major copy.
bool tiles_only_fit(const Ctx& c, const slfmm_config* cfg, uint64_t n, uint64_t p) {
    if (c.precision != SLFMM_PREC_SPLIT_FP8 || cfg->impute != SLFMM_IMPUTE_MEAN) return false;
    const int l = (int)cfg->k + (int)cfg->oversampling;
    if (l > 64) return false;
    (void)p;
    const Fp8Plan col = fp8_plan(pad16(l), true, ceil_div(n, 128));
    return col.ok && col.n_ind != 0;
}

// One trait of slfmm_fit_traits on context c: its sample subset taken from
// the resident matrix g on the device, then a d = 1 fit.
void fit_trait(Ctx& c, const Geno& g, const double* y, const uint8_t* masks, uint32_t n_traits, uint32_t t,
               const slfmm_config* cfg, slfmm_results* res) {
    std::vector<uint64_t> keep;
    std::vector<double> xt;
    for (uint64_t i = 0; i < g.n; ++i)
        if (masks[i * n_traits + t]) {
            keep.push_back(i);
            xt.push_back(y[i * n_traits + t]);
        }
    try {
        SLFMM_REQUIRE(!keep.empty(), SLFMM_ERR_BAD_ARG, "no samples");
        Geno sub;
        phase(c, "", true);
        if (tiles_only_fit(c, cfg, keep.size(), g.p)) {
            std::vector<uint32_t> k32(keep.begin(), keep.end());
            DBuf<uint32_t> keep_d = upload(c, k32.data(), k32.size());
            tiles_subset_samples(c, g, keep_d.get(), keep.size(), sub);
            sync(c);
        } else {
            geno_subset_samples(c, g, keep, sub);
        }
        phase(c, "trait sample subset");
        fit_impl(c, sub, sub, xt.data(), 1, cfg, nullptr, &res[t]);
    } catch (const Error& e) {
        throw Error(e.code, "trait " + std::to_string(t) + ": " + e.what());
    }
}

// one problem of slfmm_fit_many on a worker's context (the body of
// slfmm_fit_host with every SNP in the estimation)
void fit_problem(Ctx& c, const slfmm_problem& pr) {
    SLFMM_REQUIRE(pr.packed && pr.x && pr.cfg, SLFMM_ERR_BAD_ARG, "null problem input");
    Geno full;
    Presketch ps;
    const bool pre = presketch_eligible(c, pr.n_physical, pr.n_snps, pr.x, (int)pr.d, pr.cfg, pr.omega, ps);
    upload_geno(c, full, pr.packed, pr.n_physical, pr.n_snps, nullptr, 0, nullptr,
                pre ? &ps : nullptr);
    if (pre) {
        const int e = fetch(c, ps.err.get(), 1)[0];
        if (e) throw_tc8_timeout(e);
        ps.finish(c, full);
    }
    fit_impl(c, full, full, pr.x, (int)pr.d, pr.cfg, pr.omega, pr.res, pre ? &ps : nullptr);
}
}  // namespace
}  // namespace slfmm

int slfmm_fit_traits(slfmm_ctx* c, const slfmm_geno* g, const double* y, const uint8_t* masks,
                     uint32_t n_traits, const slfmm_config* cfg, slfmm_results* res) {
    if (!c || !g || !y || !masks || !cfg || !res) return SLFMM_ERR_BAD_ARG;
    API_TRY
    SLFMM_CUDA(cudaSetDevice(c->device));
    SLFMM_REQUIRE(n_traits >= 1, SLFMM_ERR_BAD_ARG, "no traits");
    for (uint32_t t = 0; t < n_traits; ++t) fit_trait(*c, *g, y, masks, n_traits, t, cfg, res);
    API_CATCH(c)
}

int slfmm_fit_many(slfmm_ctx* c, const slfmm_problem* problems, uint32_t n_problems, uint32_t n_streams,
                   int* status) {
    if (!c || (!problems && n_problems)) return SLFMM_ERR_BAD_ARG;
    API_TRY
    SLFMM_CUDA(cudaSetDevice(c->device));
    if (n_problems == 0) return SLFMM_OK;
    // default 8 workers: on the 64-problem set, 206-210 ms per step against
    // 222 ms with 4 and 271 ms with 2 (16: 207 ms)
    const uint32_t workers = std::max<uint32_t>(1, std::min(n_streams ? n_streams : 8u, n_problems));
    std::vector<int> st(n_problems, SLFMM_OK);
    std::vector<std::string> msg(n_problems);
    std::atomic<uint32_t> next{0};
    // each worker owns a context (its own streams) on the same device and
    // takes problems in order; kernels of different workers run concurrently
    auto work = [&]() {
        Ctx w;
        try {
            ctx_open(w, c->device, c->precision, 0, nullptr);
            w.autotune = c->autotune;
            w.rng = c->rng;
        } catch (const Error& e) {
            for (uint32_t i = next.fetch_add(1); i < n_problems; i = next.fetch_add(1)) {
                st[i] = e.code;
                msg[i] = e.what();
            }
            return;
        }
        for (uint32_t i = next.fetch_add(1); i < n_problems; i = next.fetch_add(1)) {
            try {
                fit_problem(w, problems[i]);
            } catch (const Error& e) {
                st[i] = e.code;
                msg[i] = e.what();
            } catch (const std::bad_alloc&) {
                st[i] = SLFMM_ERR_NOMEM;
                msg[i] = "host allocation failed";
            } catch (const std::exception& e) {
                st[i] = SLFMM_ERR_CUDA;
                msg[i] = e.what();
            }
        }
        ctx_close(w);
    };
    std::vector<std::thread> pool;
    for (uint32_t k = 1; k < workers; ++k) pool.emplace_back(work);
    work();
    for (auto& th : pool) th.join();
    int first = SLFMM_OK;
    for (uint32_t i = 0; i < n_problems; ++i) {
        if (status) status[i] = st[i];
        if (st[i] != SLFMM_OK && first == SLFMM_OK) {
            first = st[i];
            c->last_error = "problem " + std::to_string(i) + ": " + msg[i];
        }
    }
    return first;
    API_CATCH(c)
}

int slfmm_simulate(slfmm_ctx* c, uint64_t n, uint64_t p, uint32_t n_pop, const float* admix, double fst,
                   double f_lo, double f_hi, double miss_rate, double inbreeding, uint64_t seed, slfmm_geno** out) {
    if (!c || !admix || !out) return SLFMM_ERR_BAD_ARG;
    *out = nullptr;
    API_TRY
    SLFMM_CUDA(cudaSetDevice(c->device));
    SLFMM_REQUIRE(n > 0 && p > 0 && n < (1ull << 31), SLFMM_ERR_BAD_ARG, "bad cohort shape");
    std::unique_ptr<slfmm_geno> g(new slfmm_geno());
    g->n = n;
    g->p = p;
    g->stride = round_up(ceil_div(n, 4), 128);
    g->packed.alloc(p * g->stride, c->stream);
    g->counts.alloc(p * 4, c->stream);
    DBuf<float> q = upload(*c, admix, n * n_pop);
    launch_simulate(*c, n, p, (int)n_pop, q.get(), fst, f_lo, f_hi, miss_rate, inbreeding, seed, g->packed.get(),
                    g->stride);
    launch_snp_counts(*c, *g, nullptr);
    sync(*c);
    *out = g.release();
    API_CATCH(c)
}

int slfmm_geno_download(slfmm_ctx* c, const slfmm_geno* g, uint8_t* packed_out) {
    if (!c || !g || !packed_out) return SLFMM_ERR_BAD_ARG;
    API_TRY
    SLFMM_CUDA(cudaSetDevice(c->device));
    const uint64_t bps = ceil_div(g->n, 4);
    if (g->p)
        SLFMM_CUDA(cudaMemcpy2DAsync(packed_out, bps, g->packed.get(), g->stride, bps, g->p, cudaMemcpyDeviceToHost,
                                     c->stream));
    sync(*c);
    API_CATCH(c)
}

int slfmm_host_alloc(size_t bytes, void** out) {
    if (!out) return SLFMM_ERR_BAD_ARG;
    *out = nullptr;
    if (bytes == 0) return SLFMM_OK;
    cudaError_t e = cudaMallocHost(out, bytes);
    if (e != cudaSuccess) {
        *out = nullptr;
        return e == cudaErrorMemoryAllocation ? SLFMM_ERR_NOMEM : SLFMM_ERR_CUDA;
    }
    return SLFMM_OK;
}

int slfmm_host_free(void* p) {
    if (p && cudaFreeHost(p) != cudaSuccess) return SLFMM_ERR_CUDA;
    return SLFMM_OK;
}

int slfmm_profile_enable(slfmm_ctx* c, int on) {
    if (!c) return SLFMM_ERR_BAD_ARG;
    API_TRY
    profile_collect(*c);
    c->prof.clear();
    clear_phase_marks(*c);
    c->profiling = on != 0;
    API_CATCH(c)
}

int slfmm_profile_read(slfmm_ctx* c, const char* kernel, double* total_ms, uint64_t* launches, double* bytes,
                       double* flops) {
    if (!c || !kernel) return SLFMM_ERR_BAD_ARG;
    API_TRY
    profile_collect(*c);
    auto it = c->prof.find(kernel);
    const ProfRec empty;
    const ProfRec& r = it == c->prof.end() ? empty : it->second;
    if (total_ms) *total_ms = r.ms;
    if (launches) *launches = r.launches;
    if (bytes) *bytes = r.bytes;
    if (flops) *flops = r.flops;
    API_CATCH(c)
}

int slfmm_debug_expire_next_wait(slfmm_ctx* c, uint64_t cycles) {
    if (!c || cycles == 0 || cycles > (uint64_t)kWaitCyclesMax) return SLFMM_ERR_BAD_ARG;
    c->expire_next_wait = (long long)cycles;
    return SLFMM_OK;
}

int slfmm_phase_count(const slfmm_ctx* c) {
    return c && c->phase_marks.size() > 1 ? (int)c->phase_marks.size() - 1 : 0;
}

int slfmm_phase_read(slfmm_ctx* c, int i, char* name, size_t name_len, double* device_ms, double* host_ms) {
    if (!c || i < 0 || (size_t)i + 1 >= c->phase_marks.size()) return SLFMM_ERR_BAD_ARG;
    API_TRY
    const auto& a = c->phase_marks[(size_t)i];
    const auto& b = c->phase_marks[(size_t)i + 1];
    if (name && name_len) snprintf(name, name_len, "%s", b.name.c_str());
    if (device_ms) {
        float ms = 0.f;
        SLFMM_CUDA(cudaEventSynchronize(b.ev));
        SLFMM_CUDA(cudaEventElapsedTime(&ms, a.ev, b.ev));
        *device_ms = ms;
    }
    if (host_ms) *host_ms = b.host_ms - a.host_ms;
    API_CATCH(c)
}

int slfmm_contract_raw(slfmm_ctx* c, const slfmm_geno* g, int flags, const double* w_host, uint32_t w,
                       float* out) {
    if (!c || !g || !w_host || !out) return SLFMM_ERR_BAD_ARG;
    API_TRY
    SLFMM_CUDA(cudaSetDevice(c->device));
    const bool transposed = (flags & 1) != 0, with_ind = (flags & 2) != 0;
    const int wp = pad16((int)w);
    SLFMM_REQUIRE(wp <= kMaxW, SLFMM_ERR_BAD_ARG, "operand wider than 128 columns");
    const uint64_t K = transposed ? g->p : g->n, rows = transposed ? g->n : g->p;
    const uint64_t K_pad = round_up(K, 256);
    DBuf<double> Wd = upload(*c, w_host, K * w);
    DBuf<float> o(std::max<uint64_t>(rows, 1) * wp, c->stream);
    if (c->precision == SLFMM_PREC_SPLIT_FP8) {
        const TileView tv = build_tiles(*c, *g, transposed);
        const uint64_t tiles = ceil_div(rows, 128);
        const Fp8Plan pl = fp8_plan(wp, with_ind, tiles, true);
        SLFMM_REQUIRE(pl.ok || !with_ind, SLFMM_ERR_BAD_ARG, "indicator operand too wide for one launch");
        const int cb = pl.ok ? wp : 64;
        for (int c0 = 0; c0 < (int)w; c0 += cb) {
            const int wb = std::min(cb, (int)w - c0), bp = std::min(cb, pad16(wb));
            const Fp8Plan pb = bp == wp ? pl : fp8_plan(bp, false, tiles);
            DBuf<uint8_t> B((uint64_t)pb.n_total * K_pad, c->stream);
            DBuf<float> isc(pb.n_total, c->stream);
            launch_fp8_terms_f64(*c, Wd.get() + c0, (int)w, K, wb, bp, K_pad, nullptr, 4, 0, (int)pb.n_total,
                                 B.get(), isc.get());
            if (with_ind && !pb.ind_shared)
                launch_fp8_terms_f64(*c, Wd.get() + c0, (int)w, K, wb, bp, K_pad, nullptr, 3, (int)pb.n_main,
                                     (int)pb.n_total, B.get(), isc.get());
            launch_tc8_rows(*c, pb, tv, rows, K, B.get(), isc.get(), K_pad, 0, nullptr, nullptr, nullptr,
                            o.get() + c0, wp, 1, 0);
        }
    } else {
        SLFMM_REQUIRE(!with_ind, SLFMM_ERR_BAD_ARG, "indicator operand needs the split-FP8 precision");
        if (transposed) build_transposed(*c, *g);
        const uint8_t* pk = transposed ? g->packedT.get() : g->packed.get();
        const uint64_t st = transposed ? g->strideT : g->stride;
        DBuf<__nv_bfloat16> bs(2 * (uint64_t)wp * K_pad, c->stream);
        launch_split_bf16_f64(*c, Wd.get(), (int)w, K, (int)w, wp, K_pad, nullptr, bs.get());
        launch_tc_rows(*c, pk, st, rows, K, bs.get(), K_pad, wp, o.get(), wp, 1, 0);
    }
    SLFMM_CUDA(cudaMemcpy2DAsync(out, w * sizeof(float), o.get(), wp * sizeof(float), w * sizeof(float), rows,
                                 cudaMemcpyDeviceToHost, c->stream));
    sync(*c);
    API_CATCH(c)
}

int slfmm_gif_noalloc(slfmm_ctx* c, const float* t_dev, uint64_t p, uint32_t d, double* gif_dev) {
    if (!c) return SLFMM_ERR_BAD_ARG;
    API_TRY
    SLFMM_CUDA(cudaSetDevice(c->device));
    SLFMM_REQUIRE(d <= (uint32_t)kGifNoAllocMaxTraits, SLFMM_ERR_BAD_ARG,
                  "slfmm_gif_noalloc handles at most " + std::to_string(kGifNoAllocMaxTraits) +
                      " traits (its static histogram holds " + std::to_string(kGifNoAllocMaxTraits) +
                      " x 100000 counters); got " + std::to_string(d));
    launch_gif_noalloc(*c, t_dev, p, (int)d, gif_dev);
    API_CATCH(c)
}

int slfmm_format_exp6(double v, char* buf, size_t len) { return format_exp6(v, buf, len); }

int slfmm_write_tsv(const char* path, uint64_t p, uint32_t d, const char* const* chrom, const uint64_t* pos,
                    const char* const* snp_id, const char* const* cov_names, const slfmm_results* res,
                    int n_threads) {
    if (!path || !res || !chrom || !pos || !snp_id || !cov_names) return SLFMM_ERR_BAD_ARG;
    if (!res->pvalue || !res->beta || !res->tstat || !res->r2) return SLFMM_ERR_BAD_ARG;
    FILE* f = std::fopen(path, "wb");
    if (!f) return SLFMM_ERR_IO;
    int rc = SLFMM_OK;
    try {
        rc = write_tsv_body(f, p, d, chrom, pos, snp_id, cov_names, res, n_threads) ? SLFMM_OK : SLFMM_ERR_IO;
    } catch (const std::bad_alloc&) {
        rc = SLFMM_ERR_NOMEM;
    } catch (...) {
        rc = SLFMM_ERR_IO;
    }
    if (std::fclose(f) != 0 && rc == SLFMM_OK) rc = SLFMM_ERR_IO;
    return rc;
}

}  // extern "C"

namespace slfmm {
// the TSV rows after the file is open: header, then blocks of rows formatted
// on n_threads threads and written in order
// Rows [r0, r1) of <out>.tsv appended to s: chr, pos, snp_id, then
// p/beta/t per covariate and the three r2 columns, each "{:.6e}".  The
// buffer is sized from the row bound (14 characters per number at most).
void format_tsv_rows(uint64_t r0, uint64_t r1, uint32_t d, const char* const* chrom, const uint64_t* pos,
                     const char* const* snp_id, const slfmm_results* res, std::string& s) {
    size_t cap = 0;
    for (uint64_t i = r0; i < r1; ++i) cap += std::strlen(chrom[i]) + std::strlen(snp_id[i]);
    cap += (r1 - r0) * (24 + (size_t)(3 * d + 3) * 16);
    s.resize(cap);
    char* o = &s[0];
    for (uint64_t i = r0; i < r1; ++i) {
        for (const char* c = chrom[i]; *c; ++c) *o++ = *c;
        *o++ = '\t';
        char dig[24];
        int n = 0;
        uint64_t x = pos[i];
        do {
            dig[n++] = (char)('0' + x % 10);
            x /= 10;
        } while (x);
        while (n) *o++ = dig[--n];
        *o++ = '\t';
        for (const char* c = snp_id[i]; *c; ++c) *o++ = *c;
        for (uint32_t j = 0; j < d; ++j) {
            const double vals[3] = {res->pvalue[i * d + j], res->beta[i * d + j], res->tstat[i * d + j]};
            for (double v : vals) {
                *o++ = '\t';
                o += format_exp6(v, o, 32);
            }
        }
        for (int k = 0; k < 3; ++k) {
            *o++ = '\t';
            o += format_exp6(res->r2[i * 3 + k], o, 32);
        }
        *o++ = '\n';
    }
    s.resize((size_t)(o - &s[0]));
}

bool write_tsv_body(FILE* f, uint64_t p, uint32_t d, const char* const* chrom, const uint64_t* pos,
                    const char* const* snp_id, const char* const* cov_names, const slfmm_results* res,
                    int n_threads) {
    std::string head = "chr\tpos\tsnp_id";
    for (uint32_t j = 0; j < d; ++j) {
        const std::string nm = cov_names[j];
        head += "\tp_" + nm + "\tbeta_" + nm + "\tt_" + nm;
    }
    head += "\tr2_cov\tr2_latent\tr2_resid\n";
    if (std::fwrite(head.data(), 1, head.size(), f) != head.size()) return false;
    const int nt = n_threads > 0 ? n_threads : (int)std::max(1u, std::thread::hardware_concurrency());
    // batches of nt blocks: the threads format batch k + 1 while one thread
    // writes batch k (the file is written in row order)
    const uint64_t block = std::max<uint64_t>(1024, std::min<uint64_t>(32768, ceil_div(p, 4 * (uint64_t)nt)));
    const uint64_t batch = block * (uint64_t)nt;
    std::vector<std::string> cur(nt), next(nt);
    std::atomic<bool> ok{true};
    std::thread writer;
    auto format_batch = [&](uint64_t b0, std::vector<std::string>& parts) {
        std::vector<std::thread> th;
        std::vector<char> failed(nt, 0);
        auto fmt = [&](int t) {
            try {
                const uint64_t r0 = std::min(p, b0 + (uint64_t)t * block), r1 = std::min(p, r0 + block);
                parts[t].clear();
                if (r1 > r0) format_tsv_rows(r0, r1, d, chrom, pos, snp_id, res, parts[t]);
            } catch (...) {
                failed[t] = 1;
            }
        };
        int started = 1;
        try {
            for (; started < nt; ++started) th.emplace_back(fmt, started);
        } catch (...) {
            // threads that did not start: their blocks are formatted below
        }
        fmt(0);
        for (int t = started; t < nt; ++t) fmt(t);
        for (auto& x : th) x.join();
        for (int t = 0; t < nt; ++t)
            if (failed[t]) ok = false;
    };
    try {
        for (uint64_t b0 = 0; b0 < p && ok; b0 += batch) {
            format_batch(b0, next);
            if (writer.joinable()) writer.join();
            if (!ok) break;
            std::swap(cur, next);
            writer = std::thread([&] {
                for (auto& s : cur)
                    if (ok && !s.empty() && std::fwrite(s.data(), 1, s.size(), f) != s.size()) ok = false;
            });
        }
    } catch (...) {
        if (writer.joinable()) writer.join();
        throw;
    }
    if (writer.joinable()) writer.join();
    return ok;
}
}  // namespace slfmm
