// <out>.parquet: the --format parquet output of the reference
// (coalesce_output_parquet, src/testing.rs:818-983), written directly from the
// result arrays.
//
// Schema (build_calibrated_schema, src/testing.rs:620-640), every field
// REQUIRED: chr (UTF8), pos (INT64), snp_id (UTF8), p_<cov>..., beta_<cov>...,
// t_<cov>..., r2_cov, r2_latent, r2_resid (DOUBLE).  The reference encodes
// chunks on worker threads and concatenates their row groups, so its rows are
// not in SNP order; here rows stay in SNP order.  Row groups of 2^18 rows, one
// PLAIN data page (v1, no levels: every column is required) per column chunk,
// compressed with ZSTD (the reference's codec) or left uncompressed; the
// column chunks of a row group are encoded on n_threads host threads.
//
// The file layout and the footer follow the Apache Parquet format
// specification; the footer and page headers are Thrift compact-protocol
// structs, encoded here field by field.  libzstd is loaded at run time
// (libzstd.so.1, its public ZSTD_compress / ZSTD_compressBound /
// ZSTD_isError entry points), so the library builds without its headers.
#include <dlfcn.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "slfmm_internal.h"

namespace slfmm {
namespace {

// Parquet enums (parquet.thrift)
enum : int32_t { kInt64T = 2, kDoubleT = 5, kByteArrayT = 6 };
enum : int32_t { kRequired = 0 };
enum : int32_t { kUtf8 = 0 };
enum : int32_t { kPlain = 0, kRle = 3 };
enum : int32_t { kDataPage = 0 };

// Thrift compact protocol: field headers carry the id delta in the high
// nibble (or a zigzag i16 after the type byte), integers are zigzag ULEB128,
// structs end with a stop byte, lists carry their size and element type
class Compact {
public:
    std::string out;
    Compact() { last_.push_back(0); }
    void varint(uint64_t v) {
        while (v >= 0x80) {
            out.push_back((char)(uint8_t)(v | 0x80));
            v >>= 7;
        }
        out.push_back((char)(uint8_t)v);
    }
    void zigzag(int64_t v) { varint(((uint64_t)v << 1) ^ (uint64_t)(v < 0 ? -1 : 0)); }
    void field(int16_t id, uint8_t type) {
        const int d = id - last_.back();
        if (d > 0 && d <= 15) {
            out.push_back((char)(uint8_t)((d << 4) | type));
        } else {
            out.push_back((char)type);
            zigzag(id);
        }
        last_.back() = id;
    }
    void i32(int16_t id, int32_t v) { field(id, 5); zigzag(v); }
    void i64(int16_t id, int64_t v) { field(id, 6); zigzag(v); }
    void str(int16_t id, const std::string& s) {
        field(id, 8);
        varint(s.size());
        out += s;
    }
    void list(int16_t id, uint8_t elem, size_t n) {
        field(id, 9);
        if (n < 15) {
            out.push_back((char)(uint8_t)((n << 4) | elem));
        } else {
            out.push_back((char)(uint8_t)(0xF0 | elem));
            varint(n);
        }
    }
    void struct_begin(int16_t id) { field(id, 12); last_.push_back(0); }
    void elem_begin() { last_.push_back(0); }    // a struct element of a list
    void struct_end() { out.push_back(0); last_.pop_back(); }
    void stop() { out.push_back(0); }              // end of the outermost struct

private:
    std::vector<int16_t> last_;
};

struct Zstd {
    size_t (*bound)(size_t) = nullptr;
    size_t (*compress)(void*, size_t, const void*, size_t, int) = nullptr;
    unsigned (*is_error)(size_t) = nullptr;
    bool ok = false;
    Zstd() {
        void* h = dlopen("libzstd.so.1", RTLD_NOW | RTLD_LOCAL);
        if (!h) return;
        bound = (size_t(*)(size_t))dlsym(h, "ZSTD_compressBound");
        compress = (size_t(*)(void*, size_t, const void*, size_t, int))dlsym(h, "ZSTD_compress");
        is_error = (unsigned (*)(size_t))dlsym(h, "ZSTD_isError");
        ok = bound && compress && is_error;
    }
};

const Zstd& zstd() {
    static const Zstd z;
    return z;
}

struct Column {
    std::string name;
    int32_t type;
    bool utf8;
};

struct ColumnChunk {
    std::string bytes;                   // page header + (compressed) page
    int64_t uncompressed = 0;            // header + uncompressed page
    bool ok = true;
};

struct Table {
    uint64_t p;
    uint32_t d;
    const char* const* chrom;
    const uint64_t* pos;
    const char* const* snp_id;
    const slfmm_results* res;
};

void put_u32(std::string& s, uint32_t v) {
    const char b[4] = {(char)(v & 0xff), (char)((v >> 8) & 0xff), (char)((v >> 16) & 0xff), (char)(v >> 24)};
    s.append(b, 4);
}

void put_u64(std::string& s, uint64_t v) {
    char b[8];
    for (int i = 0; i < 8; ++i) b[i] = (char)((v >> (8 * i)) & 0xff);
    s.append(b, 8);
}

// PLAIN values of column `c` for rows [r0, r1)
std::string plain_values(const Table& t, uint32_t c, uint64_t r0, uint64_t r1) {
    std::string v;
    const uint32_t d = t.d;
    auto strings = [&](const char* const* col) {
        for (uint64_t i = r0; i < r1; ++i) {
            const size_t len = std::strlen(col[i]);
            put_u32(v, (uint32_t)len);
            v.append(col[i], len);
        }
    };
    auto doubles = [&](const double* a, uint64_t stride, uint64_t off) {
        v.resize((r1 - r0) * 8);
        for (uint64_t i = r0; i < r1; ++i) {
            uint64_t bits;
            std::memcpy(&bits, &a[i * stride + off], 8);
            for (int b = 0; b < 8; ++b) v[(i - r0) * 8 + b] = (char)((bits >> (8 * b)) & 0xff);
        }
    };
    if (c == 0) {
        strings(t.chrom);
    } else if (c == 1) {
        v.reserve((r1 - r0) * 8);
        for (uint64_t i = r0; i < r1; ++i) put_u64(v, t.pos[i]);
    } else if (c == 2) {
        strings(t.snp_id);
    } else if (c < 3 + d) {
        doubles(t.res->pvalue, d, c - 3);
    } else if (c < 3 + 2 * d) {
        doubles(t.res->beta, d, c - 3 - d);
    } else if (c < 3 + 3 * d) {
        doubles(t.res->tstat, d, c - 3 - 2 * d);
    } else {
        doubles(t.res->r2, 3, c - 3 - 3 * d);
    }
    return v;
}

ColumnChunk encode_chunk(const Table& t, uint32_t c, uint64_t r0, uint64_t r1, int codec) {
    ColumnChunk cc;
    const std::string raw = plain_values(t, c, r0, r1);
    std::string body;
    if (codec == SLFMM_PARQUET_ZSTD) {
        const Zstd& z = zstd();
        body.resize(z.bound(raw.size()));
        const size_t n = z.compress(&body[0], body.size(), raw.data(), raw.size(), 1);
        if (z.is_error(n)) {
            cc.ok = false;
            return cc;
        }
        body.resize(n);
    } else {
        body = raw;
    }
    if (raw.size() > 0x7fffffffu || body.size() > 0x7fffffffu) {
        cc.ok = false;   // a page size is an i32
        return cc;
    }
    Compact h;   // PageHeader
    h.i32(1, kDataPage);
    h.i32(2, (int32_t)raw.size());
    h.i32(3, (int32_t)body.size());
    h.struct_begin(5);   // DataPageHeader
    h.i32(1, (int32_t)(r1 - r0));
    h.i32(2, kPlain);
    h.i32(3, kRle);
    h.i32(4, kRle);
    h.struct_end();
    h.stop();
    cc.uncompressed = (int64_t)(h.out.size() + raw.size());
    cc.bytes = std::move(h.out);
    cc.bytes += body;
    return cc;
}

struct ChunkMeta {
    int64_t offset, uncompressed, compressed;
};

// the file body after a successful fopen: magic, row groups, footer
bool write_parquet_file(FILE* f, uint64_t p, uint32_t d, const char* const* chrom, const uint64_t* pos,
                        const char* const* snp_id, const char* const* cov_names, const slfmm_results* res,
                        int compression, int n_threads) {
    std::vector<Column> cols = {{"chr", kByteArrayT, true}, {"pos", kInt64T, false}, {"snp_id", kByteArrayT, true}};
    for (const char* pre : {"p_", "beta_", "t_"})
        for (uint32_t j = 0; j < d; ++j) cols.push_back({std::string(pre) + cov_names[j], kDoubleT, false});
    for (const char* nm : {"r2_cov", "r2_latent", "r2_resid"}) cols.push_back({nm, kDoubleT, false});
    const uint32_t nc = (uint32_t)cols.size();

    bool ok = std::fwrite("PAR1", 1, 4, f) == 4;
    int64_t off = 4;
    const Table t{p, d, chrom, pos, snp_id, res};
    const uint64_t rg_rows = 1ull << 18;
    const int nt = n_threads > 0 ? n_threads : (int)std::max(1u, std::thread::hardware_concurrency());
    std::vector<std::vector<ChunkMeta>> groups;
    std::vector<uint64_t> group_rows;
    for (uint64_t r0 = 0; r0 < p && ok; r0 += rg_rows) {
        const uint64_t r1 = std::min(p, r0 + rg_rows);
        std::vector<ColumnChunk> chunks(nc);
        std::atomic<uint32_t> next{0};
        auto work = [&]() {
            for (uint32_t c = next++; c < nc; c = next++) {
                try {
                    chunks[c] = encode_chunk(t, c, r0, r1, compression);
                } catch (...) {
                    chunks[c].ok = false;
                }
            }
        };
        std::vector<std::thread> th;
        try {
            for (int i = 1; i < std::min<int>(nt, (int)nc); ++i) th.emplace_back(work);
        } catch (...) {
            // fewer threads: those started and this one take the columns
        }
        work();
        for (auto& x : th) x.join();
        std::vector<ChunkMeta> meta(nc);
        for (uint32_t c = 0; c < nc && ok; ++c) {
            ok = chunks[c].ok && std::fwrite(chunks[c].bytes.data(), 1, chunks[c].bytes.size(), f) ==
                                     chunks[c].bytes.size();
            meta[c] = {off, chunks[c].uncompressed, (int64_t)chunks[c].bytes.size()};
            off += (int64_t)chunks[c].bytes.size();
        }
        groups.push_back(std::move(meta));
        group_rows.push_back(r1 - r0);
    }

    Compact m;   // FileMetaData
    m.i32(1, 1);
    m.list(2, 12, nc + 1);
    m.elem_begin();   // root
    m.str(4, "schema");
    m.i32(5, (int32_t)nc);
    m.struct_end();
    for (const Column& c : cols) {
        m.elem_begin();
        m.i32(1, c.type);
        m.i32(3, kRequired);
        m.str(4, c.name);
        if (c.utf8) m.i32(6, kUtf8);
        m.struct_end();
    }
    m.i64(3, (int64_t)p);
    m.list(4, 12, groups.size());
    for (size_t g = 0; g < groups.size(); ++g) {
        m.elem_begin();   // RowGroup
        m.list(1, 12, nc);
        int64_t total = 0, total_c = 0;
        for (uint32_t c = 0; c < nc; ++c) {
            const ChunkMeta& cm = groups[g][c];
            total += cm.uncompressed;
            total_c += cm.compressed;
            m.elem_begin();   // ColumnChunk
            m.i64(2, cm.offset);
            m.struct_begin(3);   // ColumnMetaData
            m.i32(1, cols[c].type);
            m.list(2, 5, 1);
            m.zigzag(kPlain);
            m.list(3, 8, 1);
            m.varint(cols[c].name.size());
            m.out += cols[c].name;
            m.i32(4, compression);
            m.i64(5, (int64_t)group_rows[g]);
            m.i64(6, cm.uncompressed);
            m.i64(7, cm.compressed);
            m.i64(9, cm.offset);
            m.struct_end();
            m.struct_end();
        }
        m.i64(2, total);
        m.i64(3, (int64_t)group_rows[g]);
        m.i64(5, groups[g].empty() ? 0 : groups[g][0].offset);
        m.i64(6, total_c);
        m.struct_end();
    }
    m.str(6, "schnellfmm_gb300");
    m.stop();
    if (ok) {
        std::string tail = m.out;
        put_u32(tail, (uint32_t)m.out.size());
        tail += "PAR1";
        ok = std::fwrite(tail.data(), 1, tail.size(), f) == tail.size();
    }
    return ok;
}

}  // namespace
}  // namespace slfmm

extern "C" int slfmm_write_parquet(const char* path, uint64_t p, uint32_t d, const char* const* chrom,
                                   const uint64_t* pos, const char* const* snp_id, const char* const* cov_names,
                                   const slfmm_results* res, int compression, int n_threads) {
    using namespace slfmm;
    if (!path || !res || (p && (!chrom || !pos || !snp_id)) || (d && !cov_names)) return SLFMM_ERR_BAD_ARG;
    if (p && (!res->pvalue || !res->beta || !res->tstat || !res->r2)) return SLFMM_ERR_BAD_ARG;
    if (compression != SLFMM_PARQUET_UNCOMPRESSED && compression != SLFMM_PARQUET_ZSTD) return SLFMM_ERR_BAD_ARG;
    if (compression == SLFMM_PARQUET_ZSTD && !zstd().ok) return SLFMM_ERR_IO;
    FILE* f = std::fopen(path, "wb");
    if (!f) return SLFMM_ERR_IO;
    int rc = SLFMM_OK;
    try {
        rc = write_parquet_file(f, p, d, chrom, pos, snp_id, cov_names, res, compression, n_threads)
                 ? SLFMM_OK
                 : SLFMM_ERR_IO;
    } catch (const std::bad_alloc&) {
        rc = SLFMM_ERR_NOMEM;
    } catch (...) {
        rc = SLFMM_ERR_IO;
    }
    if (std::fclose(f) != 0 && rc == SLFMM_OK) rc = SLFMM_ERR_IO;
    return rc;
}
