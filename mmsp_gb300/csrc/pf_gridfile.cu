// pf_gridfile.cu -- MMSP grid files written from host memory (host code).
//
// The reference compresses the whole payload with one compress2 call at
// level 9 (write_buffer, include/MMSP.grid.cpp:1880-1895), on one core.
// Payloads up to kDeflateChunk bytes are written the same way, so those
// files are byte-identical to the reference's.  Larger payloads are split
// into kDeflateChunk pieces deflated in parallel, each primed with the 32 KB
// before it as a preset dictionary and ended with a sync flush, the last
// with the end-of-stream block; the pieces are joined under one zlib header
// and the Adler-32 of the whole payload (RFC 1950/1951).  That is one valid
// zlib stream, so the reference's uncompress (include/MMSP.grid.cpp:1313)
// reads it, and its bytes depend on the chunk size only, not on the number
// of threads.
#include <stdio.h>
#include <string.h>
#include <zlib.h>

#include <atomic>
#include <thread>
#include <vector>

#include "MMSP.gpu.h"
#include "pf_gridfile.h"

namespace pf {

size_t payload_bytes(const GridFileInfo& fi, int fields)
{
    size_t cells = 1;
    for (int a = 0; a < fi.dim; a++) cells *= (size_t)fi.n[a];
    const size_t es = fi.f64 ? sizeof(double) : sizeof(float);
    return fi.vector ? cells * (sizeof(int32_t) + (size_t)fields * es) : cells * es;
}

std::string grid_header(const GridFileInfo& fi)
{
    std::string s = std::string("grid:") + (fi.vector ? "vector:" : "") + (fi.f64 ? "double" : "float") + "\n";
    char line[96];
    snprintf(line, sizeof(line), "%d\n%d\n", fi.dim, fi.fields_line);
    s += line;
    for (int a = 0; a < fi.dim; a++) {
        snprintf(line, sizeof(line), "%d %d\n", fi.g0[a], fi.g0[a] + fi.n[a]);
        s += line;
    }
    // ostream << double with default flags prints like %g (precision 6)
    for (int a = 0; a < fi.dim; a++) {
        snprintf(line, sizeof(line), "%g\n", fi.dx[a]);
        s += line;
    }
    return s;
}

namespace {

struct Piece {
    std::vector<unsigned char> out;
    uLong adler = 1;
    size_t len = 0;
    bool ok = false;
};

// Raw deflate of base[off, off+len), primed with the preceding 32 KB.
// Leaves p->ok false on any failure, allocation included (it runs on
// worker threads, which must not throw).
void deflate_piece(const unsigned char* base, size_t off, size_t len, bool last, int level, Piece* p)
{
    z_stream s;
    memset(&s, 0, sizeof(s));
    if (deflateInit2(&s, level, Z_DEFLATED, -15, 8, Z_DEFAULT_STRATEGY) != Z_OK) return;
    const size_t dict = off < 32768 ? off : 32768;
    if (dict && deflateSetDictionary(&s, base + off - dict, (uInt)dict) != Z_OK) {
        deflateEnd(&s);
        return;
    }
    try {
        p->out.resize(deflateBound(&s, (uLong)len) + 64);   // room for the sync-flush marker too
    } catch (...) {
        deflateEnd(&s);
        return;
    }
    s.next_in = const_cast<Bytef*>(base + off);
    s.avail_in = (uInt)len;
    s.next_out = p->out.data();
    s.avail_out = (uInt)p->out.size();
    const int rc = deflate(&s, last ? Z_FINISH : Z_SYNC_FLUSH);
    p->ok = s.avail_in == 0 && (last ? rc == Z_STREAM_END : rc == Z_OK);
    p->out.resize(p->out.size() - s.avail_out);
    deflateEnd(&s);
    p->adler = adler32(1L, base + off, (uInt)len);
    p->len = len;
}

// The two-byte zlib header deflate writes for `level` with a 32 KB window
// (RFC 1950: CM 8, CINFO 7, FLEVEL from the level, FCHECK making it a
// multiple of 31).
void zlib_header(int level, unsigned char out[2])
{
    const unsigned flevel = level < 2 ? 0 : level < 6 ? 1 : level == 6 ? 2 : 3;
    unsigned h = (0x78u << 8) | (flevel << 6);
    h += 31 - h % 31;
    out[0] = (unsigned char)(h >> 8);
    out[1] = (unsigned char)(h & 0xff);
}

struct File {
    FILE* f = nullptr;
    bool ok = true;
    explicit File(const char* name) : f(fopen(name, "wb")) {}
    ~File()
    {
        if (f) fclose(f);
    }
    void put(const void* p, size_t n)
    {
        if (ok && n && fwrite(p, 1, n, f) != n) ok = false;
    }
    bool close()
    {
        const bool good = ok && fclose(f) == 0;
        f = nullptr;
        return good;
    }
};

}  // namespace

static int write_grid_file_impl(const char* filename, const GridFileInfo& fi, const void* payload,
                                size_t size_in_mem, int level, int threads, std::string* why);

// No exception leaves: allocation failures (buffers, threads) become
// MMSP_GPU_ENOMEM.
int write_grid_file(const char* filename, const GridFileInfo& fi, const void* payload, size_t size_in_mem, int level,
                    int threads, std::string* why)
{
    try {
        return write_grid_file_impl(filename, fi, payload, size_in_mem, level, threads, why);
    } catch (...) {
        if (why) *why = "out of host memory or threads while writing the grid file";
        return MMSP_GPU_ENOMEM;
    }
}

static int write_grid_file_impl(const char* filename, const GridFileInfo& fi, const void* payload,
                                size_t size_in_mem, int level, int threads, std::string* why)
{
    if (!filename || !payload || level < 0 || level > 9) {
        if (why) *why = "write_grid_file: bad argument";
        return MMSP_GPU_EINVAL;
    }
    const unsigned char* raw = static_cast<const unsigned char*>(payload);
    std::vector<unsigned char> whole;   // one compress2 stream
    std::vector<Piece> pieces;          // or header + pieces + Adler-32
    unsigned char head[2], tail[4];
    uint64_t size_on_disk = size_in_mem;
    bool compressed = level > 0;
    if (compressed && size_in_mem <= kDeflateChunk) {
        uLongf n = compressBound((uLong)size_in_mem);
        whole.resize(n);
        if (compress2(whole.data(), &n, raw, (uLong)size_in_mem, level) != Z_OK) {
            if (why) *why = "zlib compress2 failed";
            return MMSP_GPU_ENOMEM;
        }
        whole.resize(n);
        size_on_disk = n;
    } else if (compressed) {
        const size_t np = (size_in_mem + kDeflateChunk - 1) / kDeflateChunk;
        pieces.resize(np);
        int nt = threads > 0 ? threads : (int)std::thread::hardware_concurrency();
        if (nt < 1) nt = 1;
        if ((size_t)nt > np) nt = (int)np;
        std::atomic<size_t> next(0);
        auto work = [&]() {
            for (size_t i; (i = next.fetch_add(1)) < np;) {
                const size_t off = i * kDeflateChunk;
                const size_t len = size_in_mem - off < kDeflateChunk ? size_in_mem - off : kDeflateChunk;
                deflate_piece(raw, off, len, i + 1 == np, level, &pieces[i]);
            }
        };
        std::vector<std::thread> pool;
        pool.reserve(nt);
        for (int t = 1; t < nt; t++) {
            try {
                pool.emplace_back(work);
            } catch (...) {
                break;   // fewer threads: the pieces left are taken by those running
            }
        }
        work();
        for (auto& t : pool) t.join();
        uLong adler = 1;
        size_on_disk = 2 + 4;
        for (const Piece& p : pieces) {
            if (!p.ok) {
                if (why) *why = "zlib deflate failed";
                return MMSP_GPU_ENOMEM;
            }
            adler = adler32_combine(adler, p.adler, (z_off_t)p.len);
            size_on_disk += p.out.size();
        }
        zlib_header(level, head);
        tail[0] = (unsigned char)(adler >> 24);
        tail[1] = (unsigned char)(adler >> 16);
        tail[2] = (unsigned char)(adler >> 8);
        tail[3] = (unsigned char)adler;
    }
    // A stream exactly as long as the payload would read back as raw data.
    if (compressed && size_on_disk == size_in_mem) {
        compressed = false;
        whole.clear();
        pieces.clear();
    }

    File f(filename);
    if (!f.f) {
        if (why) *why = std::string("could not open ") + filename;
        return MMSP_GPU_EIO;
    }
    const std::string hdr = grid_header(fi);
    f.put(hdr.data(), hdr.size());
    const int32_t nblocks = 1;
    f.put(&nblocks, sizeof(nblocks));
    for (int a = 0; a < fi.dim; a++) {
        const int32_t lim[2] = {fi.g0[a], fi.g0[a] + fi.n[a]};
        f.put(lim, sizeof(lim));
    }
    for (int a = 0; a < fi.dim; a++) {
        const int32_t b[2] = {fi.bc[a][0], fi.bc[a][1]};
        f.put(b, sizeof(b));
    }
    const uint64_t sizes[2] = {size_in_mem, compressed ? size_on_disk : size_in_mem};
    f.put(sizes, sizeof(sizes));
    if (!compressed) {
        f.put(raw, size_in_mem);
    } else if (!whole.empty()) {
        f.put(whole.data(), whole.size());
    } else {
        f.put(head, 2);
        for (const Piece& p : pieces) f.put(p.out.data(), p.out.size());
        f.put(tail, 4);
    }
    if (!f.close()) {
        if (why) *why = std::string("could not write ") + filename;
        return MMSP_GPU_EIO;
    }
    return MMSP_GPU_OK;
}

}  // namespace pf
