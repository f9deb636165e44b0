// Minimal HDF5 reader/writer for SpinWalk's phantom and result files, written from the HDF5
// file-format specification (no libhdf5 in this build).
//
// SpinWalk reads and writes whole datasets of the root group (src/sim/h5_helper.h:48-129):
// phantoms hold `mask` (uint8 [Nx,Ny,Nz]), optional `fieldmap` (float [Nx,Ny,Nz]) and `fov`
// (float [3]); optional start files hold `XYZ` / `M` (float [N,3]); results hold M, XYZ, T,
// scales, TE. libhdf5 with default settings stores such files with a version-0 superblock, an
// "old-style" root group (symbol-table message -> version-1 B-tree of group nodes -> symbol table
// nodes, names in a local heap), version-1 object headers and contiguous data. That subset is
// what this file reads (plus continuation blocks and 64-bit floats) and writes. The reader also
// takes chunked datasets (version-1 B-tree chunk index) with the deflate, shuffle and fletcher32
// filters, as h5py's compression="gzip" and MATLAB's compressed files store them; unwritten
// chunks read as zeros (the default fill value).
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "sw_h5.h"

namespace sw {
namespace h5 {
namespace {

constexpr uint64_t kUndef = ~uint64_t(0);
// Largest dataset read (far above any phantom: 800^3 float32 is 2 GiB).
constexpr uint64_t kMaxDatasetBytes = 1ull << 40;
const unsigned char kSig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};

// The file's bytes from its superblock on (a read-only memory map: only the pages a read
// touches are loaded).
struct View {
    const char *p = nullptr;
    uint64_t n = 0;
    const char &operator[](uint64_t i) const { return p[i]; }
    uint64_t size() const { return n; }
    const char *data() const { return p; }
};

class MappedFile {
  public:
    MappedFile() = default;
    MappedFile(const MappedFile &) = delete;
    MappedFile &operator=(const MappedFile &) = delete;
    ~MappedFile() {
        if (map_) munmap(map_, len_);
    }
    // Maps the file and drops a user block: the superblock may start at 0, 512, 1024, ...; file
    // addresses are relative to it (base address 0 in that frame). Where the file system cannot
    // map the file, the whole file is read into memory instead. A mapped file must not be
    // truncated while it is read (the process would get SIGBUS on the lost pages).
    bool open(const std::string &file, std::string &err) {
        const int fd = ::open(file.c_str(), O_RDONLY);
        if (fd < 0) { err = "cannot open " + file; return false; }
        struct stat st;
        if (fstat(fd, &st) != 0 || st.st_size < 8) {
            ::close(fd);
            err = file + " is not an HDF5 file";
            return false;
        }
        len_ = (size_t)st.st_size;
        void *m = mmap(nullptr, len_, PROT_READ, MAP_PRIVATE, fd, 0);
        const char *base = nullptr;
        if (m != MAP_FAILED) {
            map_ = m;
            base = static_cast<const char *>(m);
        } else {                                   // buffered read of the whole file
            try {
                copy_.resize(len_);
            } catch (const std::bad_alloc &) {
                ::close(fd);
                err = "cannot map or read " + file + " (out of memory)";
                return false;
            }
            size_t got = 0;
            while (got < len_) {
                const ssize_t r = ::pread(fd, copy_.data() + got, len_ - got, (off_t)got);
                if (r <= 0) break;
                got += (size_t)r;
            }
            if (got != len_) {
                ::close(fd);
                err = "cannot read " + file;
                return false;
            }
            base = copy_.data();
        }
        ::close(fd);
        for (uint64_t at = 0; at + 8 <= len_; at = at ? 2 * at : 512) {
            if (std::memcmp(base + at, kSig, 8) == 0) {
                view = View{base + at, len_ - at};
                return true;
            }
        }
        err = file + " is not an HDF5 file";
        return false;
    }
    View view;

  private:
    void *map_ = nullptr;
    std::vector<char> copy_;    // the file's bytes where it could not be mapped
    size_t len_ = 0;
};

struct Buf {
    const View &b;
    bool ok(uint64_t off, uint64_t n) const { return off <= b.size() && n <= b.size() - off; }
    uint64_t u(uint64_t off, int n) const {
        uint64_t v = 0;
        for (int i = n - 1; i >= 0; i--) v = (v << 8) | (unsigned char)b[off + i];
        return v;
    }
};

struct Msg {
    uint16_t type;
    uint64_t off, size;
};

// Whether bytes [rel, rel + n) lie inside message m.
bool fits(const Msg &m, uint64_t rel, uint64_t n) { return rel <= m.size && n <= m.size - rel; }

// r = a * b; false on overflow
bool mul_ok(uint64_t a, uint64_t b, uint64_t &r) {
    if (a != 0 && b > ~uint64_t(0) / a) return false;
    r = a * b;
    return true;
}

// Messages of a version-1 object header, following continuation blocks.
bool header_messages(const Buf &B, uint64_t addr, std::vector<Msg> &out, std::string &err) {
    if (!B.ok(addr, 16)) { err = "object header outside the file"; return false; }
    if (B.u(addr, 1) != 1) { err = "unsupported object header version (only version 1)"; return false; }
    const uint64_t nmsg = B.u(addr + 2, 2), hsize = B.u(addr + 8, 4);
    std::vector<std::pair<uint64_t, uint64_t>> blocks{{addr + 16, hsize}};
    for (size_t bi = 0; bi < blocks.size() && out.size() < nmsg; bi++) {
        uint64_t p = blocks[bi].first;
        const uint64_t end = blocks[bi].first + blocks[bi].second;
        while (p + 8 <= end && out.size() < nmsg) {
            if (!B.ok(p, 8)) { err = "truncated object header"; return false; }
            Msg m{(uint16_t)B.u(p, 2), p + 8, B.u(p + 2, 2)};
            if (!B.ok(m.off, m.size)) { err = "truncated header message"; return false; }
            if (m.type == 0x0010) blocks.push_back({B.u(m.off, 8), B.u(m.off + 8, 8)});
            out.push_back(m);
            p = m.off + ((m.size + 7) & ~uint64_t(7));
        }
    }
    return true;
}

bool read_string(const Buf &B, uint64_t off, std::string &s) {
    s.clear();
    while (B.ok(off, 1) && B.b[off] != '\0') s += B.b[off++];
    return B.ok(off, 1);
}

// Walks a version-1 B-tree of group nodes and collects (name, object header address).
bool group_entries(const Buf &B, uint64_t btree, uint64_t heap_data,
                   std::vector<std::pair<std::string, uint64_t>> &out, std::string &err,
                   uint64_t &budget, int depth = 0) {
    if (depth > 32 || budget == 0 || !B.ok(btree, 24) || std::memcmp(&B.b[btree], "TREE", 4) != 0) {
        err = "bad group B-tree";
        return false;
    }
    budget--;
    const unsigned level = (unsigned)B.u(btree + 5, 1), used = (unsigned)B.u(btree + 6, 2);
    uint64_t p = btree + 24 + 8;                 // past the first key
    for (unsigned i = 0; i < used; i++, p += 16) {
        if (!B.ok(p, 8)) { err = "truncated B-tree"; return false; }
        const uint64_t child = B.u(p, 8);
        if (level > 0) {
            if (!group_entries(B, child, heap_data, out, err, budget, depth + 1)) return false;
            continue;
        }
        if (!B.ok(child, 8) || std::memcmp(&B.b[child], "SNOD", 4) != 0) {
            err = "bad symbol table node";
            return false;
        }
        const unsigned ns = (unsigned)B.u(child + 6, 2);
        if (budget < ns) { err = "bad group B-tree"; return false; }
        budget -= ns;
        for (unsigned k = 0; k < ns; k++) {
            const uint64_t e = child + 8 + 40ull * k;
            if (!B.ok(e, 40)) { err = "truncated symbol table node"; return false; }
            std::string name;
            if (!read_string(B, heap_data + B.u(e, 8), name)) { err = "bad link name"; return false; }
            out.push_back({name, B.u(e + 8, 8)});
        }
    }
    return true;
}

bool root_entries(const Buf &B, std::vector<std::pair<std::string, uint64_t>> &out, std::string &err) {
    if (!B.ok(0, 96) || std::memcmp(B.b.data(), kSig, 8) != 0) { err = "not an HDF5 file"; return false; }
    if (B.u(8, 1) != 0 && B.u(8, 1) != 1) {
        err = "unsupported HDF5 superblock version " + std::to_string(B.u(8, 1)) + " (0/1 supported)";
        return false;
    }
    if (B.u(13, 1) != 8 || B.u(14, 1) != 8) { err = "only 8-byte offsets/lengths supported"; return false; }
    const uint64_t root = 24 + 32 + (B.u(8, 1) == 1 ? 4 : 0);   // root symbol table entry
    const uint64_t ohdr = B.u(root + 8, 8);
    std::vector<Msg> msgs;
    if (!header_messages(B, ohdr, msgs, err)) return false;
    for (const Msg &m : msgs) {
        if (m.type != 0x0011) continue;                           // symbol table message
        const uint64_t btree = B.u(m.off, 8), heap = B.u(m.off + 8, 8);
        if (!B.ok(heap, 32) || std::memcmp(&B.b[heap], "HEAP", 4) != 0) {
            err = "bad local heap";
            return false;
        }
        uint64_t budget = B.b.size() / 24 + 1;            // nodes and entries a valid tree can hold
        return group_entries(B, btree, B.u(heap + 24, 8), out, err, budget);
    }
    err = "root group has no symbol table (new-style groups are not supported)";
    return false;
}

// ---- chunked storage: the version-1 B-tree chunk index, filters and a deflate decoder ---------

// Bits of a deflate stream, least significant bit first (RFC 1951 section 3.1.1).
struct BitReader {
    const uint8_t *p;
    size_t n, pos = 0;
    uint64_t buf = 0;
    int cnt = 0;
    bool get(int k, uint32_t &v) {                     // k <= 24
        while (cnt < k) {
            if (pos >= n) return false;
            buf |= (uint64_t)p[pos++] << cnt;
            cnt += 8;
        }
        v = (uint32_t)(buf & ((1ull << k) - 1));
        buf >>= k;
        cnt -= k;
        return true;
    }
    void to_byte() {                                   // drop the bits of a partial byte
        buf >>= (cnt & 7);
        cnt -= cnt & 7;
    }
};

// A canonical Huffman code: the number of codes of each length and the symbols in code order.
struct Huffman {
    uint16_t count[16];
    uint16_t symbol[320];
};

// Returns false for an over-subscribed set of lengths; an incomplete set is accepted (its
// unused codes fail to decode).
bool huffman_build(Huffman &h, const uint8_t *len, int n) {
    std::memset(h.count, 0, sizeof h.count);
    for (int s = 0; s < n; s++) h.count[len[s]]++;
    int left = 1;
    for (int l = 1; l < 16; l++) {
        left = 2 * left - h.count[l];
        if (left < 0) return false;
    }
    uint16_t next[16];
    next[1] = 0;
    for (int l = 1; l < 15; l++) next[l + 1] = (uint16_t)(next[l] + h.count[l]);
    for (int s = 0; s < n; s++)
        if (len[s]) h.symbol[next[len[s]]++] = (uint16_t)s;
    return true;
}

// One symbol: codes are read most significant bit first; -1 when the stream ends or the code
// is not in the set.
int huffman_decode(BitReader &br, const Huffman &h) {
    int code = 0, first = 0, index = 0;
    for (int l = 1; l < 16; l++) {
        uint32_t bit;
        if (!br.get(1, bit)) return -1;
        code |= (int)bit;
        const int count = h.count[l];
        if (code - first < count) return h.symbol[index + code - first];
        index += count;
        first = (first + count) << 1;
        code <<= 1;
    }
    return -1;
}

// Literal/length and distance symbols of one compressed block (RFC 1951 section 3.2.5).
bool inflate_codes(BitReader &br, const Huffman &lit, const Huffman &dist, size_t limit,
                   std::vector<uint8_t> &out) {
    static const uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                                          31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
    static const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2,
                                          2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
    static const uint16_t kDistBase[30] = {1,    2,    3,    4,    5,    7,     9,     13,    17,  25,
                                           33,   49,   65,   97,   129,  193,   257,   385,   513, 769,
                                           1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
    static const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2,  3,  3,  4,  4,  5,  5,  6,
                                           6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
    for (;;) {
        int sym = huffman_decode(br, lit);
        if (sym < 0) return false;
        if (sym < 256) {
            if (out.size() >= limit) return false;
            out.push_back((uint8_t)sym);
            continue;
        }
        if (sym == 256) return true;
        sym -= 257;
        if (sym >= 29) return false;
        uint32_t e;
        if (!br.get(kLenExtra[sym], e)) return false;
        const size_t len = kLenBase[sym] + e;
        const int d = huffman_decode(br, dist);
        if (d < 0 || d >= 30 || !br.get(kDistExtra[d], e)) return false;
        const size_t back = kDistBase[d] + e;
        if (back > out.size() || out.size() + len > limit) return false;
        for (size_t i = 0; i < len; i++) {
            const uint8_t c = out[out.size() - back];
            out.push_back(c);
        }
    }
}

uint32_t adler32(const std::vector<uint8_t> &v) {
    uint32_t a = 1, b = 0;
    for (uint8_t c : v) {
        a = (a + c) % 65521u;
        b = (b + a) % 65521u;
    }
    return (b << 16) | a;
}

// A zlib stream (RFC 1950: header, deflate blocks, Adler-32 of the output), as HDF5's deflate
// filter writes it; at most `limit` output bytes.
bool zlib_inflate(const uint8_t *p, size_t n, size_t limit, std::vector<uint8_t> &out,
                  std::string &err) {
    out.clear();
    if (n < 6 || (p[0] & 15) != 8 || (p[0] >> 4) > 7 || ((p[0] << 8) | p[1]) % 31 != 0 ||
        (p[1] & 0x20)) {
        err = "deflate filter: not a zlib stream";
        return false;
    }
    BitReader br{p + 2, n - 2};
    uint32_t last = 0, type = 0;
    do {
        if (!br.get(1, last) || !br.get(2, type)) break;
        if (type == 0) {                                   // stored
            br.to_byte();
            uint32_t len, nlen;
            if (!br.get(16, len) || !br.get(16, nlen) || len != (~nlen & 0xffffu)) break;
            if (out.size() + len > limit) break;
            uint32_t c = 0;
            for (uint32_t i = 0; i < len && br.get(8, c); i++) out.push_back((uint8_t)c);
        } else if (type == 1) {                            // fixed codes
            static Huffman fl, fd;
            static const bool built = [] {
                uint8_t l[288];
                for (int i = 0; i < 288; i++) l[i] = i < 144 ? 8 : i < 256 ? 9 : i < 280 ? 7 : 8;
                huffman_build(fl, l, 288);
                for (int i = 0; i < 30; i++) l[i] = 5;
                huffman_build(fd, l, 30);
                return true;
            }();
            (void)built;
            if (!inflate_codes(br, fl, fd, limit, out)) break;
        } else if (type == 2) {                            // dynamic codes
            uint32_t hlit, hdist, hclen;
            if (!br.get(5, hlit) || !br.get(5, hdist) || !br.get(4, hclen)) break;
            hlit += 257;
            hdist += 1;
            hclen += 4;
            if (hlit > 286 || hdist > 30) break;
            static const uint8_t kOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5,
                                               11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t lens[320] = {0};
            bool ok = true;
            for (uint32_t i = 0; i < hclen && ok; i++) {
                uint32_t v = 0;
                ok = br.get(3, v);
                lens[kOrder[i]] = (uint8_t)v;
            }
            Huffman lc;
            if (!ok || !huffman_build(lc, lens, 19)) break;
            std::memset(lens, 0, sizeof lens);
            uint32_t idx = 0;
            while (ok && idx < hlit + hdist) {
                const int sym = huffman_decode(br, lc);
                uint32_t rep = 0, v = 0;
                uint8_t val = 0;
                if (sym < 0) { ok = false; break; }
                if (sym < 16) { lens[idx++] = (uint8_t)sym; continue; }
                if (sym == 16) {
                    if (idx == 0 || !br.get(2, v)) { ok = false; break; }
                    val = lens[idx - 1];
                    rep = 3 + v;
                } else if (sym == 17) {
                    if (!br.get(3, v)) { ok = false; break; }
                    rep = 3 + v;
                } else {
                    if (!br.get(7, v)) { ok = false; break; }
                    rep = 11 + v;
                }
                if (idx + rep > hlit + hdist) { ok = false; break; }
                while (rep--) lens[idx++] = val;
            }
            Huffman lit, dist;
            if (!ok || lens[256] == 0 || !huffman_build(lit, lens, (int)hlit) ||
                !huffman_build(dist, lens + hlit, (int)hdist) ||
                !inflate_codes(br, lit, dist, limit, out))
                break;
        } else {
            break;
        }
        if (last) {
            br.to_byte();
            uint32_t a[4];
            for (int i = 0; i < 4; i++)
                if (!br.get(8, a[i])) { err = "deflate filter: truncated stream"; return false; }
            const uint32_t want = (a[0] << 24) | (a[1] << 16) | (a[2] << 8) | a[3];
            if (want != adler32(out)) { err = "deflate filter: Adler-32 mismatch"; return false; }
            return true;
        }
    } while (true);
    err = "deflate filter: corrupt or oversized stream";
    return false;
}

struct Filter {
    uint16_t id;
    std::vector<uint32_t> cd;       // client data
};

// The filter pipeline message (0x000B), versions 1 and 2.
bool filter_pipeline(const Buf &B, const Msg &m, std::vector<Filter> &out, std::string &err) {
    const unsigned ver = (unsigned)B.u(m.off, 1), nf = (unsigned)B.u(m.off + 1, 1);
    uint64_t p = m.off + (ver == 1 ? 8 : 2);
    const uint64_t end = m.off + m.size;
    if (ver != 1 && ver != 2) { err = "unsupported filter pipeline version"; return false; }
    for (unsigned i = 0; i < nf; i++) {
        if (p + 8 > end) { err = "truncated filter pipeline"; return false; }
        Filter f;
        f.id = (uint16_t)B.u(p, 2);
        p += 2;
        uint64_t name_len = 0;
        if (ver == 1 || f.id >= 256) {
            name_len = B.u(p, 2);
            p += 2;
        }
        p += 2;                                            // flags
        const unsigned ncd = (unsigned)B.u(p, 2);
        p += 2;
        if (ver == 1) name_len = (name_len + 7) & ~uint64_t(7);
        p += name_len;
        for (unsigned k = 0; k < ncd; k++, p += 4) {
            if (p + 4 > end) { err = "truncated filter pipeline"; return false; }
            f.cd.push_back((uint32_t)B.u(p, 4));
        }
        if (ver == 1 && (ncd & 1)) p += 4;
        out.push_back(f);
    }
    return true;
}

// One chunk through the pipeline in reverse (the filters a chunk's mask marks as skipped are
// not applied to it): deflate (1), shuffle (2), fletcher32 (3).
bool unfilter(const std::vector<Filter> &fs, uint32_t mask, std::vector<uint8_t> &data,
              size_t expect, std::string &err) {
    for (size_t i = fs.size(); i-- > 0;) {
        if ((mask >> i) & 1u) continue;
        const Filter &f = fs[i];
        if (f.id == 1) {
            std::vector<uint8_t> out;
            if (!zlib_inflate(data.data(), data.size(), expect, out, err)) return false;
            data.swap(out);
        } else if (f.id == 2) {
            const size_t es = f.cd.empty() ? 1 : f.cd[0];
            if (es > 1) {
                const size_t n = data.size() / es;
                std::vector<uint8_t> out(data.size());
                for (size_t b = 0; b < es; b++)
                    for (size_t k = 0; k < n; k++) out[k * es + b] = data[b * n + k];
                std::copy(data.begin() + n * es, data.end(), out.begin() + n * es);
                data.swap(out);
            }
        } else if (f.id == 3) {
            if (data.size() < 4) { err = "fletcher32 filter: chunk shorter than its checksum"; return false; }
            data.resize(data.size() - 4);
        } else {
            err = "unsupported HDF5 filter " + std::to_string(f.id) +
                  " (deflate, shuffle and fletcher32 are supported)";
            return false;
        }
    }
    return true;
}

struct ChunkRef {
    uint64_t addr, size;
    uint32_t mask;
    std::vector<uint64_t> off;
};

// Walks the version-1 B-tree of raw data chunks (node type 1); `nd` is the dataset rank + 1.
// `budget` bounds the nodes visited and chunks listed (a damaged tree may point back at itself).
bool chunk_index(const Buf &B, uint64_t node, unsigned nd, std::vector<ChunkRef> &out,
                 std::string &err, uint64_t &budget, int depth = 0) {
    if (depth > 32 || budget == 0 || !B.ok(node, 24) || std::memcmp(&B.b[node], "TREE", 4) != 0 ||
        B.u(node + 4, 1) != 1) {
        err = "bad chunk B-tree";
        return false;
    }
    budget--;
    const unsigned level = (unsigned)B.u(node + 5, 1), used = (unsigned)B.u(node + 6, 2);
    const uint64_t key = 8 + 8ull * nd;
    uint64_t p = node + 24;
    for (unsigned i = 0; i < used; i++, p += key + 8) {
        if (!B.ok(p, key + 8)) { err = "truncated chunk B-tree"; return false; }
        const uint64_t child = B.u(p + key, 8);
        if (level > 0) {
            if (!chunk_index(B, child, nd, out, err, budget, depth + 1)) return false;
            continue;
        }
        if (budget == 0) { err = "bad chunk B-tree"; return false; }
        budget--;
        ChunkRef c{child, B.u(p, 4), (uint32_t)B.u(p + 4, 4), {}};
        for (unsigned k = 0; k < nd; k++) c.off.push_back(B.u(p + 8 + 8ull * k, 8));
        out.push_back(std::move(c));
    }
    return true;
}

// The whole dataset from its chunks; chunks that were never written read as zeros.
bool read_chunked(const Buf &B, const std::vector<uint64_t> &dims, uint64_t esz, uint64_t btree,
                  const std::vector<uint64_t> &cdim, const std::vector<Filter> &filters,
                  std::vector<char> &data, std::string &err) {
    const size_t rank = dims.size();
    if (rank == 0 || cdim.size() != rank + 1 || cdim[rank] != esz) {
        err = "chunk dimensions do not match the dataset";
        return false;
    }
    uint64_t count = 1, celems = 1, grid = 1;
    for (size_t k = 0; k < rank; k++) {
        if (cdim[k] == 0) { err = "zero chunk dimension"; return false; }
        count *= dims[k];                                  // the caller checked the total
        if (!mul_ok(celems, cdim[k], celems) || !mul_ok(grid, (dims[k] + cdim[k] - 1) / cdim[k], grid)) {
            err = "bad chunk dimensions";
            return false;
        }
    }
    if (celems > kMaxDatasetBytes / esz) { err = "bad chunk dimensions"; return false; }
    data.assign(count * esz, 0);
    if (btree == kUndef) return true;
    std::vector<ChunkRef> chunks;
    uint64_t budget = grid + B.b.size() / 24 + 1;          // chunks + nodes a valid tree can hold
    if (!chunk_index(B, btree, (unsigned)rank + 1, chunks, err, budget)) return false;
    const size_t cbytes = celems * esz;
    std::vector<uint8_t> buf;
    for (const ChunkRef &c : chunks) {
        if (c.off[rank] != 0) { err = "bad chunk offset"; return false; }
        for (size_t k = 0; k < rank; k++)
            if (c.off[k] % cdim[k] != 0 || c.off[k] >= dims[k]) { err = "bad chunk offset"; return false; }
        if (!B.ok(c.addr, c.size)) { err = "chunk outside the file"; return false; }
        buf.assign((const uint8_t *)B.b.data() + c.addr, (const uint8_t *)B.b.data() + c.addr + c.size);
        if (!unfilter(filters, c.mask, buf, cbytes, err)) return false;
        if (buf.size() != cbytes) {
            err = "chunk decodes to " + std::to_string(buf.size()) + " bytes, expected " +
                  std::to_string(cbytes);
            return false;
        }
        // copy the rows along the last dimension that lie inside the dataset
        const uint64_t run = std::min(cdim[rank - 1], dims[rank - 1] - c.off[rank - 1]);
        std::vector<uint64_t> loc(rank, 0);
        for (;;) {
            bool inside = true;
            uint64_t g = 0, l = 0;
            for (size_t k = 0; k < rank; k++) {
                const uint64_t x = c.off[k] + loc[k];
                if (x >= dims[k]) inside = false;
                g = g * dims[k] + x;
                l = l * cdim[k] + loc[k];
            }
            if (inside) std::memcpy(data.data() + g * esz, buf.data() + l * esz, run * esz);
            size_t k = rank - 1;                           // next row: odometer over dims 0..rank-2
            while (k > 0) {
                if (++loc[k - 1] < cdim[k - 1]) break;
                loc[k - 1] = 0;
                k--;
            }
            if (k == 0) break;
        }
    }
    return true;
}

}  // namespace

namespace {

bool read_impl(const std::string &file, const std::string &name, Dataset &out, std::string &err,
               bool with_data) {
    MappedFile mf;
    if (!mf.open(file, err)) return false;
    Buf B{mf.view};
    const View &bytes = mf.view;
    std::vector<std::pair<std::string, uint64_t>> ents;
    if (!root_entries(B, ents, err)) return false;
    uint64_t addr = kUndef;
    for (auto &e : ents)
        if (e.first == name) addr = e.second;
    if (addr == kUndef) { err = "dataset " + name + " not found in " + file; return false; }
    std::vector<Msg> msgs;
    if (!header_messages(B, addr, msgs, err)) return false;
    out = Dataset{};
    int dtype_class = -1;
    uint64_t dtype_size = 0, data_addr = kUndef, data_size = 0;
    bool little = true, is_signed = false, chunked = false;
    std::vector<uint64_t> cdim;
    std::vector<Filter> filters;
    for (const Msg &m : msgs) {
        if (m.type == 0x000B && !filter_pipeline(B, m, filters, err)) return false;
    }
    for (const Msg &m : msgs) {
        if (m.type == 0x0001) {                                    // dataspace
            if (!fits(m, 0, 2)) { err = "dataset " + name + ": bad dataspace"; return false; }
            const unsigned ver = (unsigned)B.u(m.off, 1), rank = (unsigned)B.u(m.off + 1, 1);
            const uint64_t rel = ver == 1 ? 8 : 4;
            if (rank > 32 || !fits(m, rel, 8ull * rank)) {
                err = "dataset " + name + ": bad dataspace";
                return false;
            }
            for (unsigned i = 0; i < rank; i++) out.dims.push_back(B.u(m.off + rel + 8ull * i, 8));
        } else if (m.type == 0x0003) {                             // datatype
            if (!fits(m, 0, 8)) { err = "dataset " + name + ": bad datatype"; return false; }
            dtype_class = (int)(B.u(m.off, 1) & 0x0f);
            const unsigned bits0 = (unsigned)B.u(m.off + 1, 1);
            little = (bits0 & 1u) == 0;
            is_signed = dtype_class == 0 && (bits0 & 8u);
            dtype_size = B.u(m.off + 4, 4);
        } else if (m.type == 0x0008) {                             // data layout
            const std::string bad = "dataset " + name + ": bad layout message";
            if (!fits(m, 0, 3)) { err = bad; return false; }
            const unsigned ver = (unsigned)B.u(m.off, 1);
            if (ver == 3 && B.u(m.off + 1, 1) == 1) {
                if (!fits(m, 2, 16)) { err = bad; return false; }
                data_addr = B.u(m.off + 2, 8);
                data_size = B.u(m.off + 10, 8);
            } else if (ver == 3 && B.u(m.off + 1, 1) == 0) {      // compact
                if (!fits(m, 2, 2)) { err = bad; return false; }
                data_size = B.u(m.off + 2, 2);
                data_addr = m.off + 4;
                if (!fits(m, 4, data_size)) { err = bad; return false; }
            } else if (ver == 3 && B.u(m.off + 1, 1) == 2) {      // chunked: B-tree, chunk dims
                const unsigned nd = (unsigned)B.u(m.off + 2, 1);
                if (nd > 33 || !fits(m, 3, 8 + 4ull * nd)) { err = bad; return false; }
                data_addr = B.u(m.off + 3, 8);
                for (unsigned i = 0; i < nd; i++) cdim.push_back(B.u(m.off + 11 + 4ull * i, 4));
                chunked = true;
            } else if ((ver == 1 || ver == 2) && B.u(m.off + 2, 1) == 2) {
                const unsigned nd = (unsigned)B.u(m.off + 1, 1);
                if (nd > 33 || !fits(m, 8, 8 + 4ull * nd)) { err = bad; return false; }
                data_addr = B.u(m.off + 8, 8);
                for (unsigned i = 0; i < nd; i++) cdim.push_back(B.u(m.off + 16 + 4ull * i, 4));
                chunked = true;
            } else if ((ver == 1 || ver == 2) && B.u(m.off + 2, 1) == 1) {
                // version 1/2: rank+1 4-byte dimensions (last = element size) after the address
                const unsigned r = (unsigned)B.u(m.off + 1, 1);
                if (r > 33 || !fits(m, 8, 8 + 4ull * r)) { err = bad; return false; }
                data_addr = B.u(m.off + 8, 8);
                data_size = 1;
                for (unsigned i = 0; i < r; i++)
                    if (!mul_ok(data_size, B.u(m.off + 16 + 4ull * i, 4), data_size)) {
                        err = bad;
                        return false;
                    }
            } else if ((ver == 1 || ver == 2) && B.u(m.off + 2, 1) == 0) {
                const unsigned r = (unsigned)B.u(m.off + 1, 1);
                const uint64_t rel = 8 + 4ull * r;
                if (r > 33 || !fits(m, rel, 4)) { err = bad; return false; }
                data_size = B.u(m.off + rel, 4);
                data_addr = m.off + rel + 4;
                if (!fits(m, rel + 4, data_size)) { err = bad; return false; }
            } else {
                err = "dataset " + name + ": unsupported storage layout";
                return false;
            }
        }
    }
    if (!little) { err = "big-endian data are not supported"; return false; }
    uint64_t count = 1, nbytes = 0;
    for (uint64_t d : out.dims)
        if (!mul_ok(count, d, count)) { err = "dataset " + name + ": bad dimensions"; return false; }
    // a file cannot hold more than deflate's ~1032:1 expansion of its own size (unwritten
    // datasets and chunks aside, which get 1 GiB): a damaged size field fails here instead of
    // allocating
    const uint64_t limit = std::min<uint64_t>(kMaxDatasetBytes,
                                              std::max<uint64_t>(1ull << 30, 1100ull * bytes.size()));
    if (!mul_ok(count, dtype_size, nbytes) || nbytes > limit) {
        err = "dataset " + name + ": size " + std::to_string(nbytes) +
              " bytes is impossible for a file of " + std::to_string(bytes.size()) + " bytes";
        return false;
    }
    if (dtype_class == 0 && dtype_size == 1) out.type = is_signed ? kI8 : kU8;
    else if (dtype_class == 0 && dtype_size == 2) out.type = is_signed ? kI16 : kU16;
    else if (dtype_class == 0 && dtype_size == 4) out.type = is_signed ? kI32 : kU32;
    else if (dtype_class == 0 && dtype_size == 8) out.type = is_signed ? kI64 : kU64;
    else if (dtype_class == 1 && dtype_size == 4) out.type = kF32;
    else if (dtype_class == 1 && dtype_size == 8) out.type = kF64;
    else { err = "dataset " + name + ": unsupported datatype"; return false; }
    if (!with_data) return true;
    if (chunked) {
        if (!read_chunked(B, out.dims, dtype_size, data_addr, cdim, filters, out.data, err)) {
            err = "dataset " + name + ": " + err;
            return false;
        }
        return true;
    }
    if (!filters.empty()) { err = "dataset " + name + ": filters on a contiguous dataset"; return false; }
    if (data_addr == kUndef) {                                     // never written: zeros
        out.data.assign(count * dtype_size, 0);
        return true;
    }
    if (data_size < count * dtype_size || !B.ok(data_addr, count * dtype_size)) {
        err = "dataset " + name + ": data outside the file";
        return false;
    }
    out.data.assign(bytes.data() + data_addr, bytes.data() + data_addr + count * dtype_size);
    return true;
}

}  // namespace

// Any allocation failure (a damaged file can claim a huge dataset) becomes an error, never an
// exception across the C ABI.
bool read(const std::string &file, const std::string &name, Dataset &out, std::string &err,
          bool with_data) {
    try {
        return read_impl(file, name, out, err, with_data);
    } catch (const std::exception &e) {
        out = Dataset{};
        err = "dataset " + name + " in " + file + ": " + e.what();
        return false;
    }
}

bool list(const std::string &file, std::vector<std::string> &names, std::string &err) {
    MappedFile mf;
    if (!mf.open(file, err)) return false;
    Buf B{mf.view};
    std::vector<std::pair<std::string, uint64_t>> ents;
    if (!root_entries(B, ents, err)) return false;
    names.clear();
    for (auto &e : ents) names.push_back(e.first);
    return true;
}

bool exists(const std::string &file, const std::string &name) {
    std::string err;
    MappedFile mf;
    if (!mf.open(file, err)) return false;
    Buf B{mf.view};
    std::vector<std::pair<std::string, uint64_t>> ents;
    if (!root_entries(B, ents, err)) return false;
    for (auto &e : ents)
        if (e.first == name) return true;
    return false;
}

// ---- writer ---------------------------------------------------------------------------------
namespace {

struct Out {
    std::vector<char> b;
    uint64_t pos() const { return b.size(); }
    void u(uint64_t v, int n) {
        for (int i = 0; i < n; i++) b.push_back((char)((v >> (8 * i)) & 0xff));
    }
    void bytes(const void *p, size_t n) { b.insert(b.end(), (const char *)p, (const char *)p + n); }
    void pad8() {
        while (b.size() % 8) b.push_back(0);
    }
    void put(uint64_t at, uint64_t v, int n) {
        for (int i = 0; i < n; i++) b[at + i] = (char)((v >> (8 * i)) & 0xff);
    }
};

void msg(Out &o, uint16_t type, const std::vector<char> &data, uint8_t flags = 0) {
    o.u(type, 2);
    const size_t sz = (data.size() + 7) & ~size_t(7);
    o.u(sz, 2);
    o.u(flags, 1);
    o.u(0, 3);
    o.bytes(data.data(), data.size());
    for (size_t i = data.size(); i < sz; i++) o.b.push_back(0);
}

std::vector<char> le(uint64_t v, int n) {
    std::vector<char> r;
    for (int i = 0; i < n; i++) r.push_back((char)((v >> (8 * i)) & 0xff));
    return r;
}
void app(std::vector<char> &a, const std::vector<char> &b) { a.insert(a.end(), b.begin(), b.end()); }

}  // namespace

bool write(const std::string &file, const std::vector<std::pair<std::string, Dataset>> &sets,
           std::string &err) {
    constexpr unsigned kLeafK = 4, kInternalK = 16;
    if (sets.size() > 2 * kLeafK) { err = "too many datasets for one symbol table node"; return false; }
    std::vector<std::pair<std::string, const Dataset *>> sorted;
    for (auto &s : sets) sorted.push_back({s.first, &s.second});
    std::sort(sorted.begin(), sorted.end(), [](auto &a, auto &b) { return a.first < b.first; });

    Out o;
    // superblock (version 0); addresses patched at the end
    o.bytes(kSig, 8);
    o.u(0, 1); o.u(0, 1); o.u(0, 1); o.u(0, 1);      // versions, reserved
    o.u(0, 1); o.u(8, 1); o.u(8, 1); o.u(0, 1);      // shared header version, offsets, lengths
    o.u(kLeafK, 2); o.u(kInternalK, 2);
    o.u(0, 4);                                         // consistency flags
    o.u(0, 8);                                         // base address
    o.u(kUndef, 8);                                    // free-space info
    const uint64_t at_eof = o.pos();
    o.u(0, 8);                                         // end of file address
    o.u(kUndef, 8);                                    // driver information
    // root group symbol table entry
    o.u(0, 8);
    const uint64_t at_root_ohdr = o.pos();
    o.u(0, 8);
    o.u(1, 4);                                         // cache type 1: B-tree + heap in scratch
    o.u(0, 4);
    const uint64_t at_scratch = o.pos();
    o.u(0, 8);
    o.u(0, 8);

    // local heap: data segment = "" + names (8-byte aligned)
    std::vector<char> heap(8, 0);
    std::vector<uint64_t> name_off;
    for (auto &s : sorted) {
        name_off.push_back(heap.size());
        heap.insert(heap.end(), s.first.begin(), s.first.end());
        heap.push_back(0);
        while (heap.size() % 8) heap.push_back(0);
    }
    heap.resize(std::max<size_t>(heap.size(), 88), 0);
    o.pad8();
    const uint64_t heap_addr = o.pos();
    o.bytes("HEAP", 4);
    o.u(0, 1); o.u(0, 3);
    o.u(heap.size(), 8);
    o.u(kUndef, 8);                                    // no free list
    o.u(heap_addr + 32, 8);
    o.bytes(heap.data(), heap.size());

    // data of every dataset, then its object header
    std::vector<uint64_t> ohdr(sorted.size());
    for (size_t i = 0; i < sorted.size(); i++) {
        const Dataset &d = *sorted[i].second;
        if (!valid_type(d.type)) { err = "dataset " + sorted[i].first + ": unknown type"; return false; }
        const uint64_t esz = type_size(d.type);
        uint64_t count = 1;
        for (uint64_t x : d.dims) count *= x;
        if (d.data.size() != count * esz) { err = "dataset " + sorted[i].first + ": size mismatch"; return false; }
        o.pad8();
        const uint64_t data_addr = count ? o.pos() : kUndef;
        o.bytes(d.data.data(), d.data.size());
        o.pad8();
        std::vector<char> sp{1, (char)d.dims.size(), 0, 0, 0, 0, 0, 0};
        for (uint64_t x : d.dims) app(sp, le(x, 8));
        std::vector<char> dt;
        if (!is_float(d.type)) {                           // version 1, fixed-point, LE
            dt = {0x10, (char)(is_signed_int(d.type) ? 0x08 : 0), 0, 0};
            app(dt, le(esz, 4));
            app(dt, le(0, 2));                             // bit offset
            app(dt, le(8 * esz, 2));                       // bit precision
        } else {
            const bool f32 = d.type == kF32;
            dt = {0x11, 0x20, (char)(f32 ? 31 : 63), 0};   // version 1, IEEE float, LE
            app(dt, le(f32 ? 4 : 8, 4));
            app(dt, le(0, 2));
            app(dt, le(f32 ? 32 : 64, 2));
            dt.push_back((char)(f32 ? 23 : 52));           // exponent location
            dt.push_back((char)(f32 ? 8 : 11));            // exponent size
            dt.push_back(0);                               // mantissa location
            dt.push_back((char)(f32 ? 23 : 52));           // mantissa size
            app(dt, le(f32 ? 127 : 1023, 4));
        }
        std::vector<char> fill{2, 1, 2, 0};                // version 2, early alloc, fill if set, undefined
        std::vector<char> lay{3, 1};
        app(lay, le(data_addr, 8));
        app(lay, le(count * esz, 8));
        ohdr[i] = o.pos();
        o.u(1, 1); o.u(0, 1);
        o.u(4, 2);                                         // messages
        o.u(1, 4);                                         // reference count
        const uint64_t at_size = o.pos();
        o.u(0, 4);
        o.u(0, 4);                                         // alignment padding
        const uint64_t start = o.pos();
        msg(o, 0x0001, sp);
        msg(o, 0x0003, dt, 1);                             // constant
        msg(o, 0x0005, fill, 1);
        msg(o, 0x0008, lay);
        o.put(at_size, o.pos() - start, 4);
    }

    // symbol table node with all entries, then the B-tree leaf that points to it
    o.pad8();
    const uint64_t snod = o.pos();
    o.bytes("SNOD", 4);
    o.u(1, 1); o.u(0, 1);
    o.u(sorted.size(), 2);
    for (unsigned k = 0; k < 2 * kLeafK; k++) {
        if (k < sorted.size()) {
            o.u(name_off[k], 8);
            o.u(ohdr[k], 8);
        } else {
            o.u(0, 8);
            o.u(0, 8);
        }
        o.u(0, 4); o.u(0, 4);
        o.u(0, 8); o.u(0, 8);
    }
    const uint64_t btree = o.pos();
    o.bytes("TREE", 4);
    o.u(0, 1);                                         // group node
    o.u(0, 1);                                         // leaf
    o.u(sorted.empty() ? 0 : 1, 2);
    o.u(kUndef, 8);
    o.u(kUndef, 8);
    o.u(0, 8);                                         // key 0: ""
    o.u(snod, 8);                                      // child 0
    o.u(sorted.empty() ? 0 : name_off.back(), 8);      // key 1: largest name
    for (unsigned k = 1; k < 2 * kInternalK; k++) {    // unused slots of a full-size node
        o.u(0, 8);
        o.u(0, 8);
    }

    // root group object header: symbol table message
    o.pad8();
    const uint64_t root = o.pos();
    o.u(1, 1); o.u(0, 1);
    o.u(1, 2);
    o.u(1, 4);
    const uint64_t at_rsize = o.pos();
    o.u(0, 4);
    o.u(0, 4);
    const uint64_t rstart = o.pos();
    std::vector<char> stab = le(btree, 8);
    app(stab, le(heap_addr, 8));
    msg(o, 0x0011, stab);
    o.put(at_rsize, o.pos() - rstart, 4);

    o.put(at_root_ohdr, root, 8);
    o.put(at_scratch, btree, 8);
    o.put(at_scratch + 8, heap_addr, 8);
    o.put(at_eof, o.pos(), 8);

    std::ofstream f(file, std::ios::binary | std::ios::trunc);
    if (!f) { err = "cannot write " + file; return false; }
    f.write(o.b.data(), (std::streamsize)o.b.size());
    if (!f) { err = "write failed: " + file; return false; }
    return true;
}

}  // namespace h5
}  // namespace sw
