// Minimal HDF5 reader/writer for SpinWalk's phantom and result files, written from the HDF5
// file-format specification (no libhdf5 in this build).
//
// SpinWalk reads and writes whole datasets of the root group (src/sim/h5_helper.h:48-129):
// phantoms hold `mask` (uint8 [Nx,Ny,Nz]), optional `fieldmap` (float [Nx,Ny,Nz]) and `fov`
// (float [3]); optional start files hold `XYZ` / `M` (float [N,3]); results hold M, XYZ, T,
// scales, TE. libhdf5 with default settings stores such files with a version-0 superblock, an
// "old-style" root group (symbol-table message -> version-1 B-tree of group nodes -> symbol table
// nodes, names in a local heap), version-1 object headers and contiguous data. That subset is
// what this file reads (plus continuation blocks and 64-bit floats) and writes.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "sw_h5.h"

namespace sw {
namespace h5 {
namespace {

constexpr uint64_t kUndef = ~uint64_t(0);
const unsigned char kSig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};

struct Buf {
    const std::vector<char> &b;
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
                   std::vector<std::pair<std::string, uint64_t>> &out, std::string &err, int depth = 0) {
    if (depth > 32 || !B.ok(btree, 24) || std::memcmp(&B.b[btree], "TREE", 4) != 0) {
        err = "bad group B-tree";
        return false;
    }
    const unsigned level = (unsigned)B.u(btree + 5, 1), used = (unsigned)B.u(btree + 6, 2);
    uint64_t p = btree + 24 + 8;                 // past the first key
    for (unsigned i = 0; i < used; i++, p += 16) {
        if (!B.ok(p, 8)) { err = "truncated B-tree"; return false; }
        const uint64_t child = B.u(p, 8);
        if (level > 0) {
            if (!group_entries(B, child, heap_data, out, err, depth + 1)) return false;
            continue;
        }
        if (!B.ok(child, 8) || std::memcmp(&B.b[child], "SNOD", 4) != 0) {
            err = "bad symbol table node";
            return false;
        }
        const unsigned ns = (unsigned)B.u(child + 6, 2);
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
        return group_entries(B, btree, B.u(heap + 24, 8), out, err);
    }
    err = "root group has no symbol table (new-style groups are not supported)";
    return false;
}

// Loads the file and drops a user block: the superblock may start at 0, 512, 1024, ...; file
// addresses are relative to it (base address 0 in that frame).
bool load(const std::string &file, std::vector<char> &b, std::string &err) {
    std::ifstream f(file, std::ios::binary);
    if (!f) { err = "cannot open " + file; return false; }
    b.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
    for (uint64_t at = 0; at + 8 <= b.size(); at = at ? 2 * at : 512) {
        if (std::memcmp(b.data() + at, kSig, 8) == 0) {
            if (at) b.erase(b.begin(), b.begin() + (std::ptrdiff_t)at);
            return true;
        }
    }
    err = file + " is not an HDF5 file";
    return false;
}

}  // namespace

bool read(const std::string &file, const std::string &name, Dataset &out, std::string &err) {
    std::vector<char> bytes;
    if (!load(file, bytes, err)) return false;
    Buf B{bytes};
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
    bool little = true, is_signed = false;
    for (const Msg &m : msgs) {
        if (m.type == 0x0001) {                                    // dataspace
            const unsigned ver = (unsigned)B.u(m.off, 1), rank = (unsigned)B.u(m.off + 1, 1);
            const uint64_t p = m.off + (ver == 1 ? 8 : 4);
            for (unsigned i = 0; i < rank; i++) out.dims.push_back(B.u(p + 8ull * i, 8));
        } else if (m.type == 0x0003) {                             // datatype
            dtype_class = (int)(B.u(m.off, 1) & 0x0f);
            const unsigned bits0 = (unsigned)B.u(m.off + 1, 1);
            little = (bits0 & 1u) == 0;
            is_signed = dtype_class == 0 && (bits0 & 8u);
            dtype_size = B.u(m.off + 4, 4);
        } else if (m.type == 0x0008) {                             // data layout
            const unsigned ver = (unsigned)B.u(m.off, 1);
            if (ver == 3 && B.u(m.off + 1, 1) == 1) {
                data_addr = B.u(m.off + 2, 8);
                data_size = B.u(m.off + 10, 8);
            } else if (ver == 3 && B.u(m.off + 1, 1) == 0) {      // compact
                data_size = B.u(m.off + 2, 2);
                data_addr = m.off + 4;
            } else if ((ver == 1 || ver == 2) && B.u(m.off + 2, 1) == 1) {
                // version 1/2: rank+1 4-byte dimensions (last = element size) after the address
                const unsigned r = (unsigned)B.u(m.off + 1, 1);
                data_addr = B.u(m.off + 8, 8);
                data_size = 1;
                for (unsigned i = 0; i < r; i++) data_size *= B.u(m.off + 16 + 4ull * i, 4);
            } else if ((ver == 1 || ver == 2) && B.u(m.off + 2, 1) == 0) {
                const unsigned r = (unsigned)B.u(m.off + 1, 1);
                const uint64_t p = m.off + 8 + 4ull * r;
                data_size = B.u(p, 4);
                data_addr = p + 4;
            } else {
                err = "dataset " + name + ": only contiguous/compact layouts are supported";
                return false;
            }
        }
    }
    if (!little) { err = "big-endian data are not supported"; return false; }
    uint64_t count = 1;
    for (uint64_t d : out.dims) count *= d;
    if (dtype_class == 0 && dtype_size == 1) out.type = is_signed ? kI8 : kU8;
    else if (dtype_class == 0 && dtype_size == 2) out.type = is_signed ? kI16 : kU16;
    else if (dtype_class == 0 && dtype_size == 4) out.type = is_signed ? kI32 : kU32;
    else if (dtype_class == 0 && dtype_size == 8) out.type = is_signed ? kI64 : kU64;
    else if (dtype_class == 1 && dtype_size == 4) out.type = kF32;
    else if (dtype_class == 1 && dtype_size == 8) out.type = kF64;
    else { err = "dataset " + name + ": unsupported datatype"; return false; }
    if (data_addr == kUndef) {                                     // never written: zeros
        out.data.assign(count * dtype_size, 0);
        return true;
    }
    if (data_size < count * dtype_size || !B.ok(data_addr, count * dtype_size)) {
        err = "dataset " + name + ": data outside the file";
        return false;
    }
    out.data.assign(bytes.begin() + data_addr, bytes.begin() + data_addr + count * dtype_size);
    return true;
}

bool list(const std::string &file, std::vector<std::string> &names, std::string &err) {
    std::vector<char> bytes;
    if (!load(file, bytes, err)) return false;
    Buf B{bytes};
    std::vector<std::pair<std::string, uint64_t>> ents;
    if (!root_entries(B, ents, err)) return false;
    names.clear();
    for (auto &e : ents) names.push_back(e.first);
    return true;
}

bool exists(const std::string &file, const std::string &name) {
    std::vector<char> bytes;
    std::string err;
    if (!load(file, bytes, err)) return false;
    Buf B{bytes};
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
