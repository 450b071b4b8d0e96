// Reader of TSDF map files in the reference's HDF5 layout, without the HDF5
// library.  The reference writes them through HighFive (GlobalMap,
// src/util/global_map.cpp:12-170: group "/map", one dataset per chunk named
// "<x>_<y>_<z>", edge^3 uint32 cells, tsdf.h:11-33) and reads them back in
// createTSDFMap (include/tsdf_localization/map/map_util.h:17-113): the
// group's names in listing order (by name), split at '_', each part
// converted with std::stoi.
//
// The structures read are those of the published HDF5 file format
// specification: superblock versions 0 to 3; object header versions 1 and 2
// with their continuation blocks; groups stored as symbol tables (version 1
// B-tree of group nodes, local heap, symbol table nodes) or as compact link
// messages; dataspace, datatype (class, size and byte order; a map chunk must
// be 4-byte fixed point), fill value and data layout (contiguous or compact)
// messages.  Dense link storage, chunked, filtered or external datasets are
// reported as unsupported.  The checksums of the version 2 structures read
// (superblock versions 2 and 3, version 2 object headers and their
// continuation blocks) are verified: the format's metadata checksum is Bob
// Jenkins' lookup3 hash ("hashlittle", published 2006) of the structure's
// bytes with initial value 0.
#include <algorithm>
#include <cctype>
#include <cerrno>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include <sys/types.h>

#include "map_host.h"
#include "tsdfl.h"

namespace tsdfl {
namespace {

constexpr uint64_t kUndef = ~0ull;
constexpr int kMaxDepth = 64;            // B-tree levels followed
constexpr size_t kMaxBlocks = 1u << 16;  // continuation blocks of one object header
constexpr size_t kMaxNodes = 1u << 20;   // B-tree and symbol table nodes visited per group
constexpr uint64_t kMaxCells = 1ull << 32;   // cells of one chunk that has no stored data

struct H5Error {
    int code;
    std::string msg;
};

[[noreturn]] void fail(int code, const std::string& msg) { throw H5Error{code, msg}; }

uint64_t le(const uint8_t* p, int n)
{
    uint64_t v = 0;
    for (int i = n - 1; i >= 0; --i) v = (v << 8) | p[i];
    return v;
}

// lookup3's hashlittle (Jenkins 2006), byte by byte: the metadata checksum of
// the HDF5 file format for every version 2 structure.
uint32_t lookup3(const uint8_t* k, size_t n, uint32_t init)
{
    auto rot = [](uint32_t x, int r) { return (x << r) | (x >> (32 - r)); };
    uint32_t a, b, c;
    a = b = c = 0xdeadbeefu + (uint32_t)n + init;
    auto word = [&](const uint8_t* p, size_t m) {   // up to 4 bytes, little-endian
        uint32_t v = 0;
        for (size_t i = 0; i < m; ++i) v |= (uint32_t)p[i] << (8 * i);
        return v;
    };
    while (n > 12) {
        a += word(k, 4);
        b += word(k + 4, 4);
        c += word(k + 8, 4);
        a -= c; a ^= rot(c, 4);  c += b;
        b -= a; b ^= rot(a, 6);  a += c;
        c -= b; c ^= rot(b, 8);  b += a;
        a -= c; a ^= rot(c, 16); c += b;
        b -= a; b ^= rot(a, 19); a += c;
        c -= b; c ^= rot(b, 4);  b += a;
        n -= 12;
        k += 12;
    }
    if (n == 0) return c;
    a += word(k, n < 4 ? n : 4);
    if (n > 4) b += word(k + 4, n < 8 ? n - 4 : 4);
    if (n > 8) c += word(k + 8, n - 8);
    c ^= b; c -= rot(b, 14);
    a ^= c; a -= rot(c, 11);
    b ^= a; b -= rot(a, 25);
    c ^= b; c -= rot(b, 16);
    a ^= c; a -= rot(c, 4);
    b ^= a; b -= rot(a, 14);
    c ^= b; c -= rot(b, 24);
    return c;
}

struct Msg {
    uint16_t type;
    uint64_t pos;    // absolute file position of the message data
    uint32_t size;
};

struct DatasetInfo {
    std::vector<uint64_t> dims;   // dataspace extents, slowest first
    uint64_t count = 0;     // elements
    int type_class = -1;    // datatype class: 0 fixed point, 1 floating point, ...
    uint32_t elem = 0;      // bytes per element
    uint64_t address = kUndef;   // absolute file position of the data, kUndef: none stored
    bool big_endian = false;
    uint32_t fill = 0;      // fill value of a 4-byte type
    std::vector<uint8_t> compact;   // compact layout: the data itself
};

class H5File {
public:
    explicit H5File(const char* path)
    {
        f_ = std::fopen(path, "rb");
        if (!f_) fail(TSDFL_ERR_INVALID_ARG, std::string("cannot open ") + path);
        if (std::fseek(f_, 0, SEEK_END) != 0) fail(TSDFL_ERR_INVALID_ARG, "cannot seek");
        const long long sz = (long long)ftello(f_);
        if (sz < 0) fail(TSDFL_ERR_INVALID_ARG, "cannot tell the file size");
        size_ = (uint64_t)sz;
        superblock();
    }
    ~H5File()
    {
        if (f_) std::fclose(f_);
    }
    H5File(const H5File&) = delete;
    H5File& operator=(const H5File&) = delete;

    uint64_t root() const { return root_; }

    void read(uint64_t pos, void* dst, size_t n) const
    {
        if (pos > size_ || n > size_ - pos) fail(TSDFL_ERR_INVALID_ARG, "truncated file (read past its end)");
        if (fseeko(f_, (off_t)pos, SEEK_SET) != 0 || std::fread(dst, 1, n, f_) != n)
            fail(TSDFL_ERR_INVALID_ARG, "read error");
    }

    // Absolute position of a file address (addresses are relative to the base).
    uint64_t at(uint64_t addr) const
    {
        if (addr == kUndef || addr > size_ || base_ > size_ - addr) fail(TSDFL_ERR_INVALID_ARG, "address outside the file");
        return base_ + addr;
    }

    uint64_t addr(const uint8_t* p) const
    {
        const uint64_t v = le(p, so_);
        return (so_ == 8 ? v == kUndef : v == (1ull << (8 * so_)) - 1) ? kUndef : v;
    }
    uint64_t len(const uint8_t* p) const { return le(p, sl_); }
    int so() const { return so_; }
    int sl() const { return sl_; }

    // All messages of the object header at addr, continuation blocks included.
    std::vector<Msg> messages(uint64_t addr) const
    {
        std::vector<Msg> out;
        const uint64_t pos = at(addr);
        uint8_t h[16] = {};
        read(pos, h, std::min<uint64_t>(16, size_ - pos));
        std::vector<std::pair<uint64_t, uint64_t>> blocks;   // (start, end) of message regions
        bool v2 = false;
        uint8_t flags = 0;
        if (std::memcmp(h, "OHDR", 4) == 0) {
            if (h[4] != 2) fail(TSDFL_ERR_UNSUPPORTED, "object header version " + std::to_string(h[4]));
            v2 = true;
            flags = h[5];
            uint64_t q = 6;
            if (flags & 0x20) q += 16;   // access, modification, change, birth times
            if (flags & 0x10) q += 4;    // attribute storage phase change values
            const int w = 1 << (flags & 3);
            uint8_t s[8] = {};
            read(pos + q, s, (size_t)w);
            const uint64_t chunk0 = le(s, w);
            q += (uint64_t)w;
            if (chunk0 > size_ || pos + q + chunk0 + 4 > size_)
                fail(TSDFL_ERR_INVALID_ARG, "object header chunk larger than the file");
            verify_checksum(pos, q + chunk0, "object header");
            blocks.push_back({pos + q, pos + q + chunk0});
        } else if (h[0] == 1) {
            const uint64_t hsize = le(h + 8, 4);
            blocks.push_back({pos + 16, pos + 16 + hsize});   // 12-byte prefix padded to 8
        } else {
            fail(TSDFL_ERR_UNSUPPORTED, "object header version " + std::to_string(h[0]));
        }
        const uint64_t prefix = v2 ? ((flags & 0x04) ? 6u : 4u) : 8u;
        for (size_t b = 0; b < blocks.size(); ++b) {
            if (blocks.size() > kMaxBlocks) fail(TSDFL_ERR_INVALID_ARG, "too many object header blocks");
            const uint64_t start = blocks[b].first, end = blocks[b].second;
            if (end > size_ || end < start) fail(TSDFL_ERR_INVALID_ARG, "object header block outside the file");
            std::vector<uint8_t> buf((size_t)(end - start));
            read(start, buf.data(), buf.size());
            uint64_t p = 0;
            while (p + prefix <= buf.size()) {
                const uint8_t* m = buf.data() + p;
                uint16_t type;
                uint32_t msize;
                if (v2) {
                    type = m[0];
                    msize = (uint32_t)le(m + 1, 2);
                } else {
                    type = (uint16_t)le(m, 2);
                    msize = (uint32_t)le(m + 2, 2);
                }
                if (p + prefix + msize > buf.size()) fail(TSDFL_ERR_INVALID_ARG, "object header message overruns its block");
                const uint64_t data = start + p + prefix;
                if (type == 0x10) {   // continuation: the next block of messages
                    if (msize < (uint32_t)(so_ + sl_)) fail(TSDFL_ERR_INVALID_ARG, "short continuation message");
                    const uint64_t cpos = at(addr_of(m + prefix));
                    const uint64_t clen = len(m + prefix + so_);
                    if (v2) {
                        uint8_t sig[4];
                        read(cpos, sig, 4);
                        if (std::memcmp(sig, "OCHK", 4) != 0 || clen < 8 || cpos + clen > size_)
                            fail(TSDFL_ERR_INVALID_ARG, "bad object header continuation block");
                        verify_checksum(cpos, clen - 4, "object header continuation block");
                        blocks.push_back({cpos + 4, cpos + clen - 4});   // signature .. checksum
                    } else {
                        blocks.push_back({cpos, cpos + clen});
                    }
                } else if (type != 0) {   // 0: NIL (padding)
                    out.push_back(Msg{type, data, msize});
                }
                p += prefix + msize;
                if (!v2) p = (p + 7) & ~7ull;   // version 1 messages are 8-byte aligned
            }
        }
        return out;
    }

    std::vector<uint8_t> data(const Msg& m) const
    {
        std::vector<uint8_t> d(m.size);
        if (m.size) read(m.pos, d.data(), m.size);
        return d;
    }

    // The hard links of the group whose object header is at addr: (name, object header address).
    std::vector<std::pair<std::string, uint64_t>> links(uint64_t addr) const
    {
        std::vector<std::pair<std::string, uint64_t>> out;
        for (const Msg& m : messages(addr)) {
            const std::vector<uint8_t> d = data(m);
            if (m.type == 0x11) {   // symbol table: v1 B-tree + local heap
                if (d.size() < (size_t)(2 * so_)) fail(TSDFL_ERR_INVALID_ARG, "short symbol table message");
                symbol_table(addr_of(d.data()), addr_of(d.data() + so_), out);
            } else if (m.type == 0x02) {   // link info: dense storage lives in a fractal heap
                if (d.size() < 2) fail(TSDFL_ERR_INVALID_ARG, "short link info message");
                const size_t q = 2 + ((d[1] & 1) ? 8 : 0);
                if (d.size() < q + (size_t)so_) fail(TSDFL_ERR_INVALID_ARG, "short link info message");
                if (addr_of(d.data() + q) != kUndef)
                    fail(TSDFL_ERR_UNSUPPORTED, "groups with dense link storage");
            } else if (m.type == 0x06) {   // link
                link_message(d, out);
            }
        }
        return out;
    }

    uint64_t child(uint64_t group, const std::string& name) const
    {
        for (const auto& l : links(group))
            if (l.first == name) return l.second;
        fail(TSDFL_ERR_INVALID_ARG, "no object \"" + name + "\"");
    }

    // The dataset whose object header is at addr: its dataspace, element type
    // and storage, checked against the file's size.
    DatasetInfo describe(uint64_t addr) const
    {
        DatasetInfo info;
        bool have_space = false, have_type = false, have_layout = false;
        uint64_t layout_size = 0;
        for (const Msg& m : messages(addr)) {
            const std::vector<uint8_t> d = data(m);
            auto need = [&](size_t n) {
                if (d.size() < n) fail(TSDFL_ERR_INVALID_ARG, "short message of type " + std::to_string(m.type));
            };
            switch (m.type) {
            case 0x01: {   // dataspace
                need(4);
                const int ver = d[0], rank = d[1];
                size_t q;
                uint64_t n = 1;
                if (ver == 1) {
                    q = 8;
                } else if (ver == 2) {
                    q = 4;
                    if (d[3] == 2) n = 0;   // null dataspace
                } else {
                    fail(TSDFL_ERR_UNSUPPORTED, "dataspace version " + std::to_string(ver));
                }
                need(q + (size_t)rank * sl_);
                info.dims.clear();
                for (int r = 0; r < rank; ++r) {
                    const uint64_t dim = len(d.data() + q + (size_t)r * sl_);
                    if (dim && n > UINT64_MAX / dim) fail(TSDFL_ERR_INVALID_ARG, "dataspace too large");
                    n *= dim;
                    info.dims.push_back(dim);
                }
                info.count = n;
                have_space = true;
                break;
            }
            case 0x03: {   // datatype
                need(8);
                info.type_class = d[0] & 0x0f;
                info.elem = (uint32_t)le(d.data() + 4, 4);
                if (info.elem == 0) fail(TSDFL_ERR_INVALID_ARG, "datatype of 0 bytes");
                info.big_endian = (d[1] & 1) != 0;   // byte order of the fixed- and floating-point classes
                have_type = true;
                break;
            }
            case 0x04: {   // old fill value: size, value
                need(4);
                if (le(d.data(), 4) == 4 && d.size() >= 8) info.fill = (uint32_t)le(d.data() + 4, 4);
                break;
            }
            case 0x05: {   // fill value
                need(1);
                size_t q = 0;
                bool defined = false;
                if (d[0] == 1 || d[0] == 2) {
                    need(4);
                    defined = d[3] != 0 || d[0] == 1;
                    q = 4;
                } else if (d[0] == 3) {
                    need(2);
                    defined = (d[1] & 0x20) != 0;
                    q = 2;
                } else {
                    fail(TSDFL_ERR_UNSUPPORTED, "fill value message version " + std::to_string(d[0]));
                }
                if (defined && d.size() >= q + 4 && le(d.data() + q, 4) == 4 && d.size() >= q + 8)
                    info.fill = (uint32_t)le(d.data() + q + 4, 4);
                break;
            }
            case 0x07:
                fail(TSDFL_ERR_UNSUPPORTED, "datasets in external files");
            case 0x0B: {   // filter pipeline
                need(2);
                if (d[1] != 0) fail(TSDFL_ERR_UNSUPPORTED, "filtered (compressed) datasets");
                break;
            }
            case 0x08: {   // data layout
                need(2);
                const int ver = d[0];
                if (ver == 3 || ver == 4) {
                    const int cls = d[1];
                    if (cls == 0) {
                        need(4);
                        const size_t cs = (size_t)le(d.data() + 2, 2);
                        need(4 + cs);
                        info.compact.assign(d.begin() + 4, d.begin() + 4 + (long)cs);
                        layout_size = cs;
                    } else if (cls == 1) {
                        need(2 + (size_t)so_ + (size_t)sl_);
                        const uint64_t a = addr_of(d.data() + 2);
                        info.address = a == kUndef ? kUndef : at(a);
                        layout_size = len(d.data() + 2 + so_);
                    } else {
                        fail(TSDFL_ERR_UNSUPPORTED, "chunked or virtual dataset layout");
                    }
                } else if (ver == 1 || ver == 2) {
                    need(8);
                    const int rank = d[1], cls = d[2];
                    size_t q = 8;
                    if (cls == 2) fail(TSDFL_ERR_UNSUPPORTED, "chunked dataset layout");
                    if (cls == 1) {
                        need(q + (size_t)so_);
                        const uint64_t a = addr_of(d.data() + q);
                        info.address = a == kUndef ? kUndef : at(a);
                        q += (size_t)so_;
                    }
                    need(q + 4u * (size_t)rank);
                    q += 4u * (size_t)rank;
                    layout_size = UINT64_MAX;   // the dataspace decides
                    if (cls == 0) {
                        need(q + 4);
                        const size_t cs = (size_t)le(d.data() + q, 4);
                        need(q + 4 + cs);
                        info.compact.assign(d.begin() + (long)q + 4, d.begin() + (long)(q + 4 + cs));
                        layout_size = cs;
                    }
                } else {
                    fail(TSDFL_ERR_UNSUPPORTED, "data layout version " + std::to_string(ver));
                }
                have_layout = true;
                break;
            }
            default:
                break;
            }
        }
        if (!have_space || !have_type || !have_layout) fail(TSDFL_ERR_INVALID_ARG, "object is not a dataset");
        const uint64_t e = info.elem;
        if (info.count > UINT64_MAX / e || (layout_size != UINT64_MAX && layout_size < e * info.count))
            fail(TSDFL_ERR_INVALID_ARG, "dataset storage smaller than its dataspace");
        if (info.address != kUndef && (info.address > size_ || e * info.count > size_ - info.address))
            fail(TSDFL_ERR_INVALID_ARG, "dataset storage outside the file");
        if (info.address == kUndef && info.compact.empty() && info.count > kMaxCells)
            fail(TSDFL_ERR_INVALID_ARG, "dataset without storage larger than a chunk can be");
        return info;
    }

    // A map chunk: a dataset of 4-byte integers (tsdf.h:11-33, TSDFValue's raw word).
    DatasetInfo dataset(uint64_t addr) const
    {
        DatasetInfo info = describe(addr);
        if (info.type_class != 0) fail(TSDFL_ERR_UNSUPPORTED, "datasets of a non-integer type");
        if (info.elem != 4) fail(TSDFL_ERR_UNSUPPORTED, "integers of other than 4 bytes");
        return info;
    }

    // The dataset's elements as uint32 in host order.
    void read_dataset(const DatasetInfo& info, uint32_t* out) const
    {
        const size_t n = (size_t)info.count;
        if (!info.compact.empty()) {
            std::memcpy(out, info.compact.data(), 4 * n);
        } else if (info.address == kUndef) {   // never written: the fill value
            std::fill(out, out + n, info.fill);
            return;
        } else {
            read(info.address, out, 4 * n);
        }
        for (size_t i = 0; i < n; ++i) {   // file bytes -> value, independent of the host's byte order
            const uint8_t* b = reinterpret_cast<const uint8_t*>(out + i);
            out[i] = info.big_endian ? ((uint32_t)b[0] << 24 | (uint32_t)b[1] << 16 | (uint32_t)b[2] << 8 | b[3])
                                     : ((uint32_t)b[3] << 24 | (uint32_t)b[2] << 16 | (uint32_t)b[1] << 8 | b[0]);
        }
    }

private:
    uint64_t addr_of(const uint8_t* p) const { return addr(p); }

    // The n bytes at pos are followed by their lookup3 checksum.
    void verify_checksum(uint64_t pos, uint64_t n, const char* what) const
    {
        if (n > (1ull << 30) || pos + n + 4 > size_) fail(TSDFL_ERR_INVALID_ARG, std::string(what) + " outside the file");
        std::vector<uint8_t> buf((size_t)n + 4);
        read(pos, buf.data(), buf.size());
        if (lookup3(buf.data(), (size_t)n, 0) != (uint32_t)le(buf.data() + n, 4))
            fail(TSDFL_ERR_INVALID_ARG, std::string(what) + " checksum mismatch");
    }

    void superblock()
    {
        static const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
        uint64_t pos = 0;
        for (;;) {   // at 0, 512, 1024, 2048, ...
            if (pos + 8 > size_) fail(TSDFL_ERR_INVALID_ARG, "not an HDF5 file (no superblock)");
            uint8_t s[8];
            read(pos, s, 8);
            if (std::memcmp(s, sig, 8) == 0) break;
            pos = pos ? 2 * pos : 512;
        }
        uint8_t sb[160] = {};
        read(pos, sb, (size_t)std::min<uint64_t>(sizeof(sb), size_ - pos));
        const int ver = sb[8];
        if (ver == 0 || ver == 1) {
            so_ = sb[13];
            sl_ = sb[14];
            check_sizes();
            size_t q = 24 + (ver == 1 ? 4 : 0);
            base_ = le(sb + q, so_);
            q += 4 * (size_t)so_;                 // base, free space, end of file, driver information
            root_ = addr(sb + q + so_);          // root symbol table entry: name offset, header address
        } else if (ver == 2 || ver == 3) {
            so_ = sb[9];
            sl_ = sb[10];
            check_sizes();
            verify_checksum(pos, 12 + 4 * (uint64_t)so_, "superblock");
            base_ = le(sb + 12, so_);
            root_ = addr(sb + 12 + 3 * (size_t)so_);   // after base, extension, end of file
        } else {
            fail(TSDFL_ERR_UNSUPPORTED, "superblock version " + std::to_string(ver));
        }
        if (root_ == kUndef) fail(TSDFL_ERR_INVALID_ARG, "no root group");
    }

    void check_sizes() const
    {
        if ((so_ != 2 && so_ != 4 && so_ != 8) || (sl_ != 2 && sl_ != 4 && sl_ != 8))
            fail(TSDFL_ERR_UNSUPPORTED, "sizes of offsets / lengths other than 2, 4 or 8 bytes");
    }

    void symbol_table(uint64_t btree, uint64_t heap, std::vector<std::pair<std::string, uint64_t>>& out) const
    {
        uint8_t h[32] = {};
        const uint64_t hp = at(heap);
        read(hp, h, 8 + 2 * (size_t)sl_ + (size_t)so_);
        if (std::memcmp(h, "HEAP", 4) != 0) fail(TSDFL_ERR_INVALID_ARG, "bad local heap");
        const uint64_t dsize = len(h + 8);
        const uint64_t daddr = addr(h + 8 + 2 * sl_);
        if (dsize > size_) fail(TSDFL_ERR_INVALID_ARG, "local heap larger than the file");
        std::vector<uint8_t> names((size_t)dsize);
        if (dsize) read(at(daddr), names.data(), names.size());
        size_t visited = 0;
        if (btree != kUndef) btree_node(btree, names, out, 0, visited);
    }

    void btree_node(uint64_t node, const std::vector<uint8_t>& names,
                    std::vector<std::pair<std::string, uint64_t>>& out, int depth, size_t& visited) const
    {
        if (depth > kMaxDepth) fail(TSDFL_ERR_INVALID_ARG, "B-tree too deep");
        if (++visited > kMaxNodes) fail(TSDFL_ERR_INVALID_ARG, "B-tree with too many nodes");
        const uint64_t pos = at(node);
        const size_t hdr = 8 + 2 * (size_t)so_;
        uint8_t h[24];
        read(pos, h, hdr);
        if (std::memcmp(h, "TREE", 4) != 0) fail(TSDFL_ERR_INVALID_ARG, "bad B-tree node");
        if (h[4] != 0) fail(TSDFL_ERR_INVALID_ARG, "B-tree node of a group is not a group node");
        const int level = h[5];
        const size_t entries = (size_t)le(h + 6, 2);
        const size_t step = (size_t)sl_ + (size_t)so_;
        std::vector<uint8_t> kc(entries * step + sl_);
        read(pos + hdr, kc.data(), kc.size());
        for (size_t i = 0; i < entries; ++i) {
            const uint64_t c = addr(kc.data() + i * step + sl_);
            if (level > 0) {
                btree_node(c, names, out, depth + 1, visited);
            } else {
                if (++visited > kMaxNodes) fail(TSDFL_ERR_INVALID_ARG, "B-tree with too many nodes");
                symbol_node(c, names, out);
            }
        }
    }

    void symbol_node(uint64_t node, const std::vector<uint8_t>& names,
                     std::vector<std::pair<std::string, uint64_t>>& out) const
    {
        const uint64_t pos = at(node);
        uint8_t h[8];
        read(pos, h, 8);
        if (std::memcmp(h, "SNOD", 4) != 0) fail(TSDFL_ERR_INVALID_ARG, "bad symbol table node");
        const size_t n = (size_t)le(h + 6, 2);
        const size_t es = 2 * (size_t)so_ + 24;   // name offset, header address, cache type, reserved, scratch
        std::vector<uint8_t> e(n * es);
        read(pos + 8, e.data(), e.size());
        for (size_t i = 0; i < n; ++i) {
            const uint64_t off = le(e.data() + i * es, so_);   // into the heap's data segment
            const uint64_t hdr = addr(e.data() + i * es + so_);
            if (off >= names.size()) fail(TSDFL_ERR_INVALID_ARG, "link name outside the local heap");
            const char* s = reinterpret_cast<const char*>(names.data() + off);
            const size_t sl = strnlen(s, names.size() - (size_t)off);
            out.push_back({std::string(s, sl), hdr});
        }
    }

    void link_message(const std::vector<uint8_t>& d, std::vector<std::pair<std::string, uint64_t>>& out) const
    {
        if (d.size() < 2 || d[0] != 1) fail(TSDFL_ERR_UNSUPPORTED, "link message version");
        const uint8_t fl = d[1];
        size_t q = 2;
        int type = 0;
        if (fl & 0x08) type = d.at(q++);
        if (fl & 0x04) q += 8;   // creation order
        if (fl & 0x10) q += 1;   // character set
        const int w = 1 << (fl & 3);
        if (d.size() < q + (size_t)w) fail(TSDFL_ERR_INVALID_ARG, "short link message");
        const uint64_t nl = le(d.data() + q, w);
        q += (size_t)w;
        if (nl > d.size() - q) fail(TSDFL_ERR_INVALID_ARG, "short link message");
        std::string name(reinterpret_cast<const char*>(d.data() + q), (size_t)nl);
        q += (size_t)nl;
        if (type != 0) fail(TSDFL_ERR_UNSUPPORTED, "soft or external link \"" + name + "\"");
        if (d.size() < q + (size_t)so_) fail(TSDFL_ERR_INVALID_ARG, "short link message");
        out.push_back({name, addr(d.data() + q)});
    }

    FILE* f_ = nullptr;
    uint64_t size_ = 0;
    uint64_t base_ = 0;
    uint64_t root_ = kUndef;
    int so_ = 8, sl_ = 8;
};

// createTSDFMap's reading of a chunk name (map_util.h:28-40): parts between
// '_', each converted as std::stoi does (leading white space, a sign, digits;
// the rest of the part ignored).  Three parts are required.
bool parse_tag(const std::string& tag, int32_t out[3])
{
    std::vector<std::string> parts;
    size_t start = 0;
    for (;;) {
        const size_t u = tag.find('_', start);
        parts.push_back(tag.substr(start, u == std::string::npos ? std::string::npos : u - start));
        if (u == std::string::npos) break;
        start = u + 1;
    }
    if (parts.size() != 3) return false;
    for (int a = 0; a < 3; ++a) {
        const char* s = parts[a].c_str();
        char* end = nullptr;
        errno = 0;
        const long v = std::strtol(s, &end, 10);
        if (end == s || errno == ERANGE || v < INT_MIN || v > INT_MAX) return false;
        out[a] = (int32_t)v;
    }
    return true;
}

}  // namespace
}  // namespace tsdfl

extern "C" int tsdfl_read_map_h5(const char* path, int32_t** chunk_pos, uint32_t** chunks, size_t* n_chunks,
                                 int32_t* edge)
{
    using namespace tsdfl;
    if (!path || !chunk_pos || !chunks || !n_chunks || !edge) {
        set_error("tsdfl_read_map_h5: invalid argument");
        return TSDFL_ERR_INVALID_ARG;
    }
    *chunk_pos = nullptr;
    *chunks = nullptr;
    *n_chunks = 0;
    *edge = 0;
    int32_t* pos = nullptr;
    uint32_t* raw = nullptr;
    try {
        H5File f(path);
        std::vector<std::pair<std::string, uint64_t>> items = f.links(f.child(f.root(), "map"));
        // the group's listing order: by name, byte-wise
        std::sort(items.begin(), items.end(),
                  [](const std::pair<std::string, uint64_t>& a, const std::pair<std::string, uint64_t>& b) {
                      return a.first < b.first;
                  });
        std::vector<DatasetInfo> info;
        info.reserve(items.size());
        uint64_t count = 0;
        for (size_t i = 0; i < items.size(); ++i) {
            info.push_back(f.dataset(items[i].second));
            if (i == 0) count = info[0].count;
            else if (info[i].count != count)
                fail(TSDFL_ERR_INVALID_ARG, "chunk \"" + items[i].first + "\" has another size");
        }
        int32_t e = 0;
        if (!items.empty()) {
            e = (int32_t)std::llround(std::cbrt((double)count));
            if (e <= 0 || (uint64_t)e * (uint64_t)e * (uint64_t)e != count)
                fail(TSDFL_ERR_INVALID_ARG, "chunks of " + std::to_string(count) + " cells are not cubes");
        }
        const size_t n = items.size();
        if (n && (uint64_t)count > (uint64_t)(SIZE_MAX / sizeof(uint32_t)) / n)
            fail(TSDFL_ERR_OUT_OF_MEMORY, "map larger than the address space");
        pos = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * 3 * (n ? n : 1)));
        raw = static_cast<uint32_t*>(std::malloc(sizeof(uint32_t) * (n ? n * (size_t)count : 1)));
        if (!pos || !raw) fail(TSDFL_ERR_OUT_OF_MEMORY, "out of host memory");
        for (size_t i = 0; i < n; ++i) {
            if (!parse_tag(items[i].first, pos + 3 * i))
                fail(TSDFL_ERR_INVALID_ARG, "chunk name \"" + items[i].first + "\" is not <x>_<y>_<z>");
            f.read_dataset(info[i], raw + i * (size_t)count);
        }
        *chunk_pos = pos;
        *chunks = raw;
        *n_chunks = n;
        *edge = e;
        return TSDFL_OK;
    } catch (const H5Error& err) {
        std::free(pos);
        std::free(raw);
        set_error("tsdfl_read_map_h5: %s", err.msg.c_str());
        return err.code;
    } catch (const std::bad_alloc&) {
        std::free(pos);
        std::free(raw);
        set_error("tsdfl_read_map_h5: out of host memory");
        return TSDFL_ERR_OUT_OF_MEMORY;
    }
}
