// h5.cpp -- the reference's HDF5 matrix files without libhdf5, behind the C ABI (dimgpu_h5_*).
//
// The reference keeps matrices in HDF5 through libhdf5 (include/dim/io/h5.h:68-115,
// libs/dim/io/h5.cpp:12-74):
//   * a MATLAB-compatible CSR group (write_matlab_compatible / read_matlab_compatible, h5.h:68-97):
//     datasets `data` (f64), `ir` (u32 column indices), `jc` (u32 row offsets) and the scalar u32
//     attribute `MATLAB_sparse` = column count;
//   * a CSR5 group (store / load_csr5, h5.cpp:45-74): the attribute `column_count` and the datasets
//     `vals`, `col_idx`, `row_ptr`, `tile_ptr`, `tile_desc` (an H5T array of 4 u32 per tile, h5.cpp:12-22),
//     `tile_desc_offset_ptr`, `tile_desc_offset`;
//   * result vectors (f64 datasets, benchmarks/csr5/dim/main.cpp:35-43).
// No HDF5 library exists where this is built or run, so this file implements the part of the HDF5 File
// Format Specification these files use, written from the specification:
//   writer -- the layout libhdf5 produces with its default ("earliest") format settings: superblock
//     version 0, version-1 object headers, groups as symbol tables (a version-1 B-tree of symbol-table
//     nodes plus a local heap of names), contiguous datasets, version-1 attributes.  The bytes are the
//     ones the package's Python writer (io/h5.py) produces for the same content, which the tests check.
//   reader -- that layout, plus what libhdf5 writes when the reference's dataset properties ask for
//     chunks and compression (h5.cpp:34-43): chunked 1-D datasets indexed by a version-1 B-tree, the
//     deflate filter (decoded below), and object-header continuation blocks.  Version-2 object headers
//     (files written with libver "latest") are refused with an error.
// Everything here runs on the host.  Failures return DIMGPU_ERR_IO (a file that cannot be read or
// written, or that is not in this subset) or DIMGPU_ERR_INVALID_ARGUMENT, with a message.
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "internal.hpp"

namespace dimgpu {
namespace h5 {
namespace {

constexpr uint8_t kSignature[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
constexpr uint64_t kUndef = ~0ull;
constexpr int kLeafK = 4;          // a symbol-table node holds up to 2K entries
constexpr int kInternalK = 16;     // a group B-tree node holds up to 2K children
constexpr uint64_t kHeapFreeNull = 1;

struct format_error : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct io_error : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// ------------------------------------------------------------------------------------------------
// little-endian bytes
// ------------------------------------------------------------------------------------------------

struct bytes {
    std::vector<uint8_t> b;
    bytes& u8(uint8_t v) {
        b.push_back(v);
        return *this;
    }
    bytes& u16(uint16_t v) { return u8(v & 0xFF).u8(v >> 8); }
    bytes& u32(uint32_t v) { return u16(v & 0xFFFF).u16(v >> 16); }
    bytes& u64(uint64_t v) { return u32((uint32_t)v).u32((uint32_t)(v >> 32)); }
    bytes& zeros(size_t n) {
        b.insert(b.end(), n, 0);
        return *this;
    }
    bytes& raw(const void* p, size_t n) {
        const uint8_t* q = static_cast<const uint8_t*>(p);
        b.insert(b.end(), q, q + n);
        return *this;
    }
    bytes& append(const bytes& o) { return raw(o.b.data(), o.b.size()); }
    bytes& pad8() { return zeros((8 - b.size() % 8) % 8); }
    size_t size() const { return b.size(); }
};

inline uint16_t rd16(const uint8_t* p) { return (uint16_t)(p[0] | (p[1] << 8)); }
inline uint32_t rd32(const uint8_t* p) { return (uint32_t)rd16(p) | ((uint32_t)rd16(p + 2) << 16); }
inline uint64_t rd64(const uint8_t* p) { return (uint64_t)rd32(p) | ((uint64_t)rd32(p + 4) << 32); }

// ------------------------------------------------------------------------------------------------
// element types
// ------------------------------------------------------------------------------------------------

enum class kind : uint8_t { u, i, f };

struct etype {
    kind k = kind::f;
    uint32_t base = 8;   // bytes of the scalar type
    uint32_t inner = 0;  // > 0: an array type of `inner` scalars per dataset element (tile_desc: 4 x u32)
    uint32_t element_bytes() const { return base * (inner ? inner : 1); }
};

const etype kF64{kind::f, 8, 0};
const etype kU32{kind::u, 4, 0};

// Datatype message body (class 0 fixed-point, 1 floating-point, 10 array of either).
bytes datatype_of(const etype& t) {
    bytes s;
    if (t.k == kind::f) {
        if (t.base == 8)
            s.u8(0x11).u8(0x20).u8(63).u8(0).u32(8).u16(0).u16(64).u8(52).u8(11).u8(0).u8(52).u32(1023);
        else if (t.base == 4)
            s.u8(0x11).u8(0x20).u8(31).u8(0).u32(4).u16(0).u16(32).u8(23).u8(8).u8(0).u8(23).u32(127);
        else
            throw format_error("only 4- and 8-byte floats");
    } else {
        s.u8(0x10).u8(t.k == kind::i ? 0x08 : 0x00).u8(0).u8(0).u32(t.base).u16(0).u16((uint16_t)(8 * t.base));
    }
    if (!t.inner)
        return s;
    bytes a;  // array type, version 2: rank, dimensions, permutation, base type
    a.u8(0x2A).u8(0).u8(0).u8(0).u32(t.base * t.inner);
    a.u8(1).zeros(3).u32(t.inner).u32(0);
    return a.append(s);
}

// ------------------------------------------------------------------------------------------------
// in-memory tree of a file (what the writer writes, and what an appending writer reads back first)
// ------------------------------------------------------------------------------------------------

struct attribute {
    std::string name;
    etype t;
    std::vector<uint8_t> value;  // `count` elements
    uint64_t count = 1;
};

struct node {
    bool is_group = true;
    std::vector<std::pair<std::string, std::unique_ptr<node>>> members;  // insertion order
    std::vector<attribute> attrs;                                        // insertion order
    // dataset
    etype t;
    std::vector<uint64_t> shape;
    std::vector<uint8_t> data;
    const uint8_t* ext = nullptr;  // caller-owned bytes to write instead of `data`
    uint64_t ext_bytes = 0;

    node* member(const std::string& name) {
        for (auto& m : members)
            if (m.first == name)
                return m.second.get();
        return nullptr;
    }
    // the member slot `name` (replaced in place when present, appended when not)
    std::unique_ptr<node>& slot(const std::string& name) {
        for (auto& m : members)
            if (m.first == name)
                return m.second;
        members.emplace_back(name, nullptr);
        return members.back().second;
    }
    uint64_t payload_bytes() const { return ext ? ext_bytes : data.size(); }
    const uint8_t* payload() const { return ext ? ext : data.data(); }
};

std::vector<std::string> split_path(const std::string& path) {
    std::vector<std::string> out;
    size_t i = 0;
    while (i <= path.size()) {
        const size_t j = path.find('/', i);
        const std::string part = path.substr(i, j == std::string::npos ? std::string::npos : j - i);
        if (!part.empty())
            out.push_back(part);
        if (j == std::string::npos)
            break;
        i = j + 1;
    }
    return out;
}

node* group_at(node& root, const std::vector<std::string>& parts, size_t count) {
    node* g = &root;
    for (size_t i = 0; i < count; ++i) {
        std::unique_ptr<node>& s = g->slot(parts[i]);
        if (!s)
            s = std::make_unique<node>();
        if (!s->is_group)
            throw std::invalid_argument("'" + parts[i] + "' is a dataset");
        g = s.get();
    }
    return g;
}

void remove_member(node& root, const std::string& path) {
    const auto parts = split_path(path);
    if (parts.empty())
        return;
    node* g = group_at(root, parts, parts.size() - 1);
    auto& v = g->members;
    v.erase(std::remove_if(v.begin(), v.end(), [&](const auto& m) { return m.first == parts.back(); }), v.end());
}

node& put_dataset(node& root, const std::string& path, const etype& t, std::vector<uint64_t> shape) {
    const auto parts = split_path(path);
    if (parts.empty())
        throw std::invalid_argument("empty dataset path");
    node* g = group_at(root, parts, parts.size() - 1);
    std::unique_ptr<node>& s = g->slot(parts.back());
    s = std::make_unique<node>();
    s->is_group = false;
    s->t = t;
    s->shape = std::move(shape);
    return *s;
}

void put_attribute(node& root, const std::string& path, const std::string& name, const etype& t, const void* v) {
    node* g = group_at(root, split_path(path), split_path(path).size());
    attribute a{name, t, std::vector<uint8_t>(static_cast<const uint8_t*>(v), static_cast<const uint8_t*>(v) + t.base)};
    for (auto& x : g->attrs)
        if (x.name == name) {
            x = std::move(a);
            return;
        }
    g->attrs.push_back(std::move(a));
}

// ------------------------------------------------------------------------------------------------
// writer: objects are laid out in the order they are made, each at an 8-byte boundary, so the file is
// written front to back; the superblock (which holds the end-of-file address) goes in last
// ------------------------------------------------------------------------------------------------

class image {
public:
    explicit image(const std::string& path) : path_(path) {
        f_ = std::fopen(path.c_str(), "wb");
        if (!f_)
            throw io_error("cannot create " + path + ": " + std::strerror(errno));
    }
    ~image() {
        if (f_)
            std::fclose(f_);
    }
    // appends `n` bytes (zero-padded to 8), returns their address
    uint64_t put(const void* p, uint64_t n) {
        const uint64_t a = end_;
        write(p, n);
        static const uint8_t z[8] = {};
        const uint64_t pad = (8 - n % 8) % 8;
        write(z, pad);
        return a;
    }
    uint64_t put(const bytes& b) { return put(b.b.data(), b.size()); }
    uint64_t end() const { return end_; }
    void patch(uint64_t addr, const bytes& b) {
        if (std::fseek(f_, (long)addr, SEEK_SET) != 0 || std::fwrite(b.b.data(), 1, b.size(), f_) != b.size())
            throw io_error("cannot write " + path_);
    }
    void close() {
        const int rc = std::fclose(f_);
        f_ = nullptr;
        if (rc != 0)
            throw io_error("cannot write " + path_);
    }

private:
    void write(const void* p, uint64_t n) {
        if (n && std::fwrite(p, 1, n, f_) != n)
            throw io_error("cannot write " + path_ + ": " + std::strerror(errno));
        end_ += n;
    }
    std::string path_;
    FILE* f_ = nullptr;
    uint64_t end_ = 0;
};

bytes message(uint16_t type, bytes data, uint8_t flags = 0) {
    data.pad8();
    bytes m;
    m.u16(type).u16((uint16_t)data.size()).u8(flags).zeros(3);
    return m.append(data);
}

bytes object_header(const std::vector<bytes>& msgs) {
    bytes body;
    for (const auto& m : msgs)
        body.append(m);
    bytes h;
    h.u8(1).u8(0).u16((uint16_t)msgs.size()).u32(1).u32((uint32_t)body.size()).zeros(4);
    return h.append(body);
}

bytes dataspace(const std::vector<uint64_t>& shape) {
    bytes s;
    s.u8(1).u8((uint8_t)shape.size()).u8(0).u8(0).zeros(4);
    for (uint64_t d : shape)
        s.u64(d);
    return s;
}

bytes attribute_message(const attribute& a) {
    const bytes dt = datatype_of(a.t);
    const bytes sp = dataspace({});
    bytes nm;
    nm.raw(a.name.data(), a.name.size()).u8(0);
    bytes d;
    d.u8(1).u8(0).u16((uint16_t)nm.size()).u16((uint16_t)dt.size()).u16((uint16_t)sp.size());
    bytes x = nm;
    d.append(x.pad8());
    x = dt;
    d.append(x.pad8());
    x = sp;
    d.append(x.pad8());
    d.raw(a.value.data(), a.value.size());
    return message(0x000C, d);
}

struct written {
    uint64_t header, tree = kUndef, heap = kUndef;
    bool group = false;
};

written write_dataset(image& img, const node& ds) {
    const uint64_t n = ds.payload_bytes();
    const uint64_t daddr = n ? img.put(ds.payload(), n) : kUndef;
    std::vector<bytes> msgs;
    msgs.push_back(message(0x0001, dataspace(ds.shape)));
    msgs.push_back(message(0x0003, datatype_of(ds.t), 1));  // constant
    bytes fill;
    fill.u8(2).u8(2).u8(2).u8(0);  // version 2, late allocation, never written, no value defined
    msgs.push_back(message(0x0005, fill));
    bytes layout;
    layout.u8(3).u8(1).u64(daddr).u64(n);  // version 3, contiguous
    msgs.push_back(message(0x0008, layout));
    return {img.put(object_header(msgs))};
}

written write_group(image& img, const node& g) {
    std::vector<std::pair<std::string, written>> child;
    for (const auto& m : g.members)  // children first, in insertion order
        child.emplace_back(m.first, m.second->is_group ? write_group(img, *m.second) : write_dataset(img, *m.second));
    std::vector<std::string> names;
    for (const auto& c : child)
        names.push_back(c.first);
    std::sort(names.begin(), names.end());  // symbol-table nodes keep their entries in name order
    auto info = [&](const std::string& nm) -> const written& {
        for (const auto& c : child)
            if (c.first == nm)
                return c.second;
        throw std::logic_error("member");
    };
    // local heap: "" at offset 0, then every name
    bytes seg;
    seg.zeros(8);
    std::vector<uint64_t> offs;
    for (const auto& nm : names) {
        offs.push_back(seg.size());
        seg.raw(nm.data(), nm.size()).u8(0).pad8();
    }
    const uint64_t seg_addr = img.put(seg);
    bytes heap;
    heap.raw("HEAP", 4).u8(0).zeros(3).u64(seg.size()).u64(kHeapFreeNull).u64(seg_addr);
    const uint64_t heap_addr = img.put(heap);
    // symbol-table nodes of at most 2K entries under one leaf B-tree node
    const size_t per = 2 * kLeafK;
    const size_t nchunks = names.empty() ? 1 : (names.size() + per - 1) / per;
    if (nchunks > 2 * kInternalK)
        throw std::invalid_argument("a group holds at most " + std::to_string(2 * kInternalK * per) + " members");
    std::vector<std::pair<uint64_t, uint64_t>> snods;
    for (size_t c = 0; c < nchunks; ++c) {
        const size_t lo = c * per, hi = std::min(names.size(), lo + per);
        bytes sn;
        sn.raw("SNOD", 4).u8(1).u8(0).u16((uint16_t)(hi - lo));
        for (size_t i = lo; i < hi; ++i) {
            const written& w = info(names[i]);
            sn.u64(offs[i]).u64(w.header);
            if (w.group)
                sn.u32(1).u32(0).u64(w.tree).u64(w.heap);
            else
                sn.u32(0).u32(0).zeros(16);
        }
        sn.zeros(8 + per * 40 - sn.size());
        snods.emplace_back(img.put(sn), hi > lo ? offs[hi - 1] : 0);
    }
    bytes tree;
    tree.raw("TREE", 4).u8(0).u8(0).u16((uint16_t)snods.size()).u64(kUndef).u64(kUndef).u64(0);
    for (const auto& s : snods)
        tree.u64(s.first).u64(s.second);
    tree.zeros(24 + (2 * kInternalK + 1) * 8 + 2 * kInternalK * 8 - tree.size());
    const uint64_t tree_addr = img.put(tree);
    std::vector<bytes> msgs;
    bytes stab;
    stab.u64(tree_addr).u64(heap_addr);
    msgs.push_back(message(0x0011, stab));
    for (const auto& a : g.attrs)
        msgs.push_back(attribute_message(a));
    written w{img.put(object_header(msgs)), tree_addr, heap_addr, true};
    return w;
}

// Writes the tree to `path` (through a temporary file renamed over it, so an appending writer never
// truncates the file it read from while the new one is incomplete).
void write_file(const std::string& path, const node& root) {
    const std::string tmp = path + ".dimgpu-tmp";
    try {
        image img(tmp);
        bytes zero;
        zero.zeros(96);
        img.put(zero);  // the superblock, written last
        const written r = write_group(img, root);
        bytes sb;
        sb.raw(kSignature, 8).u8(0).u8(0).u8(0).u8(0).u8(0).u8(8).u8(8).u8(0).u16(kLeafK).u16(kInternalK).u32(0);
        sb.u64(0).u64(kUndef).u64(img.end()).u64(kUndef);
        sb.u64(0).u64(r.header).u32(1).u32(0).u64(r.tree).u64(r.heap);
        img.patch(0, sb);
        img.close();
    } catch (...) {
        std::remove(tmp.c_str());
        throw;
    }
    if (std::rename(tmp.c_str(), path.c_str()) != 0) {
        std::remove(tmp.c_str());
        throw io_error("cannot replace " + path + ": " + std::strerror(errno));
    }
}

// ------------------------------------------------------------------------------------------------
// inflate (RFC 1950 zlib stream around RFC 1951 deflate blocks), for chunks with the deflate filter
// ------------------------------------------------------------------------------------------------

class inflater {
public:
    // `limit`: the most bytes the stream may produce (a chunk's size); a stream that would produce more is
    // not a chunk of this dataset
    inflater(const uint8_t* in, size_t n, std::vector<uint8_t>& out, size_t limit)
        : in_(in), n_(n), out_(out), limit_(limit), start_(out.size()) {}

    void run() {
        if (n_ < 2)
            throw format_error("deflate chunk: truncated zlib header");
        const uint8_t cmf = in_[0], flg = in_[1];
        if ((cmf & 0x0F) != 8 || ((cmf << 8) | flg) % 31 != 0 || (flg & 0x20))
            throw format_error("deflate chunk: not a zlib stream this reader supports");
        pos_ = 2;
        bool last = false;
        while (!last) {
            last = bits(1) != 0;
            const uint32_t type = bits(2);
            if (type == 0)
                stored();
            else if (type == 1)
                fixed();
            else if (type == 2)
                dynamic();
            else
                throw format_error("deflate chunk: invalid block type");
        }
        // the zlib trailer: Adler-32 (RFC 1950 section 8) of the bytes this stream produced, big-endian,
        // at the next byte boundary; a mismatch is a corrupt chunk, as libhdf5's deflate filter reports it
        buf_ = 0;
        cnt_ = 0;
        if (pos_ + 4 > n_)
            throw format_error("deflate chunk: truncated (no Adler-32 check value)");
        const uint32_t want = ((uint32_t)in_[pos_] << 24) | ((uint32_t)in_[pos_ + 1] << 16) |
                              ((uint32_t)in_[pos_ + 2] << 8) | (uint32_t)in_[pos_ + 3];
        if (adler32(out_.data() + start_, out_.size() - start_) != want)
            throw format_error("deflate chunk: Adler-32 check value does not match");
    }

private:
    // Adler-32 (RFC 1950): a = 1 + the sum of the bytes, b = the sum of the successive a, both mod 65521.
    // The sums are reduced every 5552 bytes, the most after which b still fits in 32 bits.
    static uint32_t adler32(const uint8_t* p, size_t n) {
        constexpr uint32_t kMod = 65521;
        uint32_t a = 1, b = 0;
        while (n) {
            const size_t k = n < 5552 ? n : 5552;
            for (size_t i = 0; i < k; ++i) {
                a += p[i];
                b += a;
            }
            a %= kMod;
            b %= kMod;
            p += k;
            n -= k;
        }
        return (b << 16) | a;
    }

    struct huffman {
        uint16_t count[16] = {};  // codes of each length
        uint16_t symbol[320] = {};  // symbols ordered by code
    };

    uint32_t bits(int need) {
        while (cnt_ < need) {
            if (pos_ >= n_)
                throw format_error("deflate chunk: truncated");
            buf_ |= (uint32_t)in_[pos_++] << cnt_;
            cnt_ += 8;
        }
        const uint32_t v = buf_ & ((1u << need) - 1u);
        buf_ >>= need;
        cnt_ -= need;
        return v;
    }

    // canonical code from code lengths (RFC 1951 3.2.2); incomplete codes are allowed, over-full ones not
    static void build(huffman& h, const uint8_t* len, int n) {
        std::memset(h.count, 0, sizeof(h.count));
        for (int s = 0; s < n; ++s)
            h.count[len[s]]++;
        h.count[0] = 0;
        int left = 1;
        for (int l = 1; l < 16; ++l) {
            left = 2 * left - h.count[l];
            if (left < 0)
                throw format_error("deflate chunk: over-subscribed code");
        }
        uint16_t off[16] = {};
        for (int l = 1; l < 15; ++l)
            off[l + 1] = off[l] + h.count[l];
        for (int s = 0; s < n; ++s)
            if (len[s])
                h.symbol[off[len[s]]++] = (uint16_t)s;
    }

    int decode(const huffman& h) {
        int code = 0, first = 0, index = 0;
        for (int l = 1; l < 16; ++l) {
            code |= (int)bits(1);
            const int c = h.count[l];
            if (code - first < c)
                return h.symbol[index + (code - first)];
            index += c;
            first = (first + c) << 1;
            code <<= 1;
        }
        throw format_error("deflate chunk: invalid code");
    }

    void stored() {
        buf_ = 0;
        cnt_ = 0;  // to the byte boundary
        if (pos_ + 4 > n_)
            throw format_error("deflate chunk: truncated stored block");
        const uint16_t len = rd16(in_ + pos_), nlen = rd16(in_ + pos_ + 2);
        pos_ += 4;
        if ((uint16_t)~nlen != len || pos_ + len > n_)
            throw format_error("deflate chunk: bad stored block");
        room(len);
        out_.insert(out_.end(), in_ + pos_, in_ + pos_ + len);
        pos_ += len;
    }

    void codes(const huffman& lit, const huffman& dist) {
        static const uint16_t lbase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                                           31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
        static const uint8_t lextra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2,
                                           2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
        static const uint16_t dbase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                           193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
        static const uint8_t dextra[30] = {0, 0, 0, 0, 1, 1, 2, 2,  3,  3,  4,  4,  5,  5,  6,
                                           6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
        for (;;) {
            int s = decode(lit);
            if (s < 256) {
                room(1);
                out_.push_back((uint8_t)s);
            } else if (s == 256) {
                return;
            } else {
                s -= 257;
                if (s >= 29)
                    throw format_error("deflate chunk: invalid length code");
                const uint32_t len = lbase[s] + bits(lextra[s]);
                const int d = decode(dist);
                if (d >= 30)
                    throw format_error("deflate chunk: invalid distance code");
                const uint32_t back = dbase[d] + bits(dextra[d]);
                if (back > out_.size())
                    throw format_error("deflate chunk: distance before the start");
                const size_t from = out_.size() - back;
                room(len);
                for (uint32_t k = 0; k < len; ++k)
                    out_.push_back(out_[from + k]);
            }
        }
    }

    void fixed() {
        uint8_t len[288 + 30];
        for (int s = 0; s < 144; ++s)
            len[s] = 8;
        for (int s = 144; s < 256; ++s)
            len[s] = 9;
        for (int s = 256; s < 280; ++s)
            len[s] = 7;
        for (int s = 280; s < 288; ++s)
            len[s] = 8;
        huffman lit, dist;
        build(lit, len, 288);
        for (int s = 0; s < 30; ++s)
            len[s] = 5;
        build(dist, len, 30);
        codes(lit, dist);
    }

    void dynamic() {
        static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
        const int nlen = (int)bits(5) + 257, ndist = (int)bits(5) + 1, ncode = (int)bits(4) + 4;
        if (nlen > 286 || ndist > 30)
            throw format_error("deflate chunk: bad code counts");
        uint8_t len[320] = {};
        for (int i = 0; i < ncode; ++i)
            len[order[i]] = (uint8_t)bits(3);
        huffman cl;
        build(cl, len, 19);
        int i = 0;
        uint8_t lens[320] = {};
        while (i < nlen + ndist) {
            const int s = decode(cl);
            if (s < 16) {
                lens[i++] = (uint8_t)s;
                continue;
            }
            uint8_t v = 0;
            int rep;
            if (s == 16) {
                if (i == 0)
                    throw format_error("deflate chunk: repeat with no length");
                v = lens[i - 1];
                rep = 3 + (int)bits(2);
            } else if (s == 17) {
                rep = 3 + (int)bits(3);
            } else {
                rep = 11 + (int)bits(7);
            }
            if (i + rep > nlen + ndist)
                throw format_error("deflate chunk: too many lengths");
            while (rep--)
                lens[i++] = v;
        }
        if (lens[256] == 0)
            throw format_error("deflate chunk: no end-of-block code");
        huffman lit, dist;
        build(lit, lens, nlen);
        build(dist, lens + nlen, ndist);
        codes(lit, dist);
    }

    void room(size_t more) const {
        if (out_.size() + more > limit_)
            throw format_error("deflate chunk: expands past the chunk's size");
    }

    const uint8_t* in_;
    size_t n_, pos_ = 0;
    uint32_t buf_ = 0;
    int cnt_ = 0;
    std::vector<uint8_t>& out_;
    size_t limit_;
    size_t start_;  // out_'s size before this stream
};

// ------------------------------------------------------------------------------------------------
// reader
// ------------------------------------------------------------------------------------------------

class mapped_file {
public:
    explicit mapped_file(const std::string& path) : path_(path) {
        const int fd = ::open(path.c_str(), O_RDONLY);
        if (fd < 0)
            throw io_error("cannot open " + path + ": " + std::strerror(errno));
        struct stat st {};
        if (::fstat(fd, &st) != 0) {
            ::close(fd);
            throw io_error("cannot stat " + path);
        }
        size_ = (uint64_t)st.st_size;
        if (size_) {
            void* p = ::mmap(nullptr, size_, PROT_READ, MAP_PRIVATE, fd, 0);
            if (p == MAP_FAILED) {
                ::close(fd);
                throw io_error("cannot map " + path);
            }
            data_ = static_cast<const uint8_t*>(p);
        }
        ::close(fd);
    }
    ~mapped_file() {
        if (data_)
            ::munmap(const_cast<uint8_t*>(data_), size_);
    }
    mapped_file(const mapped_file&) = delete;
    mapped_file& operator=(const mapped_file&) = delete;

    // the bytes [addr, addr + n), or a format error when they are not all in the file
    const uint8_t* at(uint64_t addr, uint64_t n) const {
        if (addr > size_ || n > size_ - addr)
            throw format_error(path_ + ": a structure points past the end of the file");
        return data_ + addr;
    }
    uint64_t size() const { return size_; }
    const std::string& path() const { return path_; }

private:
    std::string path_;
    const uint8_t* data_ = nullptr;
    uint64_t size_ = 0;
};

struct msg {
    uint16_t type;
    const uint8_t* data;
    uint16_t size;
};

// a * b, or a format error when the product of sizes read from the file does not fit in 64 bits
uint64_t checked_mul(uint64_t a, uint64_t b, const char* what) {
    uint64_t r = 0;
    if (__builtin_mul_overflow(a, b, &r))
        throw format_error(std::string(what) + ": size overflows 64 bits");
    return r;
}

// the host's physical memory in bytes: no dataset larger than it is read (a corrupt dataspace must not
// size an allocation the system cannot back)
uint64_t host_memory_bytes() {
    const long pages = sysconf(_SC_PHYS_PAGES), page = sysconf(_SC_PAGE_SIZE);
    return (pages > 0 && page > 0) ? (uint64_t)pages * (uint64_t)page : std::numeric_limits<uint64_t>::max();
}

struct dataset_info {
    etype t;
    std::vector<uint64_t> shape;
    const uint8_t* layout = nullptr;
    uint16_t layout_size = 0;
    std::vector<uint16_t> filters;
    uint64_t count() const {
        uint64_t n = 1;
        for (uint64_t d : shape)
            n = checked_mul(n, d, "dataspace");
        return n;
    }
    uint64_t bytes() const { return checked_mul(count(), t.element_bytes(), "dataset"); }
};

// datatype at p (inside a message of `n` bytes from `start`); returns the type and advances p
etype parse_type(const uint8_t* start, size_t n, size_t& p) {
    if (p + 8 > n)
        throw format_error("truncated datatype");
    const uint8_t cv = start[p];
    const int cls = cv & 0x0F, ver = cv >> 4;
    const uint32_t bits = start[p + 1] | (start[p + 2] << 8) | (start[p + 3] << 16);
    const uint32_t size = rd32(start + p + 4);
    size_t q = p + 8;
    etype t;
    if (cls == 0) {
        if (bits & 1)
            throw format_error("big-endian integers are not supported");
        t = {(bits & 0x08) ? kind::i : kind::u, size, 0};
        q += 4;
    } else if (cls == 1) {
        if (bits & 1)
            throw format_error("big-endian floats are not supported");
        t = {kind::f, size, 0};
        q += 12;
    } else if (cls == 10) {
        if (q + 4 > n)
            throw format_error("truncated array datatype");
        const int nd = start[q];
        q += 4;
        uint64_t inner = 1;
        for (int d = 0; d < nd; ++d) {
            if (q + 4 > n)
                throw format_error("truncated array datatype");
            inner = checked_mul(inner, rd32(start + q), "array datatype");
            q += 4;
        }
        if (inner == 0 || inner > 65536)
            throw format_error("array datatype of " + std::to_string(inner) + " elements is not supported");
        if (ver < 3)
            q += 4 * nd;  // permutation indices
        etype b = parse_type(start, n, q);
        if (b.inner)
            throw format_error("nested array datatypes are not supported");
        t = {b.k, b.base, (uint32_t)inner};
        p = q;
        return t;
    } else {
        throw format_error("datatype class " + std::to_string(cls) + " is not supported");
    }
    if ((t.k == kind::f && t.base != 4 && t.base != 8) || (t.k != kind::f && t.base != 1 && t.base != 2 &&
                                                            t.base != 4 && t.base != 8))
        throw format_error("element size " + std::to_string(t.base) + " is not supported");
    p = q;
    return t;
}

std::vector<uint64_t> parse_space(const uint8_t* d, size_t n) {
    if (n < 4)
        throw format_error("truncated dataspace");
    const int ver = d[0], rank = d[1];
    size_t q;
    if (ver == 1) {
        q = 8;
    } else if (ver == 2) {
        if (d[3] == 2)
            return {};  // null dataspace
        q = 4;
    } else {
        throw format_error("dataspace version " + std::to_string(ver));
    }
    if (q + 8 * (size_t)rank > n)
        throw format_error("truncated dataspace");
    std::vector<uint64_t> s(rank);
    for (int i = 0; i < rank; ++i)
        s[i] = rd64(d + q + 8 * i);
    return s;
}

class reader {
public:
    explicit reader(const std::string& path) : f_(path) {
        const uint8_t* b = f_.at(0, 24);
        if (std::memcmp(b, kSignature, 8) != 0)
            throw format_error(path + " is not an HDF5 file");
        const int ver = b[8];
        if (ver != 0 && ver != 1)
            throw format_error("superblock version " + std::to_string(ver) +
                               " (files written with libver 'latest') is not supported");
        if (b[13] != 8 || b[14] != 8)
            throw format_error("only 8-byte offsets and lengths are supported");
        const uint64_t p = 24 + (ver == 1 ? 4 : 0);
        base_ = rd64(f_.at(p, 8));
        root_ = rd64(f_.at(p + 32 + 8, 8)) + base_;
    }

    uint64_t resolve(const std::string& path) const {
        uint64_t a = root_;
        for (const auto& part : split_path(path)) {
            bool found = false;
            for (const auto& m : members(a))
                if (m.first == part) {
                    a = m.second;
                    found = true;
                    break;
                }
            if (!found)
                throw std::invalid_argument("'" + part + "' not found in " + f_.path());
        }
        return a;
    }

    bool contains(const std::string& path) const {
        try {
            resolve(path);
            return true;
        } catch (const std::invalid_argument&) {
            return false;
        }
    }

    // messages of the version-1 object header at addr, continuation blocks included
    std::vector<msg> messages(uint64_t addr) const {
        const uint8_t* h = f_.at(addr, 16);
        if (std::memcmp(h, "OHDR", 4) == 0)
            throw format_error("version-2 object headers are not supported");
        if (h[0] != 1)
            throw format_error("object header version " + std::to_string(h[0]));
        const uint16_t n = rd16(h + 2);
        std::vector<std::pair<uint64_t, uint64_t>> blocks{{addr + 16, rd32(h + 8)}};
        std::vector<msg> out;
        for (size_t bi = 0; bi < blocks.size() && out.size() < n; ++bi) {
            uint64_t p = blocks[bi].first;
            const uint64_t end = p + blocks[bi].second;
            f_.at(blocks[bi].first, blocks[bi].second);
            while (p + 8 <= end && out.size() < n) {
                const uint8_t* m = f_.at(p, 8);
                const uint16_t type = rd16(m), size = rd16(m + 2);
                const uint8_t* data = f_.at(p + 8, size);
                if (type == 0x0010) {
                    if (size < 16)
                        throw format_error("truncated continuation message");
                    if (blocks.size() > 4096)
                        throw format_error("too many object header continuation blocks");
                    blocks.emplace_back(rd64(data) + base_, rd64(data + 8));
                }
                out.push_back({type, data, size});
                p += 8 + size;
            }
        }
        return out;
    }

    bool is_group(uint64_t addr) const {
        for (const auto& m : messages(addr))
            if (m.type == 0x0011)
                return true;
        return false;
    }

    // (name, object header address) of a symbol-table group's members, in name order
    std::vector<std::pair<std::string, uint64_t>> members(uint64_t addr) const {
        const msg* stab = nullptr;
        const auto ms = messages(addr);
        for (const auto& m : ms)
            if (m.type == 0x0011)
                stab = &m;
        if (!stab || stab->size < 16)
            throw format_error("not a group (no symbol table message; link-message groups are not supported)");
        const uint64_t tree = rd64(stab->data), heap = rd64(stab->data + 8) + base_;
        const uint8_t* hp = f_.at(heap, 32);
        if (std::memcmp(hp, "HEAP", 4) != 0)
            throw format_error("bad local heap");
        const uint64_t seg = rd64(hp + 24) + base_, seg_size = rd64(hp + 8);
        std::vector<std::pair<std::string, uint64_t>> out;
        walk_group(tree, seg, seg_size, out, 0);
        std::sort(out.begin(), out.end());
        return out;
    }

    std::vector<attribute> attributes(uint64_t addr) const {
        std::vector<attribute> out;
        for (const auto& m : messages(addr)) {
            if (m.type != 0x000C)
                continue;
            const uint8_t* d = m.data;
            if (m.size < 8)
                throw format_error("truncated attribute message");
            const int ver = d[0];
            const uint16_t nsz = rd16(d + 2), tsz = rd16(d + 4), ssz = rd16(d + 6);
            size_t p = 8 + (ver == 3 ? 1 : 0);
            auto rnd = [&](size_t x) { return ver == 1 ? (x + 7) / 8 * 8 : x; };
            if (p + nsz > m.size)
                throw format_error("truncated attribute name");
            std::string name(reinterpret_cast<const char*>(d + p), strnlen(reinterpret_cast<const char*>(d + p), nsz));
            p += rnd(nsz);
            size_t tp = p;
            const etype t = parse_type(d, m.size, tp);
            p += rnd(tsz);
            if (p + ssz > m.size)
                throw format_error("truncated attribute dataspace");
            const auto shape = parse_space(d + p, ssz);
            p += rnd(ssz);
            uint64_t cnt = 1;
            for (uint64_t s : shape)
                cnt = checked_mul(cnt, s, "attribute dataspace");
            const uint64_t nb = checked_mul(cnt, t.element_bytes(), "attribute");
            if (nb > m.size || p + nb > m.size)
                throw format_error("truncated attribute value");
            out.push_back({name, t, std::vector<uint8_t>(d + p, d + p + nb), t.inner ? 0 : cnt});
        }
        return out;
    }

    dataset_info info(uint64_t addr) const {
        dataset_info di;
        bool have_t = false, have_s = false;
        for (const auto& m : messages(addr)) {
            if (m.type == 0x0001) {
                di.shape = parse_space(m.data, m.size);
                have_s = true;
            } else if (m.type == 0x0003) {
                size_t p = 0;
                di.t = parse_type(m.data, m.size, p);
                have_t = true;
            } else if (m.type == 0x0008) {
                di.layout = m.data;
                di.layout_size = m.size;
            } else if (m.type == 0x000B) {
                di.filters = parse_filters(m.data, m.size);
            }
        }
        if (!have_t || !have_s || !di.layout)
            throw format_error("not a dataset");
        if (di.layout_size < 2 || di.layout[0] != 3)
            throw format_error("layout message version " + std::to_string(di.layout_size ? di.layout[0] : 0));
        return di;
    }

    // element count of a dataset's first dimension (1 for a scalar)
    uint64_t length(uint64_t addr) const {
        const dataset_info di = info(addr);
        check_extent(di);
        return di.shape.empty() ? 1 : di.shape[0];
    }

    // The dataset's bytes, checked against what the file can hold before anything is allocated: no more
    // than the host's memory, and a contiguous dataset's stored size at least its dataspace's.
    uint64_t check_extent(const dataset_info& di) const {
        const uint64_t nbytes = di.bytes();
        if (nbytes > host_memory_bytes())
            throw format_error("dataset of " + std::to_string(nbytes) + " bytes exceeds the host's memory");
        if (di.layout[1] == 1) {
            if (di.layout_size < 18)
                throw format_error("truncated layout message");
            if (rd64(di.layout + 2) != kUndef && rd64(di.layout + 10) < nbytes)
                throw format_error("contiguous dataset stores fewer bytes than its dataspace holds");
        }
        return nbytes;
    }

    // all the bytes of a dataset (zeros where nothing was written)
    std::vector<uint8_t> read(uint64_t addr, dataset_info* out_info = nullptr) const {
        dataset_info di = info(addr);
        const uint64_t nbytes = check_extent(di);
        std::vector<uint8_t> raw;
        const uint8_t* L = di.layout;
        const int cls = L[1];
        if (cls == 0) {  // compact
            if (di.layout_size < 4)
                throw format_error("truncated layout message");
            const uint16_t sz = rd16(L + 2);
            if (4u + sz > di.layout_size)
                throw format_error("truncated compact dataset");
            raw.assign(L + 4, L + 4 + sz);
        } else if (cls == 1) {  // contiguous
            if (di.layout_size < 18)
                throw format_error("truncated layout message");
            const uint64_t a = rd64(L + 2), sz = rd64(L + 10);
            if (a != kUndef) {
                const uint64_t take = std::min(sz, nbytes);
                const uint8_t* p = f_.at(a + base_, take);
                raw.assign(p, p + take);
            }
        } else if (cls == 2) {
            raw = read_chunked(di, nbytes);
        } else {
            throw format_error("layout class " + std::to_string(cls));
        }
        raw.resize(nbytes, 0);
        if (out_info)
            *out_info = std::move(di);
        return raw;
    }

private:
    void walk_group(uint64_t node, uint64_t seg, uint64_t seg_size, std::vector<std::pair<std::string, uint64_t>>& out,
                    int depth) const {
        if (depth > 64)
            throw format_error("group B-tree too deep");
        const uint8_t* t = f_.at(node + base_, 24);
        if (std::memcmp(t, "TREE", 4) != 0)
            throw format_error("bad group B-tree node");
        const int level = t[5];
        const uint16_t used = rd16(t + 6);
        for (uint16_t i = 0; i < used; ++i) {
            const uint64_t child = rd64(f_.at(node + base_ + 24 + 8 + 16 * (uint64_t)i, 8));
            if (level > 0) {
                walk_group(child, seg, seg_size, out, depth + 1);
                continue;
            }
            const uint8_t* sn = f_.at(child + base_, 8);
            if (std::memcmp(sn, "SNOD", 4) != 0)
                throw format_error("bad symbol table node");
            const uint16_t ne = rd16(sn + 6);
            for (uint16_t e = 0; e < ne; ++e) {
                const uint8_t* q = f_.at(child + base_ + 8 + 40 * (uint64_t)e, 40);
                const uint64_t name_off = rd64(q), oh = rd64(q + 8);
                if (name_off >= seg_size)
                    throw format_error("symbol name outside the local heap");
                const char* s = reinterpret_cast<const char*>(f_.at(seg + name_off, seg_size - name_off));
                out.emplace_back(std::string(s, strnlen(s, seg_size - name_off)), oh + base_);
            }
        }
    }

    static std::vector<uint16_t> parse_filters(const uint8_t* d, size_t n) {
        if (n < 2)
            throw format_error("truncated filter pipeline");
        const int ver = d[0], nf = d[1];
        size_t p = ver == 1 ? 8 : 2;
        std::vector<uint16_t> out;
        for (int i = 0; i < nf; ++i) {
            if (p + 2 > n)
                throw format_error("truncated filter pipeline");
            const uint16_t id = rd16(d + p);
            uint16_t nval;
            if (ver == 1 || id >= 256) {
                if (p + 8 > n)
                    throw format_error("truncated filter pipeline");
                const uint16_t nlen = rd16(d + p + 2);
                nval = rd16(d + p + 6);
                p += 8 + (ver == 1 ? (nlen + 7) / 8 * 8 : nlen);
            } else {
                if (p + 6 > n)
                    throw format_error("truncated filter pipeline");
                nval = rd16(d + p + 4);
                p += 6;
            }
            p += 4 * (size_t)nval + ((ver == 1 && nval % 2) ? 4 : 0);
            out.push_back(id);
        }
        return out;
    }

    std::vector<uint8_t> read_chunked(const dataset_info& di, uint64_t nbytes) const {
        const uint8_t* L = di.layout;
        if (di.layout_size < 11)
            throw format_error("truncated layout message");
        const int nd = L[2];
        const uint64_t tree = rd64(L + 3);
        if (nd != 2 || di.layout_size < 11 + 4 * (size_t)nd)
            throw format_error("only 1-D chunked datasets are supported");
        const uint64_t chunk_elems = rd32(L + 11), esz = di.t.element_bytes();
        if (chunk_elems == 0)
            throw format_error("chunk of no elements");
        bool deflate = false;
        for (uint16_t f : di.filters) {
            if (f != 1)
                throw format_error("filter " + std::to_string(f) + " is not supported (deflate only)");
            deflate = true;
        }
        std::vector<uint8_t> out(nbytes, 0);
        if (tree != kUndef)
            walk_chunks(tree, nd, chunk_elems, esz, di.count(), deflate, out, 0);
        return out;
    }

    void walk_chunks(uint64_t node, int nd, uint64_t chunk_elems, uint64_t esz, uint64_t count, bool deflate,
                     std::vector<uint8_t>& out, int depth) const {
        if (depth > 64)
            throw format_error("chunk B-tree too deep");
        const uint8_t* t = f_.at(node + base_, 24);
        if (std::memcmp(t, "TREE", 4) != 0 || t[4] != 1)
            throw format_error("bad chunk B-tree node");
        const int level = t[5];
        const uint16_t used = rd16(t + 6);
        const uint64_t ksz = 8 + 8 * (uint64_t)nd;
        uint64_t p = node + base_ + 24;
        for (uint16_t i = 0; i < used; ++i, p += ksz + 8) {
            const uint8_t* k = f_.at(p, ksz + 8);
            const uint32_t csize = rd32(k), fmask = rd32(k + 4);
            const uint64_t off0 = rd64(k + 8), child = rd64(k + ksz);
            if (level > 0) {
                walk_chunks(child, nd, chunk_elems, esz, count, deflate, out, depth + 1);
                continue;
            }
            if (off0 >= count)
                continue;
            const uint8_t* raw = f_.at(child + base_, csize);
            const uint64_t n = std::min(chunk_elems, count - off0) * esz;
            if (deflate && !(fmask & 1)) {
                // room for the bytes this chunk contributes (the layout's chunk size is only the limit the
                // stream may not pass: a corrupt one must not size an allocation)
                std::vector<uint8_t> plain;
                plain.reserve(n);
                inflater(raw, csize, plain, chunk_elems * esz).run();
                if (plain.size() < n)
                    throw format_error("deflate chunk shorter than its elements");
                std::memcpy(out.data() + off0 * esz, plain.data(), n);
            } else {
                if (csize < n)
                    throw format_error("chunk shorter than its elements");
                std::memcpy(out.data() + off0 * esz, raw, n);
            }
        }
    }

    mapped_file f_;
    uint64_t base_ = 0, root_ = 0;
};

// Reads the whole file into a tree (for a writer that appends to it).
void load_tree(const reader& r, uint64_t addr, node& g) {
    g.attrs = r.attributes(addr);
    for (const auto& a : g.attrs)
        if (a.count != 1)
            throw format_error("attribute " + a.name + " is not a scalar; the writer keeps scalar attributes only");
    for (const auto& m : r.members(addr)) {
        auto n = std::make_unique<node>();
        if (r.is_group(m.second)) {
            load_tree(r, m.second, *n);
        } else {
            dataset_info di;
            n->is_group = false;
            n->data = r.read(m.second, &di);
            n->t = di.t;
            n->shape = di.shape;
        }
        g.members.emplace_back(m.first, std::move(n));
    }
}

node open_tree(const std::string& path, bool append) {
    node root;
    if (append) {
        uint8_t sig[8] = {};
        FILE* f = std::fopen(path.c_str(), "rb");
        const bool h5 = f && std::fread(sig, 1, 8, f) == 8 && std::memcmp(sig, kSignature, 8) == 0;
        if (f)
            std::fclose(f);
        if (h5) {
            reader r(path);
            load_tree(r, r.resolve("/"), root);
        }
    }
    return root;
}

// Elements of a dataset converted to T (as numpy's astype would; integers out of T's range are an error).
template <typename T>
std::vector<T> read_as(const reader& r, const std::string& path, uint64_t expect = kUndef) {
    const uint64_t addr = r.resolve(path);
    {  // the element count is checked before the dataset's bytes are read
        const dataset_info d0 = r.info(addr);
        const uint64_t n0 = checked_mul(d0.count(), d0.t.inner ? d0.t.inner : 1, "dataset");
        if (expect != kUndef && n0 != expect)
            throw format_error(path + ": " + std::to_string(n0) + " elements, expected " + std::to_string(expect));
    }
    dataset_info di;
    const std::vector<uint8_t> raw = r.read(addr, &di);
    const uint64_t n = di.count() * (di.t.inner ? di.t.inner : 1);
    std::vector<T> out(n);
    const uint8_t* p = raw.data();
    for (uint64_t i = 0; i < n; ++i, p += di.t.base) {
        double f = 0;
        uint64_t u = 0;
        int64_t s = 0;
        switch (di.t.base) {
        case 1: u = p[0]; s = (int8_t)p[0]; break;
        case 2: u = rd16(p); s = (int16_t)rd16(p); break;
        case 4: u = rd32(p); s = (int32_t)rd32(p); break;
        default: u = rd64(p); s = (int64_t)u; break;
        }
        if (di.t.k == kind::f) {
            if (di.t.base == 4) {
                float x;
                std::memcpy(&x, p, 4);
                f = x;
            } else {
                std::memcpy(&f, p, 8);
            }
        }
        if constexpr (std::is_floating_point_v<T>) {
            out[i] = di.t.k == kind::f ? (T)f : di.t.k == kind::i ? (T)s : (T)u;
        } else {
            if (di.t.k == kind::f)
                throw format_error(path + ": floating-point data where integers are expected");
            if ((di.t.k == kind::i && (s < 0 || (uint64_t)s > (uint64_t)std::numeric_limits<T>::max())) ||
                (di.t.k == kind::u && u > (uint64_t)std::numeric_limits<T>::max()))
                throw format_error(path + ": an index does not fit in 32 bits");
            out[i] = (T)(di.t.k == kind::i ? (uint64_t)s : u);
        }
    }
    return out;
}

uint32_t u32_attribute(const reader& r, const std::string& group, const std::string& name) {
    for (const auto& a : r.attributes(r.resolve(group)))
        if (a.name == name) {
            if (a.count != 1)
                throw format_error("attribute " + name + " is not a scalar");
            if (a.t.k == kind::f)
                throw format_error("attribute " + name + " is not an integer");
            uint64_t v = 0;
            for (uint32_t b = 0; b < a.t.base && b < 8; ++b)
                v |= (uint64_t)a.value[b] << (8 * b);
            if (a.t.k == kind::i && a.t.base < 8 && (v >> (8 * a.t.base - 1)) & 1)
                throw format_error("attribute " + name + " is negative");
            if (v > 0xFFFFFFFFull)
                throw format_error("attribute " + name + " does not fit in 32 bits");
            return (uint32_t)v;
        }
    throw format_error("group " + group + " has no attribute " + name);
}

// Runs f, turning exceptions into the library's status codes and message.
template <typename F>
int guarded(const char* what, F&& f) {
    try {
        return f();
    } catch (const std::invalid_argument& e) {
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "%s: %s", what, e.what());
    } catch (const format_error& e) {
        return fail(DIMGPU_ERR_IO, "%s: %s", what, e.what());
    } catch (const io_error& e) {
        return fail(DIMGPU_ERR_IO, "%s: %s", what, e.what());
    } catch (const std::bad_alloc&) {
        return fail(DIMGPU_ERR_OUT_OF_MEMORY, "%s: out of host memory", what);
    } catch (const std::exception& e) {
        return fail(DIMGPU_ERR_IO, "%s: %s", what, e.what());
    }
}

bool bad_str(const char* s) { return !s || !*s; }

}  // namespace
}  // namespace h5
}  // namespace dimgpu

using namespace dimgpu;
using namespace dimgpu::h5;

extern "C" {

int dimgpu_h5_csr_dimensions(const char* path, const char* group, uint32_t* rows, uint32_t* cols, uint64_t* nnz) {
    if (bad_str(path) || bad_str(group) || !rows || !cols || !nnz)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    return guarded("read_matlab_compatible", [&] {
        reader r(path);
        const std::string g(group);
        const uint64_t jc = r.length(r.resolve(g + "/jc")), data = r.length(r.resolve(g + "/data"));
        if (jc == 0 || jc - 1 > 0xFFFFFFFFull)
            throw format_error("jc must hold rows + 1 offsets");
        *rows = (uint32_t)(jc - 1);
        *cols = u32_attribute(r, g, "MATLAB_sparse");
        *nnz = data;
        return DIMGPU_OK;
    });
}

int dimgpu_h5_read_matlab_compatible(const char* path, const char* group, uint32_t* row_ptr, uint32_t* col_indices,
                                     double* values) {
    if (bad_str(path) || bad_str(group) || !row_ptr)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    return guarded("read_matlab_compatible", [&] {
        reader r(path);
        const std::string g(group);
        const auto jc = read_as<uint32_t>(r, g + "/jc");
        const uint64_t nnz = r.length(r.resolve(g + "/data"));
        const auto ir = read_as<uint32_t>(r, g + "/ir", nnz);
        const auto data = read_as<double>(r, g + "/data", nnz);
        if (jc.empty() || jc.front() != 0 || jc.back() != nnz)
            throw format_error("jc does not run from 0 to the number of elements");
        if (nnz && (!col_indices || !values))
            throw std::invalid_argument("NULL col_indices or values for a matrix with elements");
        std::memcpy(row_ptr, jc.data(), jc.size() * sizeof(uint32_t));
        if (nnz) {
            std::memcpy(col_indices, ir.data(), nnz * sizeof(uint32_t));
            std::memcpy(values, data.data(), nnz * sizeof(double));
        }
        return DIMGPU_OK;
    });
}

int dimgpu_h5_write_matlab_compatible(const char* path, const char* group, uint32_t rows, uint32_t cols, uint64_t nnz,
                                      const uint32_t* row_ptr, const uint32_t* col_indices, const double* values,
                                      int append) {
    if (bad_str(path) || bad_str(group) || !row_ptr || (nnz && (!col_indices || !values)))
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    return guarded("write_matlab_compatible", [&] {
        node root = open_tree(path, append != 0);
        const std::string g(group);
        remove_member(root, g);
        node& d = put_dataset(root, g + "/data", kF64, {nnz});
        d.ext = reinterpret_cast<const uint8_t*>(values);
        d.ext_bytes = nnz * 8;
        node& ir = put_dataset(root, g + "/ir", kU32, {nnz});
        ir.ext = reinterpret_cast<const uint8_t*>(col_indices);
        ir.ext_bytes = nnz * 4;
        node& jc = put_dataset(root, g + "/jc", kU32, {(uint64_t)rows + 1});
        jc.ext = reinterpret_cast<const uint8_t*>(row_ptr);
        jc.ext_bytes = ((uint64_t)rows + 1) * 4;
        put_attribute(root, g, "MATLAB_sparse", kU32, &cols);
        write_file(path, root);
        return DIMGPU_OK;
    });
}

int dimgpu_h5_store_csr5(const char* path, const char* group, const dimgpu_csr5* m, int append) {
    if (bad_str(path) || bad_str(group) || !m)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    dimgpu_csr5_info info{};
    DG_CHECK(dimgpu_csr5_get_info(m, &info));
    if (info.layout != DIMGPU_LAYOUT_REFERENCE || info.sigma != 16 || info.omega != 4 || info.desc_word_bytes != 4)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT,
                    "store_csr5 writes the reference's CSR5 (sigma 16, omega 4, reference layout); this matrix has "
                    "sigma %u, omega %u",
                    info.sigma, info.omega);
    return guarded("store_csr5", [&] {
        const uint64_t T = info.tile_count;
        std::vector<uint32_t> tile_ptr(T + 1), desc(T * 4), tdo_ptr(T + 1), tdo(info.tile_desc_offset_len),
            col(info.nnz), row_ptr((uint64_t)info.rows + 1);
        std::vector<double> vals(info.nnz);
        const int rc = dimgpu_csr5_export(m, tile_ptr.data(), desc.data(), tdo_ptr.data(), tdo.data(), vals.data(),
                                          col.data(), row_ptr.data());
        if (rc != DIMGPU_OK)
            return rc;
        node root = open_tree(path, append != 0);
        const std::string g(group);
        remove_member(root, g);
        put_attribute(root, g, "column_count", kU32, &info.cols);
        auto put = [&](const char* name, const etype& t, uint64_t n, const void* p, uint64_t bytes_) {
            node& d = put_dataset(root, g + "/" + name, t, {n});
            d.data.assign(static_cast<const uint8_t*>(p), static_cast<const uint8_t*>(p) + bytes_);
        };
        put("vals", kF64, info.nnz, vals.data(), info.nnz * 8);
        put("col_idx", kU32, info.nnz, col.data(), info.nnz * 4);
        put("row_ptr", kU32, row_ptr.size(), row_ptr.data(), row_ptr.size() * 4);
        put("tile_ptr", kU32, tile_ptr.size(), tile_ptr.data(), tile_ptr.size() * 4);
        put("tile_desc", etype{kind::u, 4, 4}, T, desc.data(), desc.size() * 4);
        put("tile_desc_offset_ptr", kU32, tdo_ptr.size(), tdo_ptr.data(), tdo_ptr.size() * 4);
        put("tile_desc_offset", kU32, tdo.size(), tdo.data(), tdo.size() * 4);
        write_file(path, root);
        return DIMGPU_OK;
    });
}

int dimgpu_h5_load_csr5(const char* path, const char* group, const dimgpu_csr5_options* opt, void* stream,
                        dimgpu_csr5** out) {
    if (bad_str(path) || bad_str(group) || !out)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = nullptr;
    uint32_t rows = 0, cols = 0;
    std::vector<uint32_t> row_ptr, col;
    std::vector<double> vals;
    const int rc = guarded("load_csr5", [&] {
        reader r(path);
        const std::string g(group);
        cols = u32_attribute(r, g, "column_count");
        row_ptr = read_as<uint32_t>(r, g + "/row_ptr");
        vals = read_as<double>(r, g + "/vals");
        col = read_as<uint32_t>(r, g + "/col_idx", vals.size());
        const auto tile_ptr = read_as<uint32_t>(r, g + "/tile_ptr");
        const uint64_t nnz = vals.size(), T = r.length(r.resolve(g + "/tile_desc"));
        constexpr uint64_t kSigmaRef = 16, kOmegaRef = 4, kTile = kSigmaRef * kOmegaRef;
        if (row_ptr.empty() || row_ptr.size() - 1 > 0xFFFFFFFFull)
            throw format_error("row_ptr must hold rows + 1 offsets");
        rows = (uint32_t)(row_ptr.size() - 1);
        if (T != nnz / kTile || tile_ptr.size() != T + 1)
            throw format_error(std::to_string(T) + " stored tiles for " + std::to_string(nnz) +
                               " elements: not a sigma 16 x omega 4 CSR5 group");
        if (row_ptr.front() != 0 || row_ptr.back() != nnz)
            throw format_error("row_ptr does not run from 0 to the number of elements");
        // csr5::transpose (csr5.h:463-493) stored every full tile that holds more than one row with
        // element c*sigma + r at r*omega + c; put those back into CSR order
        std::vector<double> tv(kTile);
        std::vector<uint32_t> tc(kTile);
        for (uint64_t t = 0; t < T; ++t) {
            if ((tile_ptr[t] & 0x7FFFFFFFu) == (tile_ptr[t + 1] & 0x7FFFFFFFu))
                continue;
            double* v = vals.data() + t * kTile;
            uint32_t* c = col.data() + t * kTile;
            for (uint64_t rr = 0; rr < kSigmaRef; ++rr)
                for (uint64_t cc = 0; cc < kOmegaRef; ++cc) {
                    tv[cc * kSigmaRef + rr] = v[rr * kOmegaRef + cc];
                    tc[cc * kSigmaRef + rr] = c[rr * kOmegaRef + cc];
                }
            std::copy(tv.begin(), tv.end(), v);
            std::copy(tc.begin(), tc.end(), c);
        }
        return DIMGPU_OK;
    });
    if (rc != DIMGPU_OK)
        return rc;
    return dimgpu_csr5_from_csr(rows, cols, vals.size(), row_ptr.data(), col.empty() ? nullptr : col.data(),
                                vals.empty() ? nullptr : vals.data(), DIMGPU_MEM_HOST, opt, stream, out);
}

int dimgpu_h5_vector_length(const char* path, const char* dataset, uint64_t* n) {
    if (bad_str(path) || bad_str(dataset) || !n)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    return guarded("read_vector", [&] {
        reader r(path);
        const dataset_info di = r.info(r.resolve(dataset));
        r.check_extent(di);
        *n = checked_mul(di.count(), di.t.inner ? di.t.inner : 1, "dataset");
        return DIMGPU_OK;
    });
}

int dimgpu_h5_read_vector(const char* path, const char* dataset, double* y) {
    if (bad_str(path) || bad_str(dataset))
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    return guarded("read_vector", [&] {
        reader r(path);
        const auto v = read_as<double>(r, dataset);
        if (!v.empty() && !y)
            throw std::invalid_argument("NULL y");
        std::memcpy(y, v.data(), v.size() * sizeof(double));
        return DIMGPU_OK;
    });
}

int dimgpu_h5_write_vector(const char* path, const char* dataset, uint64_t n, const double* y, int overwrite) {
    if (bad_str(path) || bad_str(dataset) || (n && !y))
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    return guarded("write_vector", [&] {
        node root = open_tree(path, true);
        const auto parts = split_path(dataset);
        if (parts.empty())
            throw std::invalid_argument("empty dataset path");
        node* g = group_at(root, parts, parts.size() - 1);
        if (g->member(parts.back()) && !overwrite)
            throw std::invalid_argument(std::string("outfile already contains ") + dataset +
                                        "; pass overwrite to replace it");
        node& d = put_dataset(root, dataset, kF64, {n});
        d.ext = reinterpret_cast<const uint8_t*>(y);
        d.ext_bytes = n * 8;
        write_file(path, root);
        return DIMGPU_OK;
    });
}

}  // extern "C"
