// teufel_hdf5_read.hpp -- a minimal reader for the HDF5 files TEUFEL's
// MeshedScreen reads (src/mesh.cpp:31-218), written from the HDF5 file-format
// specification, for builds without the HDF5 library.
//
// Supported: superblock version 0 (8-byte offsets and lengths); the root group
// as a symbol table (version-1 B-tree of group nodes, symbol-table nodes, local
// heap); version-1 object headers with continuation blocks; dataspace messages
// versions 1 and 2; fixed-point (4 or 8 byte) and IEEE floating-point (4 or 8
// byte) little-endian datatypes; contiguous and compact data layouts (layout
// message version 3); attribute messages versions 1 to 3 with scalar or
// one-element data.  Anything else (chunked or filtered data, big-endian
// types, newer superblocks) is rejected with an exception naming it.
#pragma once

#include <cstdint>
#include <cstring>
#include <fstream>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

namespace teufel_gb300 {
namespace h5 {

struct Error : std::runtime_error {
    explicit Error(const std::string& m) : std::runtime_error("HDF5 reader: " + m) {}
};

// A scalar type as stored: class 0 = fixed point, 1 = floating point.
struct Type {
    int cls = -1;
    int size = 0;
    bool is_signed = true;
};

struct Attribute {
    Type type;
    std::vector<uint8_t> data;
};

struct Dataset {
    std::vector<uint64_t> dims;
    Type type;
    uint64_t addr = 0;   // contiguous: file address of the data
    uint64_t size = 0;   // bytes
    std::vector<uint8_t> compact;
    bool is_compact = false;
    std::map<std::string, Attribute> attrs;
    uint64_t count() const {
        uint64_t n = 1;
        for (uint64_t d : dims) n *= d;
        return n;
    }
};

class File {
public:
    explicit File(const std::string& path) {
        std::ifstream f(path, std::ios::binary);
        if (!f) throw Error("cannot open " + path);
        buf_.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
        static const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
        if (buf_.size() < 96 || std::memcmp(buf_.data(), sig, 8) != 0)
            throw Error(path + " is not an HDF5 file");
        if (buf_[8] != 0) throw Error("superblock version " + std::to_string(buf_[8]));
        if (buf_[13] != 8 || buf_[14] != 8) throw Error("offsets or lengths not 8 bytes");
        // root group symbol table entry after the fixed part and four addresses
        const uint64_t root = 24 + 32;
        const uint64_t root_header = u64(root + 8);
        read_group(root_header);
    }

    bool exists(const std::string& name) const { return links_.count(name) != 0; }

    Dataset dataset(const std::string& name) const {
        auto it = links_.find(name);
        if (it == links_.end()) throw Error("no object " + name);
        return read_dataset(it->second);
    }

    // The dataset's elements as doubles (any supported numeric type).
    std::vector<double> read_double(const Dataset& d) const {
        std::vector<double> out((size_t)d.count());
        const uint8_t* p = raw(d, out.size());
        for (size_t i = 0; i < out.size(); i++) out[i] = value(d.type, p + i * d.type.size);
        return out;
    }

    std::vector<int64_t> read_int(const Dataset& d) const {
        std::vector<int64_t> out((size_t)d.count());
        const uint8_t* p = raw(d, out.size());
        for (size_t i = 0; i < out.size(); i++) out[i] = ivalue(d.type, p + i * d.type.size);
        return out;
    }

    static double attr_double(const Dataset& d, const std::string& name) {
        const Attribute& a = attr(d, name);
        return value(a.type, a.data.data());
    }
    static int64_t attr_int(const Dataset& d, const std::string& name) {
        const Attribute& a = attr(d, name);
        return ivalue(a.type, a.data.data());
    }

private:
    std::vector<uint8_t> buf_;
    std::map<std::string, uint64_t> links_;  // name -> object header address

    void need(uint64_t off, uint64_t n) const {
        if (off > buf_.size() || n > buf_.size() - off) throw Error("read past the end of the file");
    }
    uint8_t u8(uint64_t o) const { need(o, 1); return buf_[o]; }
    uint16_t u16(uint64_t o) const { need(o, 2); uint16_t v; std::memcpy(&v, &buf_[o], 2); return v; }
    uint32_t u32(uint64_t o) const { need(o, 4); uint32_t v; std::memcpy(&v, &buf_[o], 4); return v; }
    uint64_t u64(uint64_t o) const { need(o, 8); uint64_t v; std::memcpy(&v, &buf_[o], 8); return v; }
    bool sig(uint64_t o, const char* s) const { need(o, 4); return std::memcmp(&buf_[o], s, 4) == 0; }

    struct Msg {
        int type;
        uint64_t body;
        uint32_t size;
    };

    // The messages of a version-1 object header, continuation blocks included.
    std::vector<Msg> messages(uint64_t addr) const {
        if (u8(addr) != 1) throw Error("object header version " + std::to_string(u8(addr)));
        const uint32_t n = u16(addr + 2);
        std::vector<std::pair<uint64_t, uint64_t>> blocks{{addr + 16, u32(addr + 8)}};
        std::vector<Msg> out;
        for (size_t b = 0; b < blocks.size() && out.size() < n; b++) {
            uint64_t p = blocks[b].first;
            const uint64_t end = p + blocks[b].second;
            while (p + 8 <= end && out.size() < n) {
                Msg m{(int)u16(p), p + 8, u16(p + 2)};
                need(m.body, m.size);
                if (m.type == 0x10) blocks.push_back({u64(m.body), u64(m.body + 8)});
                out.push_back(m);
                p = m.body + m.size;
            }
        }
        return out;
    }

    std::string heap_string(uint64_t heap, uint64_t off) const {
        if (!sig(heap, "HEAP")) throw Error("bad local heap");
        const uint64_t s = u64(heap + 24) + off;
        std::string r;
        for (uint64_t p = s; u8(p) != 0; p++) r.push_back((char)u8(p));
        return r;
    }

    void read_btree(uint64_t node, uint64_t heap, int depth) {
        if (depth > 32 || !sig(node, "TREE") || u8(node + 4) != 0) throw Error("bad group B-tree");
        const int level = u8(node + 5);
        const int n = u16(node + 6);
        for (int i = 0; i < n; i++) {
            const uint64_t child = u64(node + 32 + 16 * (uint64_t)i);
            if (level > 0) {
                read_btree(child, heap, depth + 1);
                continue;
            }
            if (!sig(child, "SNOD")) throw Error("bad symbol table node");
            const int ns = u16(child + 6);
            for (int k = 0; k < ns; k++) {
                const uint64_t e = child + 8 + 40 * (uint64_t)k;
                links_[heap_string(heap, u64(e))] = u64(e + 8);
            }
        }
    }

    void read_group(uint64_t header) {
        for (const Msg& m : messages(header))
            if (m.type == 0x11) {  // symbol table message: B-tree, local heap
                read_btree(u64(m.body), u64(m.body + 8), 0);
                return;
            }
        throw Error("the root group is not a symbol-table group");
    }

    Type parse_type(uint64_t p) const {
        Type t;
        t.cls = u8(p) & 15;
        const uint8_t bits = u8(p + 1);
        t.size = (int)u32(p + 4);
        if (t.cls != 0 && t.cls != 1) throw Error("datatype class " + std::to_string(t.cls));
        if (bits & 1) throw Error("big-endian data");
        if (t.cls == 1 && (bits & 0x40)) throw Error("VAX-order floating point");
        t.is_signed = t.cls == 1 || (bits & 8);
        if (t.size != 4 && t.size != 8) throw Error("element size " + std::to_string(t.size));
        return t;
    }

    // dims of a dataspace message; rank 0 (scalar) gives no dims
    std::vector<uint64_t> parse_space(uint64_t p) const {
        const int ver = u8(p), rank = u8(p + 1);
        const uint64_t d0 = ver == 1 ? p + 8 : p + 4;
        if (ver != 1 && ver != 2) throw Error("dataspace version " + std::to_string(ver));
        std::vector<uint64_t> dims((size_t)rank);
        for (int i = 0; i < rank; i++) dims[(size_t)i] = u64(d0 + 8 * (uint64_t)i);
        return dims;
    }

    // Scalar numeric attributes are kept; others (strings, arrays) are skipped.
    bool parse_attribute(uint64_t p, std::string& name, Attribute& a) const {
        const int ver = u8(p);
        if (ver < 1 || ver > 3) throw Error("attribute message version " + std::to_string(ver));
        const uint64_t nlen = u16(p + 2), tlen = u16(p + 4), slen = u16(p + 6);
        auto pad = [ver](uint64_t n) { return ver == 1 ? (n + 7) & ~uint64_t(7) : n; };
        uint64_t q = p + 8 + (ver == 3 ? 1 : 0);
        need(q, nlen);
        name.assign(reinterpret_cast<const char*>(&buf_[q]), strnlen(reinterpret_cast<const char*>(&buf_[q]), nlen));
        q += pad(nlen);
        const int cls = u8(q) & 15;
        if (cls != 0 && cls != 1) return false;
        a.type = parse_type(q);
        q += pad(tlen);
        uint64_t n = 1;
        for (uint64_t dim : parse_space(q)) n *= dim;
        if (n != 1) return false;
        q += pad(slen);
        need(q, (uint64_t)a.type.size);
        a.data.assign(&buf_[q], &buf_[q] + a.type.size);
        return true;
    }

    Dataset read_dataset(uint64_t header) const {
        Dataset d;
        bool have_space = false, have_type = false, have_layout = false;
        for (const Msg& m : messages(header)) {
            const uint64_t p = m.body;
            if (m.type == 0x1) {
                d.dims = parse_space(p);
                have_space = true;
            } else if (m.type == 0x3) {
                d.type = parse_type(p);
                have_type = true;
            } else if (m.type == 0x8) {
                if (u8(p) != 3) throw Error("layout message version " + std::to_string(u8(p)));
                const int cls = u8(p + 1);
                if (cls == 0) {
                    const uint64_t n = u16(p + 2);
                    need(p + 4, n);
                    d.compact.assign(&buf_[p + 4], &buf_[p + 4] + n);
                    d.size = n;
                    d.is_compact = true;
                } else if (cls == 1) {
                    d.addr = u64(p + 2);
                    d.size = u64(p + 10);
                } else {
                    throw Error("chunked dataset");
                }
                have_layout = true;
            } else if (m.type == 0xB) {
                throw Error("filtered dataset");
            } else if (m.type == 0xC) {
                std::string name;
                Attribute a;
                if (parse_attribute(p, name, a)) d.attrs[name] = a;
            }
        }
        if (!have_space || !have_type || !have_layout) throw Error("object is not a dataset");
        return d;
    }

    const uint8_t* raw(const Dataset& d, size_t n) const {
        const uint64_t bytes = (uint64_t)n * (uint64_t)d.type.size;
        if (n == 0) return nullptr;
        if (d.is_compact) {
            if (d.compact.size() < bytes) throw Error("short compact data");
            return d.compact.data();
        }
        if (d.addr == ~uint64_t(0)) throw Error("dataset storage not allocated");
        if (d.size < bytes) throw Error("short contiguous data");
        need(d.addr, bytes);
        return &buf_[d.addr];
    }

    // Little-endian storage read on a little-endian host (x86-64 and aarch64).
    static double value(const Type& t, const uint8_t* p) {
        if (t.cls == 1) {
            if (t.size == 4) {
                float f;
                std::memcpy(&f, p, 4);
                return f;
            }
            double v;
            std::memcpy(&v, p, 8);
            return v;
        }
        return (double)ivalue(t, p);
    }

    static int64_t ivalue(const Type& t, const uint8_t* p) {
        if (t.cls == 1) return (int64_t)value(t, p);
        if (t.size == 4) {
            if (t.is_signed) {
                int32_t v;
                std::memcpy(&v, p, 4);
                return v;
            }
            uint32_t v;
            std::memcpy(&v, p, 4);
            return v;
        }
        int64_t v;
        std::memcpy(&v, p, 8);
        return v;
    }

    static const Attribute& attr(const Dataset& d, const std::string& name) {
        auto it = d.attrs.find(name);
        if (it == d.attrs.end()) throw Error("no attribute " + name);
        return it->second;
    }
};

}  // namespace h5
}  // namespace teufel_gb300
