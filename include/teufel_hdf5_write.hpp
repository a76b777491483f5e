// teufel_hdf5_write.hpp -- a minimal HDF5 writer for the observer output files
// TEUFEL writes with the HDF5 library: MeshedScreen::writeFile
// (src/mesh.cpp:428-736) and ScreenObserver::WriteTimeDomainFieldHDF5
// (src/screen.cpp:298-560).  Written from the HDF5 file-format specification
// for builds without the HDF5 library.
//
// The file has the structure the HDF5 library gives such a file when it is
// created with default properties: superblock version 0 with 8-byte offsets
// and lengths; the root group as a symbol table (one version-1 B-tree leaf of
// group-node K 16, one symbol-table node of leaf K 4, a local heap of link
// names); one version-1 object header per dataset holding a dataspace
// (version 1, maximum dimensions = dimensions), a datatype (little-endian
// IEEE 64-bit float or 32-bit signed integer, the native types on x86-64 and
// aarch64), a fill-value message, a contiguous layout (version 3) and scalar
// attributes (attribute message version 1).  Up to 8 datasets in the root
// group, which is what one symbol-table node holds; the observers write 3 or 5.
//
// Datasets reference the caller's arrays, which must stay alive until write().
#pragma once

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "teufel_hdf5_read.hpp"

namespace teufel_gb300 {
namespace h5 {

// A scalar attribute: H5T_NATIVE_INT (32-bit signed) or H5T_NATIVE_DOUBLE.
struct AttrOut {
    std::string name;
    bool is_float = false;
    int32_t i = 0;
    double d = 0.0;
    static AttrOut Int(const std::string& n, int32_t v) {
        AttrOut a;
        a.name = n;
        a.i = v;
        return a;
    }
    static AttrOut Double(const std::string& n, double v) {
        AttrOut a;
        a.name = n;
        a.is_float = true;
        a.d = v;
        return a;
    }
};

class Writer {
public:
    void add(const std::string& name, std::vector<uint64_t> dims, const double* data,
             std::vector<AttrOut> attrs = {}) {
        push(name, std::move(dims), true, data, std::move(attrs));
    }
    void add(const std::string& name, std::vector<uint64_t> dims, const int32_t* data,
             std::vector<AttrOut> attrs = {}) {
        push(name, std::move(dims), false, data, std::move(attrs));
    }

    void write(const std::string& path) const;

private:
    struct DS {
        std::string name;
        std::vector<uint64_t> dims;
        bool is_float;
        const void* data;
        std::vector<AttrOut> attrs;
        uint64_t elem() const { return is_float ? 8 : 4; }
        uint64_t bytes() const {
            uint64_t n = elem();
            for (uint64_t d : dims) n *= d;
            return n;
        }
    };
    std::vector<DS> ds_;

    void push(const std::string& name, std::vector<uint64_t> dims, bool is_float, const void* data,
              std::vector<AttrOut> attrs) {
        if (name.empty()) throw Error("empty dataset name");
        for (const DS& d : ds_)
            if (d.name == name) throw Error("dataset " + name + " added twice");
        if (ds_.size() == kMaxLinks) throw Error("more than 8 datasets in one file");
        if (dims.empty() || dims.size() > 32) throw Error("dataset rank must be 1..32");
        ds_.push_back(DS{name, std::move(dims), is_float, data, std::move(attrs)});
    }

    static constexpr std::size_t kMaxLinks = 8;      // 2 x group leaf K (4)
    static constexpr uint64_t kUndef = ~uint64_t(0);  // the undefined address
    static constexpr uint64_t kSuperblock = 96;
    static constexpr uint64_t kRootHeader = 40;       // 16 prefix + one 24-byte message
    static constexpr uint64_t kBTreeNode = 24 + 33 * 8 + 32 * 8;  // internal K 16: 2K children, 2K+1 keys
    static constexpr uint64_t kSymbolNode = 8 + kMaxLinks * 40;

    static uint64_t pad8(uint64_t n) { return (n + 7) & ~uint64_t(7); }

    // little-endian field writers into a byte buffer
    static void put(std::vector<uint8_t>& b, uint64_t v, int n) {
        for (int k = 0; k < n; k++) b.push_back((uint8_t)(v >> (8 * k)));
    }
    static void zeros(std::vector<uint8_t>& b, uint64_t n) { b.insert(b.end(), (std::size_t)n, 0); }
    static void align8(std::vector<uint8_t>& b) { zeros(b, pad8(b.size()) - b.size()); }

    static std::vector<uint8_t> datatype(bool is_float) {
        std::vector<uint8_t> b;
        if (is_float) {
            // class 1 (floating point), version 1; little-endian, implied
            // leading mantissa bit, sign at bit 63
            b = {0x11, 0x20, 0x3f, 0x00};
            put(b, 8, 4);
            put(b, 0, 2);   // bit offset
            put(b, 64, 2);  // bit precision
            b.push_back(52);  // exponent location
            b.push_back(11);  // exponent size
            b.push_back(0);   // mantissa location
            b.push_back(52);  // mantissa size
            put(b, 1023, 4);  // exponent bias
        } else {
            b = {0x10, 0x08, 0x00, 0x00};  // class 0 (fixed point), version 1; little-endian, signed
            put(b, 4, 4);
            put(b, 0, 2);
            put(b, 32, 2);
        }
        return b;
    }

    static void message(std::vector<uint8_t>& h, int type, int flags, const std::vector<uint8_t>& body) {
        put(h, (uint64_t)type, 2);
        put(h, pad8(body.size()), 2);
        put(h, (uint64_t)flags, 1);
        zeros(h, 3);
        h.insert(h.end(), body.begin(), body.end());
        align8(h);
    }

    static std::vector<uint8_t> attribute(const AttrOut& a) {
        const std::vector<uint8_t> dt = datatype(a.is_float);
        std::vector<uint8_t> b = {1, 0};
        put(b, a.name.size() + 1, 2);
        put(b, dt.size(), 2);
        put(b, 8, 2);  // scalar dataspace
        b.insert(b.end(), a.name.begin(), a.name.end());
        b.push_back(0);
        align8(b);
        b.insert(b.end(), dt.begin(), dt.end());
        align8(b);
        const uint8_t scalar[8] = {1, 0, 0, 0, 0, 0, 0, 0};  // version 1, rank 0
        b.insert(b.end(), scalar, scalar + 8);
        if (a.is_float) {
            uint64_t v;
            std::memcpy(&v, &a.d, 8);
            put(b, v, 8);
        } else {
            put(b, (uint64_t)(uint32_t)a.i, 4);
        }
        return b;
    }

    static std::vector<uint8_t> header(const DS& d, uint64_t addr) {
        std::vector<uint8_t> msgs;
        int n = 0;
        std::vector<uint8_t> b = {1, (uint8_t)d.dims.size(), 1, 0};  // version 1, rank, max dims present
        zeros(b, 4);
        for (uint64_t x : d.dims) put(b, x, 8);
        for (uint64_t x : d.dims) put(b, x, 8);
        message(msgs, 0x1, 0, b), n++;
        message(msgs, 0x3, 1, datatype(d.is_float)), n++;
        // fill value version 2: allocation late, write if set, library default value
        message(msgs, 0x5, 1, {2, 2, 2, 1, 0, 0, 0, 0}), n++;
        b = {3, 1};  // layout version 3, contiguous
        put(b, addr, 8);
        put(b, d.bytes(), 8);
        message(msgs, 0x8, 0, b), n++;
        for (const AttrOut& a : d.attrs) message(msgs, 0xC, 0, attribute(a)), n++;
        std::vector<uint8_t> h = {1, 0};
        put(h, (uint64_t)n, 2);
        put(h, 1, 4);  // reference count
        put(h, msgs.size(), 4);
        zeros(h, 4);
        h.insert(h.end(), msgs.begin(), msgs.end());
        return h;
    }
};

inline void Writer::write(const std::string& path) const {
    const uint16_t probe = 1;
    uint8_t low;
    std::memcpy(&low, &probe, 1);
    if (low != 1) throw Error("the writer needs a little-endian host");
    if (ds_.empty()) throw Error("no datasets to write");
    const std::size_t n = ds_.size();

    // link names in the local heap; offset 0 holds the empty name
    std::vector<uint8_t> heap(8, 0);
    std::vector<uint64_t> name_off(n);
    for (std::size_t i = 0; i < n; i++) {
        name_off[i] = heap.size();
        heap.insert(heap.end(), ds_[i].name.begin(), ds_[i].name.end());
        heap.push_back(0);
        align8(heap);
    }
    std::vector<std::size_t> order(n);
    for (std::size_t i = 0; i < n; i++) order[i] = i;
    std::sort(order.begin(), order.end(),
              [this](std::size_t a, std::size_t b) { return ds_[a].name < ds_[b].name; });

    const uint64_t btree_addr = kSuperblock + kRootHeader;
    const uint64_t heap_addr = btree_addr + kBTreeNode;
    const uint64_t snod_addr = heap_addr + 32 + heap.size();
    uint64_t p = snod_addr + kSymbolNode;
    std::vector<uint64_t> hdr_addr(n), data_addr(n);
    for (std::size_t i = 0; i < n; i++) {
        hdr_addr[i] = p;
        p += header(ds_[i], 0).size();
    }
    const uint64_t meta_end = p;
    for (std::size_t i = 0; i < n; i++) {
        p = pad8(p);
        data_addr[i] = ds_[i].bytes() ? p : kUndef;
        p += ds_[i].bytes();
    }
    const uint64_t eof = p;

    std::vector<uint8_t> m;
    const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    m.insert(m.end(), sig, sig + 8);
    zeros(m, 5);  // superblock, free-space, root entry and shared-header versions 0; reserved
    m.push_back(8);  // size of offsets
    m.push_back(8);  // size of lengths
    m.push_back(0);
    put(m, 4, 2);   // group leaf node K
    put(m, 16, 2);  // group internal node K
    put(m, 0, 4);   // consistency flags
    put(m, 0, 8);   // base address
    put(m, kUndef, 8);
    put(m, eof, 8);
    put(m, kUndef, 8);
    // root group symbol table entry, cache type 1 (B-tree and heap addresses)
    put(m, 0, 8);
    put(m, kSuperblock, 8);
    put(m, 1, 4);
    put(m, 0, 4);
    put(m, btree_addr, 8);
    put(m, heap_addr, 8);

    // root group object header: one symbol table message
    m.insert(m.end(), {1, 0});
    put(m, 1, 2);
    put(m, 1, 4);
    put(m, 24, 4);
    zeros(m, 4);
    put(m, 0x11, 2);
    put(m, 16, 2);
    zeros(m, 4);
    put(m, btree_addr, 8);
    put(m, heap_addr, 8);

    // group B-tree: one leaf entry pointing at the symbol table node
    m.insert(m.end(), {'T', 'R', 'E', 'E', 0, 0});
    put(m, 1, 2);
    put(m, kUndef, 8);
    put(m, kUndef, 8);
    put(m, 0, 8);
    put(m, snod_addr, 8);
    put(m, name_off[order.back()], 8);
    zeros(m, heap_addr - m.size());

    // local heap: header then data segment; free list empty (offset 1)
    m.insert(m.end(), {'H', 'E', 'A', 'P', 0, 0, 0, 0});
    put(m, heap.size(), 8);
    put(m, 1, 8);
    put(m, heap_addr + 32, 8);
    m.insert(m.end(), heap.begin(), heap.end());

    // symbol table node: the links sorted by name
    m.insert(m.end(), {'S', 'N', 'O', 'D', 1, 0});
    put(m, n, 2);
    for (std::size_t k : order) {
        put(m, name_off[k], 8);
        put(m, hdr_addr[k], 8);
        zeros(m, 24);  // cache type 0, reserved, scratch pad
    }
    zeros(m, snod_addr + kSymbolNode - m.size());

    for (std::size_t i = 0; i < n; i++) {
        const std::vector<uint8_t> h = header(ds_[i], data_addr[i]);
        m.insert(m.end(), h.begin(), h.end());
    }
    if (m.size() != meta_end) throw Error("internal layout error");

    std::ofstream f(path, std::ios::binary | std::ios::trunc);
    if (!f) throw Error("cannot create " + path);
    f.write(reinterpret_cast<const char*>(m.data()), (std::streamsize)m.size());
    uint64_t pos = m.size();
    const char pad[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (std::size_t i = 0; i < n; i++) {
        if (data_addr[i] == kUndef) continue;
        f.write(pad, (std::streamsize)(data_addr[i] - pos));
        f.write(static_cast<const char*>(ds_[i].data), (std::streamsize)ds_[i].bytes());
        pos = data_addr[i] + ds_[i].bytes();
    }
    f.close();
    if (!f) throw Error("error writing " + path);
}

}  // namespace h5
}  // namespace teufel_gb300
