// HDF5 writer of the classic file layout (host only; no HDF5 library).
//
// Byte layout, all fields little-endian, 8-byte offsets and lengths, every
// structure 8-byte aligned:
//
//   superblock v0 (96 B)      signature, versions 0, group K values, base 0,
//                             end-of-file address, root symbol-table entry
//                             (cache type 1: B-tree and heap addresses)
//   local heap "HEAP"         32 B header + data segment: "" at offset 0, then
//                             each name NUL-terminated and padded to 8, then
//                             one 16 B free block (next = 1 ends the list)
//   B-tree "TREE" (type 0)    one leaf node of 2 K_int children: key 0 = the
//                             empty name, child 0 = the symbol-table node,
//                             key 1 = the largest name
//   root object header v1     symbol-table message (B-tree, heap), one
//                             attribute message per root attribute
//   symbol-table node "SNOD"  2 K_leaf entries of 40 B, names in byte order
//   dataset object headers v1 fill value, datatype (IEEE float64 LE),
//                             dataspace v1, layout v2 (contiguous)
//   raw data                  row-major float64, one block per dataset
//
// The message encodings are those the HDF5 library itself writes for a
// float64 dataset in this layout; the output schema (names, widths, the
// time column) is the reference's (src/manager.cpp:51-201,
// src/tsurff.cpp:1018-1057).
#include "h5file.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <filesystem>

#include "common.h"

namespace tdz {

namespace {

constexpr uint64_t kUndef = ~0ull;
constexpr int kBtreeK = 16;   // group internal-node K: children per B-tree node = 2 K

uint64_t align8(uint64_t v) { return (v + 7) & ~7ull; }

struct Image {
    std::vector<uint8_t> b;
    void u8(uint64_t at, unsigned v) { b[at] = (uint8_t)v; }
    void u16(uint64_t at, unsigned v) { for (int i = 0; i < 2; ++i) b[at + i] = (uint8_t)(v >> (8 * i)); }
    void u32(uint64_t at, uint32_t v) { for (int i = 0; i < 4; ++i) b[at + i] = (uint8_t)(v >> (8 * i)); }
    void u64(uint64_t at, uint64_t v) { for (int i = 0; i < 8; ++i) b[at + i] = (uint8_t)(v >> (8 * i)); }
    void f64(uint64_t at, double v) {
        uint64_t u;
        std::memcpy(&u, &v, 8);
        u64(at, u);
    }
    void bytes(uint64_t at, const void *p, size_t n) { std::memcpy(b.data() + at, p, n); }
};

// IEEE float64, little-endian: class 1 (floating point), version 1; bit
// field: mantissa normalisation 2 (implied leading one), sign at bit 63;
// size 8; bit offset 0, precision 64, exponent at 52 (11 bits), mantissa at
// 0 (52 bits), bias 1023. 20 bytes.
constexpr size_t kF64TypeBytes = 20;
void put_f64_type(Image &im, uint64_t at) {
    im.u8(at, 0x11);
    im.u8(at + 1, 0x20);
    im.u8(at + 2, 63);
    im.u8(at + 3, 0);
    im.u32(at + 4, 8);
    im.u16(at + 8, 0);
    im.u16(at + 10, 64);
    im.u8(at + 12, 52);
    im.u8(at + 13, 11);
    im.u8(at + 14, 0);
    im.u8(at + 15, 52);
    im.u32(at + 16, 1023);
}

// Dataspace message version 1 without maximum dimensions: 8 + 8 rank bytes
// (rank 0: a scalar).
size_t dataspace_bytes(size_t rank) { return 8 + 8 * rank; }
void put_dataspace(Image &im, uint64_t at, const std::vector<uint64_t> &dims) {
    im.u8(at, 1);
    im.u8(at + 1, (unsigned)dims.size());
    for (size_t i = 0; i < dims.size(); ++i) im.u64(at + 8 + 8 * i, dims[i]);
}

uint64_t elements(const std::vector<uint64_t> &dims) {
    uint64_t n = 1;
    for (uint64_t d : dims) n *= d;
    return n;
}

// Attribute message version 1: header, name, datatype and dataspace each
// padded to 8, then the values.
size_t attr_message_bytes(const H5Array &a) {
    return align8(8 + align8(a.name.size() + 1) + align8(kF64TypeBytes) + dataspace_bytes(a.dims.size()) +
                  8 * elements(a.dims));
}

// Object-header message: type, size of the (8-padded) body, flags.
void put_message_header(Image &im, uint64_t at, unsigned type, size_t body, unsigned flags) {
    im.u16(at, type);
    im.u16(at + 2, (unsigned)body);
    im.u8(at + 4, flags);
}

void check_name(const std::string &n, const char *what) {
    TDZ_CHECK(!n.empty() && n != "." && n.find('/') == std::string::npos && n.find('\0') == std::string::npos,
              TDZ_ERR_ARG, std::string("invalid ") + what + " name '" + n + "'");
}

}  // namespace

void h5_write_file(const std::string &path, const std::vector<H5Array> &datasets_in,
                   const std::vector<H5Array> &attrs) {
    TDZ_CHECK(!path.empty(), TDZ_ERR_ARG, "empty file name");
    std::vector<H5Array> ds = datasets_in;
    std::sort(ds.begin(), ds.end(), [](const H5Array &a, const H5Array &b) {
        return std::strcmp(a.name.c_str(), b.name.c_str()) < 0;
    });
    for (size_t i = 0; i < ds.size(); ++i) {
        check_name(ds[i].name, "dataset");
        TDZ_CHECK(i == 0 || ds[i].name != ds[i - 1].name, TDZ_ERR_ARG, "duplicate dataset name '" + ds[i].name + "'");
        TDZ_CHECK(!ds[i].dims.empty() && ds[i].dims.size() <= 8, TDZ_ERR_ARG,
                  "dataset '" + ds[i].name + "' must have rank 1 to 8");
        for (uint64_t d : ds[i].dims)
            TDZ_CHECK(d >= 1 && d <= 0xffffffffull, TDZ_ERR_ARG, "dataset '" + ds[i].name + "' has an empty or too long axis");
        TDZ_CHECK(ds[i].data != nullptr, TDZ_ERR_ARG, "dataset '" + ds[i].name + "' has no data");
    }
    for (size_t i = 0; i < attrs.size(); ++i) {
        check_name(attrs[i].name, "attribute");
        for (size_t j = 0; j < i; ++j)
            TDZ_CHECK(attrs[j].name != attrs[i].name, TDZ_ERR_ARG, "duplicate attribute name '" + attrs[i].name + "'");
        TDZ_CHECK(attrs[i].dims.size() <= 8 && attrs[i].data != nullptr, TDZ_ERR_ARG,
                  "attribute '" + attrs[i].name + "' needs data and rank <= 8");
        TDZ_CHECK(attr_message_bytes(attrs[i]) <= 0xffff, TDZ_ERR_ARG,
                  "attribute '" + attrs[i].name + "' is larger than one object-header message");
    }
    const size_t n = ds.size();
    const int leaf_k = std::max<int>(4, (int)((n + 1) / 2));   // one symbol-table node holds 2 K entries

    // ---- addresses
    const uint64_t a_heap = 96, a_heap_data = a_heap + 32;
    std::vector<uint64_t> name_off(n);
    uint64_t heap_used = 8;                                    // "" at offset 0
    for (size_t i = 0; i < n; ++i) {
        name_off[i] = heap_used;
        heap_used += align8(ds[i].name.size() + 1);
    }
    const uint64_t heap_size = heap_used + 16;                 // one free block at the end
    const uint64_t a_btree = align8(a_heap_data + heap_size);
    const uint64_t btree_bytes = 24 + 2 * kBtreeK * 8 + (2 * kBtreeK + 1) * 8;
    const uint64_t a_root = a_btree + btree_bytes;
    uint64_t root_msgs = 8 + 16;                               // symbol-table message
    for (const H5Array &a : attrs) root_msgs += 8 + attr_message_bytes(a);
    const uint64_t a_snod = a_root + 16 + root_msgs;
    const uint64_t snod_bytes = 8 + (uint64_t)2 * leaf_k * 40;
    std::vector<uint64_t> a_oh(n), oh_msgs(n), a_data(n);
    uint64_t at = a_snod + snod_bytes;
    for (size_t i = 0; i < n; ++i) {
        const size_t r = ds[i].dims.size();
        oh_msgs[i] = (8 + 8) + (8 + align8(kF64TypeBytes)) + (8 + dataspace_bytes(r)) + (8 + align8(16 + 4 * (r + 1)));
        a_oh[i] = at;
        at += 16 + oh_msgs[i];
    }
    for (size_t i = 0; i < n; ++i) {
        a_data[i] = at;
        at += align8(8 * elements(ds[i].dims));
    }
    const uint64_t eof = at;

    Image im;
    im.b.assign(eof, 0);

    // ---- superblock
    const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    im.bytes(0, sig, 8);
    im.u8(13, 8);                                              // size of offsets
    im.u8(14, 8);                                              // size of lengths
    im.u16(16, (unsigned)leaf_k);
    im.u16(18, kBtreeK);
    im.u64(24, 0);                                             // base address
    im.u64(32, kUndef);                                        // free-space info
    im.u64(40, eof);
    im.u64(48, kUndef);                                        // driver info block
    im.u64(56, 0);                                             // root link name: ""
    im.u64(64, a_root);
    im.u32(72, 1);                                             // cache type 1: group
    im.u64(80, a_btree);
    im.u64(88, a_heap);

    // ---- local heap of names
    im.bytes(a_heap, "HEAP", 4);
    im.u64(a_heap + 8, heap_size);
    im.u64(a_heap + 16, heap_used);                            // head of the free list
    im.u64(a_heap + 24, a_heap_data);
    for (size_t i = 0; i < n; ++i) im.bytes(a_heap_data + name_off[i], ds[i].name.c_str(), ds[i].name.size());
    im.u64(a_heap_data + heap_used, 1);                        // next free block: none
    im.u64(a_heap_data + heap_used + 8, 16);                   // size of this free block

    // ---- B-tree: one leaf over the symbol-table node
    im.bytes(a_btree, "TREE", 4);
    im.u8(a_btree + 4, 0);                                     // node type 0: group
    im.u8(a_btree + 5, 0);                                     // level 0: leaf
    im.u16(a_btree + 6, n ? 1 : 0);
    im.u64(a_btree + 8, kUndef);
    im.u64(a_btree + 16, kUndef);
    im.u64(a_btree + 24, 0);                                   // key 0: ""
    if (n) {
        im.u64(a_btree + 32, a_snod);
        im.u64(a_btree + 40, name_off[n - 1]);                 // key 1: the largest name
    }

    // ---- root group object header
    {
        const unsigned nmsg = 1 + (unsigned)attrs.size();
        im.u8(a_root, 1);
        im.u16(a_root + 2, nmsg);
        im.u32(a_root + 4, 1);                                 // reference count
        im.u32(a_root + 8, (uint32_t)root_msgs);
        uint64_t m = a_root + 16;
        put_message_header(im, m, 0x0011, 16, 1);              // symbol table
        im.u64(m + 8, a_btree);
        im.u64(m + 16, a_heap);
        m += 24;
        for (const H5Array &a : attrs) {
            const size_t body = attr_message_bytes(a);
            put_message_header(im, m, 0x000C, body, 0);
            uint64_t p = m + 8;
            im.u8(p, 1);                                       // attribute message version 1
            im.u16(p + 2, (unsigned)(a.name.size() + 1));
            im.u16(p + 4, (unsigned)kF64TypeBytes);
            im.u16(p + 6, (unsigned)dataspace_bytes(a.dims.size()));
            p += 8;
            im.bytes(p, a.name.c_str(), a.name.size());
            p += align8(a.name.size() + 1);
            put_f64_type(im, p);
            p += align8(kF64TypeBytes);
            put_dataspace(im, p, a.dims);
            p += dataspace_bytes(a.dims.size());
            const uint64_t ne = elements(a.dims);
            for (uint64_t e = 0; e < ne; ++e) im.f64(p + 8 * e, a.data[e]);
            m += 8 + body;
        }
    }

    // ---- symbol-table node
    if (n) {
        im.bytes(a_snod, "SNOD", 4);
        im.u8(a_snod + 4, 1);                                  // version 1
        im.u16(a_snod + 6, (unsigned)n);
        for (size_t i = 0; i < n; ++i) {
            const uint64_t e = a_snod + 8 + 40 * i;
            im.u64(e, name_off[i]);
            im.u64(e + 8, a_oh[i]);                            // cache type 0, scratch zero
        }
    }

    // ---- dataset object headers and data
    for (size_t i = 0; i < n; ++i) {
        const H5Array &d = ds[i];
        const size_t r = d.dims.size();
        const uint64_t o = a_oh[i];
        im.u8(o, 1);
        im.u16(o + 2, 4);                                      // four messages
        im.u32(o + 4, 1);
        im.u32(o + 8, (uint32_t)oh_msgs[i]);
        uint64_t m = o + 16;
        // fill value, version 1: allocation late, fill written if set, the
        // default (zero) fill value
        put_message_header(im, m, 0x0005, 8, 1);
        im.u8(m + 8, 1);
        im.u8(m + 9, 2);
        im.u8(m + 10, 2);
        im.u8(m + 11, 1);
        m += 16;
        put_message_header(im, m, 0x0003, align8(kF64TypeBytes), 1);
        put_f64_type(im, m + 8);
        m += 8 + align8(kF64TypeBytes);
        put_message_header(im, m, 0x0001, dataspace_bytes(r), 0);
        put_dataspace(im, m + 8, d.dims);
        m += 8 + dataspace_bytes(r);
        // layout, version 2: contiguous, address, the dims and the element size
        const size_t lay = align8(16 + 4 * (r + 1));
        put_message_header(im, m, 0x0008, lay, 1);
        im.u8(m + 8, 2);
        im.u8(m + 9, (unsigned)(r + 1));
        im.u8(m + 10, 1);
        im.u64(m + 16, a_data[i]);
        for (size_t k = 0; k < r; ++k) im.u32(m + 24 + 4 * k, (uint32_t)d.dims[k]);
        im.u32(m + 24 + 4 * r, 8);
        const uint64_t ne = elements(d.dims);
        for (uint64_t e = 0; e < ne; ++e) im.f64(a_data[i] + 8 * e, d.data[e]);
    }

    // ---- write beside the target, then rename over it
    std::error_code ec;
    const std::filesystem::path target(path);
    if (target.has_parent_path()) std::filesystem::create_directories(target.parent_path(), ec);
    const std::string part = path + ".part";
    std::FILE *f = std::fopen(part.c_str(), "wb");
    TDZ_CHECK(f != nullptr, TDZ_ERR_ARG, "cannot create " + part);
    const bool ok = std::fwrite(im.b.data(), 1, im.b.size(), f) == im.b.size();
    const bool closed = std::fclose(f) == 0;
    if (!ok || !closed) std::remove(part.c_str());
    TDZ_CHECK(ok && closed, TDZ_ERR_INTERNAL, "cannot write " + part);
    if (std::rename(part.c_str(), path.c_str()) != 0) {
        std::remove(part.c_str());
        TDZ_CHECK(false, TDZ_ERR_INTERNAL, "cannot rename " + part + " to " + path);
    }
}

// ------------------------------------------------------------ observables

const char *const ObsFile::kNames[ObsFile::kSets] = {"dipoles", "populations", "energies", "currents",
                                                     "autocorrelation"};

ObsFile::ObsFile(const std::string &path, int dim, int n_bound, long long flush_rows)
    : path_(path), flush_rows_(flush_rows > 0 ? flush_rows : 5000) {
    TDZ_CHECK(!path.empty(), TDZ_ERR_ARG, "empty file name");
    TDZ_CHECK(dim >= 1 && dim <= 3, TDZ_ERR_ARG, "dimension must be 1, 2 or 3");
    TDZ_CHECK(n_bound >= 0, TDZ_ERR_ARG, "negative number of bound states");
    cols_ = {1 + 3 * dim, 1 + n_bound, 7, dim == 3 ? 15 : 11, 3};
}

void ObsFile::record(double t, const double *const *rows) {
    for (int s = 0; s < kSets; ++s) {
        std::vector<double> &d = data_[s];
        d.push_back(t);
        const double *r = rows ? rows[s] : nullptr;
        for (int c = 1; c < cols_[s]; ++c) d.push_back(r ? r[c - 1] : 0.0);
    }
    ++nrows_;
    if (nrows_ - written_ >= flush_rows_) flush();
}

void ObsFile::flush() {
    if (nrows_ == written_) return;
    std::vector<H5Array> sets(kSets);
    for (int s = 0; s < kSets; ++s) {
        sets[s].name = kNames[s];
        sets[s].dims = {(uint64_t)nrows_, (uint64_t)cols_[s]};
        sets[s].data = data_[s].data();
    }
    h5_write_file(path_, sets, {});
    written_ = nrows_;
}

}  // namespace tdz
