#include "signal_file.hpp"

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <functional>
#include <map>
#include <stdexcept>

namespace sassgpu {

namespace {

constexpr uint64_t kUndef = ~0ull;
constexpr uint64_t kHeapFreeNull = 1;  // "no free block" marker of local heaps as libhdf5 writes it
constexpr int kLeafK = 4;              // symbol-table node: up to 2K = 8 entries
constexpr int kInternalK = 16;         // group B-tree node: up to 2K = 32 children
constexpr uint8_t kSignature[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};

// ------------------------------------------------------------------------------------------
// writer
// ------------------------------------------------------------------------------------------
struct Out {
    std::vector<uint8_t> b;
    void u8(uint64_t v) { b.push_back((uint8_t)v); }
    void u16(uint64_t v) { for (int i = 0; i < 2; ++i) b.push_back((uint8_t)(v >> (8 * i))); }
    void u32(uint64_t v) { for (int i = 0; i < 4; ++i) b.push_back((uint8_t)(v >> (8 * i))); }
    void u64(uint64_t v) { for (int i = 0; i < 8; ++i) b.push_back((uint8_t)(v >> (8 * i))); }
    void raw(const void* p, size_t n) {
        const uint8_t* c = static_cast<const uint8_t*>(p);
        b.insert(b.end(), c, c + n);
    }
    void zeros(size_t n) { b.insert(b.end(), n, 0); }
    void pad8() { while (b.size() % 8) b.push_back(0); }
    size_t size() const { return b.size(); }
};

enum Kind { F64 = 0, I8 = 1, STR = 2 };

struct DatasetSpec {
    std::string name;
    Kind kind;
    std::vector<uint64_t> dims;  // empty = scalar
    const uint8_t* data;
    uint64_t nbytes;
    uint64_t header_addr = 0, data_addr = 0;
    std::vector<uint64_t> chunk;       // chunked storage, unlimited first dimension (empty: contiguous)
    std::vector<uint8_t> chunk_region;  // B-tree nodes + chunks, placed at data_addr
    uint64_t btree_addr = kUndef;
};

struct Message {
    uint16_t type;
    uint8_t flags;
    std::vector<uint8_t> data;  // unpadded
};

std::vector<uint8_t> dataspace_msg(const std::vector<uint64_t>& dims, bool unlimited0) {
    Out o;
    o.u8(1);                          // version 1
    o.u8(dims.size());                // dimensionality (0 = scalar)
    o.u8(dims.empty() ? 0 : 1);       // flags: maximum dimensions present
    o.u8(0);
    o.u32(0);
    for (uint64_t d : dims) o.u64(d);
    for (size_t i = 0; i < dims.size(); ++i) o.u64(i == 0 && unlimited0 ? kUndef : dims[i]);
    return o.b;
}

std::vector<uint8_t> datatype_msg(Kind k, uint64_t str_size) {
    Out o;
    if (k == F64) {
        o.u8(0x11);                   // version 1, class 1 (floating point)
        o.u8(0x20);                   // little-endian, implied msb mantissa normalisation
        o.u8(63);                     // sign bit position
        o.u8(0);
        o.u32(8);
        o.u16(0);                     // bit offset
        o.u16(64);                    // bit precision
        o.u8(52);                     // exponent location
        o.u8(11);                     // exponent size
        o.u8(0);                      // mantissa location
        o.u8(52);                     // mantissa size
        o.u32(1023);                  // exponent bias
    } else if (k == I8) {
        o.u8(0x10);                   // version 1, class 0 (fixed point)
        o.u8(0x08);                   // little-endian, signed
        o.u8(0);
        o.u8(0);
        o.u32(1);
        o.u16(0);
        o.u16(8);
    } else {
        o.u8(0x13);                   // version 1, class 3 (string)
        o.u8(0x00);                   // null-terminated, ASCII
        o.u8(0);
        o.u8(0);
        o.u32((uint32_t)str_size);
    }
    return o.b;
}

std::vector<uint8_t> fill_msg(Kind k) {
    Out o;
    o.u8(2);  // version 2
    o.u8(2);  // space allocation time: late
    o.u8(2);  // fill value write time: if set
    if (k == F64) {
        o.u8(1);  // fill value defined: 0.0 (as the reference sets, file_writer_service.cpp:49)
        o.u32(8);
        o.u64(0);
    } else {
        o.u8(0);
    }
    return o.b;
}

std::vector<uint8_t> layout_msg(uint64_t addr, uint64_t size) {
    Out o;
    o.u8(3);  // version 3
    o.u8(1);  // contiguous
    o.u64(addr);
    o.u64(size);
    return o.b;
}

// Layout message, chunked: B-tree address and chunk dimensions plus the element size.
std::vector<uint8_t> chunked_layout_msg(uint64_t btree, const std::vector<uint64_t>& chunk, uint32_t esize) {
    Out o;
    o.u8(3);  // version 3
    o.u8(2);  // chunked
    o.u8(chunk.size() + 1);
    o.u64(btree);
    for (uint64_t c : chunk) o.u32(c);
    o.u32(esize);
    return o.b;
}

// Chunked storage of a row-major float64 dataset as libhdf5 lays it out: every chunk of
// the chunk grid over the dataset's extent is stored whole (fill value 0 outside the
// extent) and indexed by a version-1 B-tree of type 1 (raw data chunks) whose nodes hold
// up to 2K = 64 entries (K = 32, the default for chunk B-trees). Nodes come first in the
// region, then the chunks. Returns the region; `root` receives the root node's address.
std::vector<uint8_t> chunked_region(const DatasetSpec& s, uint64_t base, uint64_t& root) {
    constexpr int kChunkK = 32;
    const size_t rank = s.dims.size();
    const uint64_t es = 8;
    uint64_t chunk_elems = 1;
    std::vector<uint64_t> grid(rank);
    uint64_t nchunks = 1;
    for (size_t k = 0; k < rank; ++k) {
        chunk_elems *= s.chunk[k];
        grid[k] = (s.dims[k] + s.chunk[k] - 1) / s.chunk[k];
        nchunks *= grid[k];
    }
    root = kUndef;
    if (nchunks == 0) return {};
    const uint64_t key_bytes = 8 + 8 * (rank + 1);
    const uint64_t node_bytes = 24 + (2 * kChunkK + 1) * key_bytes + 2 * kChunkK * 8;
    // chunk offsets (element coordinates) in row-major grid order
    std::vector<std::vector<uint64_t>> offs(nchunks, std::vector<uint64_t>(rank));
    for (uint64_t c = 0; c < nchunks; ++c) {
        uint64_t r = c;
        for (size_t k = rank; k-- > 0;) {
            offs[c][k] = (r % grid[k]) * s.chunk[k];
            r /= grid[k];
        }
    }
    // tree shape: levels of nodes, each over at most 64 children
    std::vector<uint64_t> level_nodes;
    for (uint64_t n = nchunks;;) {
        n = (n + 2 * kChunkK - 1) / (2 * kChunkK);
        level_nodes.push_back(n);
        if (n == 1) break;
    }
    uint64_t total_nodes = 0;
    for (uint64_t n : level_nodes) total_nodes += n;
    const uint64_t chunk_base = base + total_nodes * node_bytes;
    Out o;
    auto key = [&](uint64_t csize, const std::vector<uint64_t>& off) {
        o.u32(csize);
        o.u32(0);  // filter mask
        for (uint64_t v : off) o.u64(v);
        o.u64(0);  // offset in the element-size dimension
    };
    std::vector<uint64_t> child_addr(nchunks);
    std::vector<std::vector<uint64_t>> child_left(offs);  // left key of every child
    for (uint64_t c = 0; c < nchunks; ++c) child_addr[c] = chunk_base + c * chunk_elems * es;
    std::vector<uint64_t> right = offs.back();  // right key of the last child
    right[0] += s.chunk[0];
    uint64_t node_addr = base;
    for (size_t lvl = 0; lvl < level_nodes.size(); ++lvl) {
        std::vector<uint64_t> next_addr;
        std::vector<std::vector<uint64_t>> next_left;
        const uint64_t nchild = child_addr.size();
        for (uint64_t n = 0; n < level_nodes[lvl]; ++n) {
            const uint64_t c0 = n * 2 * kChunkK, c1 = std::min(nchild, c0 + 2 * kChunkK);
            const size_t start = o.size();
            o.raw("TREE", 4);
            o.u8(1);  // node type: raw data chunks
            o.u8(lvl);
            o.u16(c1 - c0);
            o.u64(kUndef);
            o.u64(kUndef);
            for (uint64_t c = c0; c < c1; ++c) {
                key(lvl == 0 ? chunk_elems * es : 0, child_left[c]);
                o.u64(child_addr[c]);
            }
            key(0, c1 < nchild ? child_left[c1] : right);
            o.zeros(node_bytes - (o.size() - start));
            next_addr.push_back(node_addr);
            next_left.push_back(child_left[c0]);
            node_addr += node_bytes;
        }
        child_addr = next_addr;
        child_left = next_left;
    }
    root = child_addr.front();
    // chunks, zero outside the dataset's extent
    const double* src = reinterpret_cast<const double*>(s.data);
    std::vector<double> buf(chunk_elems);
    std::vector<uint64_t> idx(rank);
    for (uint64_t c = 0; c < nchunks; ++c) {
        for (uint64_t e = 0; e < chunk_elems; ++e) {
            uint64_t r = e, lin = 0;
            bool inside = true;
            for (size_t k = rank; k-- > 0;) {
                idx[k] = r % s.chunk[k];
                r /= s.chunk[k];
            }
            for (size_t k = 0; k < rank && inside; ++k) {
                const uint64_t g = offs[c][k] + idx[k];
                inside = g < s.dims[k];
                lin = lin * s.dims[k] + g;
            }
            buf[e] = inside ? src[lin] : 0.0;
        }
        o.raw(buf.data(), chunk_elems * es);
    }
    return o.b;
}

std::vector<uint8_t> symtab_msg(uint64_t btree, uint64_t heap) {
    Out o;
    o.u64(btree);
    o.u64(heap);
    return o.b;
}

size_t header_size(const std::vector<Message>& msgs) {
    size_t n = 16;
    for (const Message& m : msgs) n += 8 + ((m.data.size() + 7) & ~(size_t)7);
    return n;
}

void emit_header(Out& o, const std::vector<Message>& msgs) {
    size_t body = header_size(msgs) - 16;
    o.u8(1);  // version 1
    o.u8(0);
    o.u16(msgs.size());
    o.u32(1);  // reference count
    o.u32(body);
    o.u32(0);  // alignment padding
    for (const Message& m : msgs) {
        size_t padded = (m.data.size() + 7) & ~(size_t)7;
        o.u16(m.type);
        o.u16(padded);
        o.u8(m.flags);
        o.zeros(3);
        o.raw(m.data.data(), m.data.size());
        o.zeros(padded - m.data.size());
    }
}

// One group's on-disk pieces: object header, local heap (+ data), B-tree node, SNOD.
struct GroupLayout {
    std::vector<std::pair<std::string, uint64_t>> entries;  // name -> object header (sorted)
    std::vector<uint64_t> cache_btree, cache_heap;          // for subgroup entries (0 = none)
    std::vector<uint64_t> name_off;
    std::vector<uint8_t> heap_data;
    uint64_t header = 0, heap = 0, btree = 0, snod = 0;

    static constexpr size_t kHeaderBytes = 16 + 8 + 16;
    static constexpr size_t kHeapHdrBytes = 32;
    static constexpr size_t kBtreeBytes = 24 + (2 * kInternalK + 1) * 8 + 2 * kInternalK * 8;
    static constexpr size_t kSnodBytes = 8 + 2 * kLeafK * 40;

    void names(const std::vector<std::string>& sorted) {
        heap_data.assign(8, 0);  // offset 0: the empty name
        for (const std::string& n : sorted) {
            name_off.push_back(heap_data.size());
            heap_data.insert(heap_data.end(), n.begin(), n.end());
            heap_data.push_back(0);
            while (heap_data.size() % 8) heap_data.push_back(0);
        }
    }
    size_t bytes() const { return kHeaderBytes + kHeapHdrBytes + heap_data.size() + kBtreeBytes + kSnodBytes; }
    void place(uint64_t base) {
        header = base;
        heap = header + kHeaderBytes;
        btree = heap + kHeapHdrBytes + heap_data.size();
        snod = btree + kBtreeBytes;
    }
    void emit(Out& o) const {
        if (entries.size() > 2 * kLeafK) throw std::runtime_error("too many entries for one symbol-table node");
        std::vector<Message> m{{0x0011, 0, symtab_msg(btree, heap)}};
        emit_header(o, m);
        // local heap
        o.raw("HEAP", 4);
        o.u8(0);
        o.zeros(3);
        o.u64(heap_data.size());
        o.u64(kHeapFreeNull);
        o.u64(heap + kHeapHdrBytes);
        o.raw(heap_data.data(), heap_data.size());
        // B-tree (type 0, one leaf pointing at one SNOD)
        size_t b0 = o.size();
        o.raw("TREE", 4);
        o.u8(0);
        o.u8(0);
        o.u16(1);
        o.u64(kUndef);
        o.u64(kUndef);
        o.u64(0);                  // key 0: ""
        o.u64(snod);               // child 0
        o.u64(name_off.back());    // key 1: last name in the child
        o.zeros(kBtreeBytes - (o.size() - b0));
        // symbol table node
        size_t s0 = o.size();
        o.raw("SNOD", 4);
        o.u8(1);
        o.u8(0);
        o.u16(entries.size());
        for (size_t i = 0; i < entries.size(); ++i) {
            o.u64(name_off[i]);
            o.u64(entries[i].second);
            bool grp = cache_btree[i] != 0;
            o.u32(grp ? 1 : 0);
            o.u32(0);
            o.u64(grp ? cache_btree[i] : 0);
            o.u64(grp ? cache_heap[i] : 0);
        }
        o.zeros(kSnodBytes - (o.size() - s0));
    }
};

// ------------------------------------------------------------------------------------------
// reader
// ------------------------------------------------------------------------------------------
struct In {
    std::vector<uint8_t> b;
    uint64_t get(uint64_t off, int n) const {
        if (off + n > b.size()) throw std::runtime_error("signal file: read past end of file");
        uint64_t v = 0;
        for (int i = 0; i < n; ++i) v |= (uint64_t)b[off + i] << (8 * i);
        return v;
    }
    bool sig(uint64_t off, const char* s) const {
        size_t n = strlen(s);
        return off + n <= b.size() && memcmp(&b[off], s, n) == 0;
    }
};

struct ObjInfo {
    std::vector<uint64_t> dims;
    bool scalar = false;
    int dclass = -1;
    uint64_t esize = 0;
    int layout_class = -1;
    uint64_t addr = kUndef, size = 0;     // contiguous
    uint64_t btree = kUndef;              // chunked
    std::vector<uint64_t> chunk;          // chunk dims (rank) + element size
    uint64_t stab_btree = kUndef, stab_heap = kUndef;
    bool filtered = false;
};

void parse_messages(const In& in, uint64_t start, uint64_t len, ObjInfo& oi, int depth);

ObjInfo parse_object(const In& in, uint64_t addr) {
    ObjInfo oi;
    if (in.get(addr, 1) != 1)
        throw std::runtime_error("signal file: object header version not supported (only version 1)");
    uint64_t body = in.get(addr + 8, 4);
    parse_messages(in, addr + 16, body, oi, 0);
    return oi;
}

void parse_messages(const In& in, uint64_t p, uint64_t len, ObjInfo& oi, int depth) {
    if (depth > 16) throw std::runtime_error("signal file: too many header continuations");
    const uint64_t end = p + len;
    while (p + 8 <= end) {
        uint16_t type = (uint16_t)in.get(p, 2);
        uint16_t size = (uint16_t)in.get(p + 2, 2);
        uint64_t d = p + 8;
        switch (type) {
            case 0x0001: {  // dataspace
                int ver = (int)in.get(d, 1), rank = (int)in.get(d + 1, 1), flags = (int)in.get(d + 2, 1);
                uint64_t q;
                if (ver == 1) {
                    q = d + 8;
                    oi.scalar = rank == 0;
                } else {
                    int stype = (int)in.get(d + 3, 1);
                    oi.scalar = stype == 0;
                    q = d + 4;
                }
                oi.dims.clear();
                for (int i = 0; i < rank; ++i) oi.dims.push_back(in.get(q + 8 * i, 8));
                (void)flags;
                break;
            }
            case 0x0003:  // datatype
                oi.dclass = (int)(in.get(d, 1) & 0x0f);
                oi.esize = in.get(d + 4, 4);
                break;
            case 0x0008: {  // layout
                int ver = (int)in.get(d, 1);
                if (ver != 3) throw std::runtime_error("signal file: layout message version not supported");
                oi.layout_class = (int)in.get(d + 1, 1);
                if (oi.layout_class == 1) {
                    oi.addr = in.get(d + 2, 8);
                    oi.size = in.get(d + 10, 8);
                } else if (oi.layout_class == 2) {
                    int nd = (int)in.get(d + 2, 1);
                    oi.btree = in.get(d + 3, 8);
                    oi.chunk.clear();
                    for (int i = 0; i < nd; ++i) oi.chunk.push_back(in.get(d + 11 + 4 * i, 4));
                } else if (oi.layout_class == 0) {
                    throw std::runtime_error("signal file: compact datasets not supported");
                }
                break;
            }
            case 0x000B:  // filter pipeline
                oi.filtered = true;
                break;
            case 0x0010:  // continuation
                parse_messages(in, in.get(d, 8) + 0, in.get(d + 8, 8), oi, depth + 1);
                break;
            case 0x0011:  // symbol table
                oi.stab_btree = in.get(d, 8);
                oi.stab_heap = in.get(d + 8, 8);
                break;
            default:
                break;
        }
        p = d + size;
    }
}

// name -> object header address for a symbol-table group
std::map<std::string, uint64_t> list_group(const In& in, const ObjInfo& g) {
    std::map<std::string, uint64_t> out;
    if (g.stab_btree == kUndef) throw std::runtime_error("signal file: not a group");
    if (!in.sig(g.stab_heap, "HEAP")) throw std::runtime_error("signal file: bad local heap");
    uint64_t heap_data = in.get(g.stab_heap + 24, 8);
    std::function<void(uint64_t, int)> walk = [&](uint64_t node, int guard) {
        if (guard > 64) throw std::runtime_error("signal file: group B-tree too deep");
        if (!in.sig(node, "TREE")) throw std::runtime_error("signal file: bad group B-tree node");
        int level = (int)in.get(node + 5, 1), used = (int)in.get(node + 6, 2);
        for (int i = 0; i < used; ++i) {
            uint64_t child = in.get(node + 24 + 8 + 16 * i, 8);
            if (level > 0) {
                walk(child, guard + 1);
            } else {
                if (!in.sig(child, "SNOD")) throw std::runtime_error("signal file: bad symbol-table node");
                int n = (int)in.get(child + 6, 2);
                for (int e = 0; e < n; ++e) {
                    uint64_t ent = child + 8 + 40 * e;
                    uint64_t noff = in.get(ent, 8), hdr = in.get(ent + 8, 8);
                    std::string name;
                    for (uint64_t k = heap_data + noff; k < in.b.size() && in.b[k]; ++k) name.push_back((char)in.b[k]);
                    out[name] = hdr;
                }
            }
        }
    };
    walk(g.stab_btree, 0);
    return out;
}

// Read a whole dataset as raw bytes (row-major, element size esize).
std::vector<uint8_t> read_dataset(const In& in, const ObjInfo& oi) {
    if (oi.filtered) throw std::runtime_error("signal file: filtered (compressed) datasets not supported");
    uint64_t n = oi.esize;
    for (uint64_t d : oi.dims) n *= d;
    std::vector<uint8_t> out(n, 0);
    if (n == 0) return out;
    if (oi.layout_class == 1) {
        if (oi.addr == kUndef) return out;
        if (oi.addr + n > in.b.size()) throw std::runtime_error("signal file: dataset past end of file");
        memcpy(out.data(), &in.b[oi.addr], n);
        return out;
    }
    if (oi.layout_class != 2) throw std::runtime_error("signal file: unknown dataset layout");
    const size_t rank = oi.dims.size();
    if (oi.chunk.size() != rank + 1) throw std::runtime_error("signal file: bad chunk dimensions");
    std::vector<uint64_t> cd(oi.chunk.begin(), oi.chunk.begin() + rank);
    uint64_t chunk_elems = 1;
    for (uint64_t c : cd) chunk_elems *= c;
    const uint64_t es = oi.esize;
    const uint64_t key_bytes = 8 + 8 * (rank + 1);
    std::function<void(uint64_t, int)> walk = [&](uint64_t node, int guard) {
        if (guard > 64) throw std::runtime_error("signal file: chunk B-tree too deep");
        if (!in.sig(node, "TREE")) throw std::runtime_error("signal file: bad chunk B-tree node");
        int level = (int)in.get(node + 5, 1), used = (int)in.get(node + 6, 2);
        for (int i = 0; i < used; ++i) {
            uint64_t key = node + 24 + i * (key_bytes + 8);
            uint64_t child = in.get(key + key_bytes, 8);
            if (level > 0) {
                walk(child, guard + 1);
                continue;
            }
            uint64_t csize = in.get(key, 4);
            std::vector<uint64_t> off(rank);
            for (size_t k = 0; k < rank; ++k) off[k] = in.get(key + 8 + 8 * k, 8);
            if (csize < chunk_elems * es || child + chunk_elems * es > in.b.size())
                throw std::runtime_error("signal file: bad chunk");
            // copy the chunk into the dataset, clipped at the dataset's extent
            std::vector<uint64_t> idx(rank, 0);
            for (uint64_t e = 0; e < chunk_elems; ++e) {
                uint64_t r = e;
                bool inside = true;
                uint64_t lin = 0;
                for (size_t k = rank; k-- > 0;) {
                    idx[k] = r % cd[k];
                    r /= cd[k];
                }
                for (size_t k = 0; k < rank; ++k) {
                    uint64_t g = off[k] + idx[k];
                    if (g >= oi.dims[k]) {
                        inside = false;
                        break;
                    }
                    lin = lin * oi.dims[k] + g;
                }
                if (inside) memcpy(&out[lin * es], &in.b[child + e * es], es);
            }
        }
    };
    if (oi.btree != kUndef) walk(oi.btree, 0);
    return out;
}

}  // namespace

void write_signal_file(const std::string& path, const SignalData& d) {
    const size_t nq = d.nq();
    std::vector<double> q(nq * 3);
    for (size_t i = 0; i < nq; ++i)
        for (int k = 0; k < 3; ++k) q[3 * i + k] = d.qvectors[i][k];
    if (d.has_fqt && d.fqt.size() != nq * d.nf * 2) throw std::runtime_error("fqt has the wrong size");
    std::vector<DatasetSpec> root_ds;
    auto f64 = [&](const char* name, const std::vector<double>& v, std::vector<uint64_t> dims,
                   std::vector<uint64_t> chunk) {
        DatasetSpec ds{name, F64, dims, reinterpret_cast<const uint8_t*>(v.data()), v.size() * 8};
        ds.chunk = chunk;
        root_ds.push_back(ds);
    };
    // chunk shapes and unlimited first dimension as the reference's writer creates them
    // (file_writer_service.cpp:68-159): rows of `chunksize`; fqt splits the chunk between
    // rows and frames when NF < chunksize
    const uint64_t cs = std::max<size_t>(d.chunksize, 1);
    const uint64_t c2 = (d.nf > 0 && d.nf < cs) ? d.nf : cs, c1 = std::max<uint64_t>(cs / c2, 1);
    f64("qvectors", q, {nq, 3}, {cs, 3});
    if (d.has_fqt) f64("fqt", d.fqt, {nq, d.nf, 2}, {c1, c2, 2});
    if (d.has_fq0) f64("fq0", d.fq0, {nq, 2}, {cs, 2});
    if (d.has_fq) f64("fq", d.fq, {nq, 2}, {cs, 2});
    if (d.has_fq2) f64("fq2", d.fq2, {nq, 2}, {cs, 2});
    std::string cfg = d.config + '\0', db = d.database + '\0';
    std::vector<DatasetSpec> meta_ds = {
        {"config", STR, {}, reinterpret_cast<const uint8_t*>(cfg.data()), cfg.size()},
        {"database", STR, {}, reinterpret_cast<const uint8_t*>(db.data()), db.size()},
        {"rawconfig", I8, {d.rawconfig.size()}, reinterpret_cast<const uint8_t*>(d.rawconfig.data()),
         d.rawconfig.size()},
    };
    auto by_name = [](const DatasetSpec& a, const DatasetSpec& b) { return a.name < b.name; };
    std::sort(root_ds.begin(), root_ds.end(), by_name);
    std::sort(meta_ds.begin(), meta_ds.end(), by_name);

    // ---- address assignment ---------------------------------------------------------------
    GroupLayout root, meta;
    std::vector<std::string> root_names;
    for (auto& s : root_ds) root_names.push_back(s.name);
    root_names.push_back("meta");
    std::sort(root_names.begin(), root_names.end());
    root.names(root_names);
    std::vector<std::string> meta_names;
    for (auto& s : meta_ds) meta_names.push_back(s.name);
    meta.names(meta_names);

    uint64_t pos = 96;  // superblock
    root.place(pos);
    pos += root.bytes();
    meta.place(pos);
    pos += meta.bytes();
    auto ds_messages = [](const DatasetSpec& s) {
        std::vector<Message> m;
        m.push_back({0x0001, 0, dataspace_msg(s.dims, !s.chunk.empty())});
        m.push_back({0x0003, 1, datatype_msg(s.kind, s.nbytes)});
        m.push_back({0x0005, 1, fill_msg(s.kind)});
        if (s.chunk.empty()) m.push_back({0x0008, 0, layout_msg(s.data_addr, s.nbytes)});
        else m.push_back({0x0008, 0, chunked_layout_msg(s.btree_addr, s.chunk, 8)});
        return m;
    };
    std::vector<DatasetSpec*> all;
    for (auto& s : root_ds) all.push_back(&s);
    for (auto& s : meta_ds) all.push_back(&s);
    for (DatasetSpec* s : all) {
        s->header_addr = pos;
        pos += header_size(ds_messages(*s));
    }
    for (DatasetSpec* s : all) {
        pos = (pos + 7) & ~(uint64_t)7;
        if (!s->chunk.empty()) {
            s->chunk_region = chunked_region(*s, pos, s->btree_addr);
            s->data_addr = s->chunk_region.empty() ? kUndef : pos;
            pos += s->chunk_region.size();
            continue;
        }
        s->data_addr = s->nbytes ? pos : kUndef;
        pos += s->nbytes;
    }
    const uint64_t eof = pos;

    for (const std::string& n : root_names) {
        if (n == "meta") {
            root.entries.emplace_back(n, meta.header);
            root.cache_btree.push_back(meta.btree);
            root.cache_heap.push_back(meta.heap);
        } else {
            for (auto& s : root_ds)
                if (s.name == n) root.entries.emplace_back(n, s.header_addr);
            root.cache_btree.push_back(0);
            root.cache_heap.push_back(0);
        }
    }
    for (auto& s : meta_ds) {
        meta.entries.emplace_back(s.name, s.header_addr);
        meta.cache_btree.push_back(0);
        meta.cache_heap.push_back(0);
    }

    // ---- serialisation ----------------------------------------------------------------------
    Out o;
    o.raw(kSignature, 8);
    o.u8(0);  // superblock version
    o.u8(0);  // free-space version
    o.u8(0);  // root group symbol table entry version
    o.u8(0);
    o.u8(0);  // shared header message format version
    o.u8(8);  // size of offsets
    o.u8(8);  // size of lengths
    o.u8(0);
    o.u16(kLeafK);
    o.u16(kInternalK);
    o.u32(0);        // file consistency flags
    o.u64(0);        // base address
    o.u64(kUndef);   // free-space info
    o.u64(eof);      // end of file address
    o.u64(kUndef);   // driver information block
    o.u64(0);        // root entry: link name offset
    o.u64(root.header);
    o.u32(1);        // cache type: group
    o.u32(0);
    o.u64(root.btree);
    o.u64(root.heap);
    if (o.size() != 96) throw std::logic_error("superblock size");
    root.emit(o);
    meta.emit(o);
    for (DatasetSpec* s : all) {
        if (o.size() != s->header_addr) throw std::logic_error("object header placement");
        emit_header(o, ds_messages(*s));
    }
    for (DatasetSpec* s : all) {
        o.pad8();
        if (!s->chunk.empty()) {
            if (!s->chunk_region.empty() && o.size() != s->data_addr) throw std::logic_error("chunk placement");
            o.raw(s->chunk_region.data(), s->chunk_region.size());
            continue;
        }
        if (s->nbytes && o.size() != s->data_addr) throw std::logic_error("data placement");
        o.raw(s->data, s->nbytes);
    }
    if (o.size() != eof) throw std::logic_error("end of file address");

    std::string tmp = path + ".tmp";
    {
        std::ofstream f(tmp, std::ios::binary | std::ios::trunc);
        if (!f) throw std::runtime_error("cannot write " + tmp);
        f.write(reinterpret_cast<const char*>(o.b.data()), (std::streamsize)o.b.size());
        if (!f) throw std::runtime_error("write failed: " + tmp);
    }
    if (std::rename(tmp.c_str(), path.c_str()) != 0) throw std::runtime_error("cannot replace " + path);
}

bool is_hdf5_file(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    uint8_t sig[8];
    for (uint64_t off = 0; f; off = off ? off * 2 : 512) {
        f.seekg((std::streamoff)off);
        f.read(reinterpret_cast<char*>(sig), 8);
        if (!f) return false;
        if (memcmp(sig, kSignature, 8) == 0) return true;
        if (off > (1ull << 30)) return false;
    }
    return false;
}

SignalData read_signal_file(const std::string& path) {
    In in;
    {
        std::ifstream f(path, std::ios::binary);
        if (!f) throw std::runtime_error("cannot open " + path);
        f.seekg(0, std::ios::end);
        in.b.resize((size_t)f.tellg());
        f.seekg(0);
        f.read(reinterpret_cast<char*>(in.b.data()), (std::streamsize)in.b.size());
    }
    uint64_t base = kUndef;
    for (uint64_t off = 0; off + 8 <= in.b.size(); off = off ? off * 2 : 512)
        if (memcmp(&in.b[off], kSignature, 8) == 0) {
            base = off;
            break;
        }
    if (base == kUndef) throw std::runtime_error(path + " does not to be a HDF5 data file. aborting...");
    int sbver = (int)in.get(base + 8, 1);
    if (sbver > 1) throw std::runtime_error("signal file: superblock version " + std::to_string(sbver) + " not supported");
    if (in.get(base + 13, 1) != 8 || in.get(base + 14, 1) != 8)
        throw std::runtime_error("signal file: only 8-byte offsets and lengths are supported");
    uint64_t entry = base + 24 + (sbver == 1 ? 4 : 0) + 32;
    uint64_t root_hdr = in.get(entry + 8, 8);
    if (base != 0) throw std::runtime_error("signal file: user blocks are not supported");
    ObjInfo root = parse_object(in, root_hdr);
    auto names = list_group(in, root);

    SignalData d;
    auto read_f64 = [&](const std::string& name, std::vector<uint64_t>& dims) -> std::vector<double> {
        ObjInfo oi = parse_object(in, names.at(name));
        if (oi.dclass != 1 || oi.esize != 8) throw std::runtime_error("signal file: " + name + " is not float64");
        dims = oi.dims;
        std::vector<uint8_t> raw = read_dataset(in, oi);
        std::vector<double> v(raw.size() / 8);
        memcpy(v.data(), raw.data(), raw.size());
        return v;
    };
    std::vector<uint64_t> dims;
    if (!names.count("qvectors")) throw std::runtime_error("signal file: no /qvectors");
    std::vector<double> q = read_f64("qvectors", dims);
    if (dims.size() != 2 || dims[1] != 3) throw std::runtime_error("signal file: bad /qvectors shape");
    for (uint64_t i = 0; i < dims[0]; ++i) d.qvectors.push_back(Vec3{q[3 * i], q[3 * i + 1], q[3 * i + 2]});
    const size_t nq = d.qvectors.size();
    d.has_fqt = names.count("fqt") > 0;
    if (d.has_fqt) {
        d.fqt = read_f64("fqt", dims);
        if (dims.size() != 3 || dims[0] != nq || dims[2] != 2) throw std::runtime_error("signal file: bad /fqt shape");
        d.nf = dims[1];
    }
    auto two = [&](const char* name, bool& has, std::vector<double>& v) {
        has = names.count(name) > 0;
        if (!has) return;
        v = read_f64(name, dims);
        if (dims.size() != 2 || dims[0] != nq || dims[1] != 2)
            throw std::runtime_error(std::string("signal file: bad /") + name + " shape");
    };
    two("fq0", d.has_fq0, d.fq0);
    two("fq", d.has_fq, d.fq);
    two("fq2", d.has_fq2, d.fq2);
    if (names.count("meta")) {
        ObjInfo mg = parse_object(in, names.at("meta"));
        auto mnames = list_group(in, mg);
        auto text = [&](const char* name) -> std::string {
            if (!mnames.count(name)) return "";
            ObjInfo oi = parse_object(in, mnames.at(name));
            std::vector<uint8_t> raw = read_dataset(in, oi);
            std::string s(raw.begin(), raw.end());
            size_t z = s.find('\0');
            if (z != std::string::npos && oi.dclass == 3) s.resize(z);
            return s;
        };
        d.rawconfig = text("rawconfig");
        d.config = text("config");
        d.database = text("database");
    }
    return d;
}

}  // namespace sassgpu
