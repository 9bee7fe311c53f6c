// h5lite.cc -- reader and writer for the HDF5 subset described in h5lite.h.
#include "h5lite.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>

#include <zlib.h>

namespace h5lite {

namespace {

constexpr uint64_t UNDEF = ~(uint64_t) 0;

struct Buf {
    std::vector<uint8_t> b;
    bool in(uint64_t off, uint64_t n) const { return off <= b.size() && n <= b.size() - off; }
    uint64_t u(uint64_t off, int n) const
    {
        uint64_t v = 0;
        for (int i = 0; i < n; i++)
            v |= (uint64_t) b[off + i] << (8 * i);
        return v;
    }
};

struct Msg {
    int type;
    uint64_t off, size;
};

bool header_messages(const Buf &f, uint64_t addr, std::vector<Msg> &msgs, std::string &err)
{
    if (!f.in(addr, 16) || f.b[addr] != 1) {
        err = "only version-1 object headers are supported";
        return false;
    }
    const int nmsg = (int) f.u(addr + 2, 2);
    const uint64_t hsize = f.u(addr + 8, 4);
    std::vector<std::pair<uint64_t, uint64_t>> blocks{{addr + 16, hsize}};
    for (size_t bi = 0; bi < blocks.size() && (int) msgs.size() < nmsg; bi++) {
        uint64_t p = blocks[bi].first;
        const uint64_t end = p + blocks[bi].second;
        while (p + 8 <= end && (int) msgs.size() < nmsg) {
            if (!f.in(p, 8)) {
                err = "truncated object header";
                return false;
            }
            const int t = (int) f.u(p, 2);
            const uint64_t sz = f.u(p + 2, 2);
            if (!f.in(p + 8, sz)) {
                err = "truncated header message";
                return false;
            }
            if (t == 0x10) {  // continuation: address, length
                if (sz < 16) {
                    err = "truncated continuation message";
                    return false;
                }
                blocks.push_back({f.u(p + 8, 8), f.u(p + 16, 8)});
            }
            msgs.push_back({t, p + 8, sz});
            p += 8 + sz;
        }
    }
    return true;
}

bool group_entries(const Buf &f, uint64_t btree, std::vector<std::pair<uint64_t, uint64_t>> &out,
                   std::string &err, int depth = 0)
{
    if (depth > 16 || !f.in(btree, 24) || memcmp(&f.b[btree], "TREE", 4) != 0) {
        err = "bad group B-tree";
        return false;
    }
    const int level = f.b[btree + 5];
    const int used = (int) f.u(btree + 6, 2);
    uint64_t p = btree + 24 + 8;  // first key
    for (int i = 0; i < used; i++) {
        if (!f.in(p, 16)) {
            err = "truncated B-tree";
            return false;
        }
        const uint64_t child = f.u(p, 8);
        p += 16;
        if (level > 0) {
            if (!group_entries(f, child, out, err, depth + 1))
                return false;
            continue;
        }
        if (!f.in(child, 8) || memcmp(&f.b[child], "SNOD", 4) != 0) {
            err = "bad symbol table node";
            return false;
        }
        const int n = (int) f.u(child + 6, 2);
        for (int e = 0; e < n; e++) {
            const uint64_t ent = child + 8 + 40 * (uint64_t) e;
            if (!f.in(ent, 40)) {
                err = "truncated symbol table node";
                return false;
            }
            out.push_back({f.u(ent, 8), f.u(ent + 8, 8)});
        }
    }
    return true;
}

// Filters of a chunked dataset's pipeline (message 0x0B), in order.
bool filter_pipeline(const Buf &f, const Msg &m, std::vector<int> &ids, std::string &err)
{
    if (!f.in(m.off, 8) || m.size < 8) {
        err = "truncated filter pipeline message";
        return false;
    }
    const int ver = f.b[m.off], nf = f.b[m.off + 1];
    uint64_t p = m.off + (ver == 1 ? 8 : 2);
    const uint64_t end = m.off + m.size;
    for (int i = 0; i < nf; i++) {
        if (p + 2 > end) {
            err = "truncated filter description";
            return false;
        }
        const int id = (int) f.u(p, 2);
        uint64_t name_len = 0;
        if (ver == 1 || id >= 256) {
            if (p + 4 > end) {
                err = "truncated filter description";
                return false;
            }
            name_len = f.u(p + 2, 2);
            p += 4;
        } else {
            p += 2;
        }
        if (p + 4 > end) {
            err = "truncated filter description";
            return false;
        }
        const uint64_t nval = f.u(p + 2, 2);
        p += 4;
        if (ver == 1)
            name_len = (name_len + 7) & ~(uint64_t) 7;
        p += name_len + 4 * nval;
        if (ver == 1 && (nval & 1))
            p += 4;
        if (p > end) {
            err = "truncated filter description";
            return false;
        }
        ids.push_back(id);
    }
    return true;
}

// Undo the byte shuffle of `n` elements of `size` bytes.
void unshuffle(std::vector<uint8_t> &v, int size)
{
    const size_t n = v.size() / (size_t) size;
    std::vector<uint8_t> out(v.size());
    for (size_t i = 0; i < n; i++)
        for (int b = 0; b < size; b++)
            out[i * size + b] = v[(size_t) b * n + i];
    v.swap(out);
}

struct ChunkInfo {
    int nd;                   // dataset rank
    std::vector<uint64_t> cd; // chunk dims
    std::vector<int> filters;
    int elem;
};

// Walk a version-1 B-tree of chunks (node type 1) and copy every chunk's
// elements into `dst` (row-major, dims `dims`).
bool read_chunks(const Buf &f, uint64_t addr, const ChunkInfo &ci, const std::vector<uint64_t> &dims,
                 uint8_t *dst, std::string &err, int depth = 0)
{
    if (depth > 32 || !f.in(addr, 24) || memcmp(&f.b[addr], "TREE", 4) != 0 || f.b[addr + 4] != 1) {
        err = "bad chunk B-tree";
        return false;
    }
    const int level = f.b[addr + 5];
    const int used = (int) f.u(addr + 6, 2);
    const int nd = ci.nd;
    const uint64_t ks = 8 + 8 * (uint64_t) (nd + 1);  // size, filter mask, nd + 1 offsets
    uint64_t p = addr + 24;
    uint64_t chunk_elems = 1;
    for (int d = 0; d < nd; d++)
        chunk_elems *= ci.cd[d];
    const uint64_t chunk_bytes = chunk_elems * (uint64_t) ci.elem;
    for (int i = 0; i < used; i++) {
        if (!f.in(p, ks + 8)) {
            err = "truncated chunk B-tree";
            return false;
        }
        const uint64_t csz = f.u(p, 4);
        const uint32_t mask = (uint32_t) f.u(p + 4, 4);
        std::vector<uint64_t> off(nd);
        for (int d = 0; d < nd; d++)
            off[d] = f.u(p + 8 + 8 * (uint64_t) d, 8);
        const uint64_t child = f.u(p + ks, 8);
        p += ks + 8;
        if (level > 0) {
            if (!read_chunks(f, child, ci, dims, dst, err, depth + 1))
                return false;
            continue;
        }
        if (!f.in(child, csz)) {
            err = "chunk extends past the end of the file";
            return false;
        }
        std::vector<uint8_t> raw(f.b.begin() + child, f.b.begin() + child + csz);
        // filters are undone in reverse order; a set mask bit skips that filter
        for (int j = (int) ci.filters.size() - 1; j >= 0; j--) {
            if (mask & (1u << j))
                continue;
            if (ci.filters[j] == 1) {
                std::vector<uint8_t> out(chunk_bytes);
                uLongf n = (uLongf) chunk_bytes;
                if (uncompress(out.data(), &n, raw.data(), (uLong) raw.size()) != Z_OK ||
                    n != chunk_bytes) {
                    err = "deflate chunk does not inflate to its size";
                    return false;
                }
                raw.swap(out);
            } else if (ci.filters[j] == 2) {
                unshuffle(raw, ci.elem);
            } else {
                err = "unsupported filter " + std::to_string(ci.filters[j]);
                return false;
            }
        }
        if (raw.size() != chunk_bytes) {
            err = "chunk has the wrong size";
            return false;
        }
        // copy the part of the chunk inside the dataset, row by row of the last dimension
        std::vector<uint64_t> idx(nd, 0);
        const uint64_t last = ci.cd[nd - 1];
        for (uint64_t r = 0; r < chunk_elems / last; r++) {
            uint64_t rem = r;
            bool inside = true;
            uint64_t at = 0;
            for (int d = nd - 2; d >= 0; d--) {
                idx[d] = rem % ci.cd[d];
                rem /= ci.cd[d];
            }
            for (int d = 0; d < nd - 1; d++) {
                const uint64_t g = off[d] + idx[d];
                if (g >= dims[d])
                    inside = false;
                at = at * dims[d] + g;
            }
            if (!inside || off[nd - 1] >= dims[nd - 1])
                continue;
            const uint64_t n = std::min<uint64_t>(last, dims[nd - 1] - off[nd - 1]);
            at = at * dims[nd - 1] + off[nd - 1];
            memcpy(dst + at * ci.elem, raw.data() + r * last * ci.elem, n * ci.elem);
        }
    }
    return true;
}

}  // namespace

bool read_file(const std::string &path, std::map<std::string, Dataset> &out, std::string &err)
{
    Buf f;
    {
        std::ifstream in(path, std::ios::binary);
        if (!in) {
            err = "cannot open " + path;
            return false;
        }
        f.b.assign(std::istreambuf_iterator<char>(in), std::istreambuf_iterator<char>());
    }
    static const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    if (!f.in(0, 96) || memcmp(f.b.data(), sig, 8) != 0) {
        err = path + " is not an HDF5 file";
        return false;
    }
    if (f.b[8] != 0 || f.b[13] != 8 || f.b[14] != 8) {
        err = "only superblock version 0 with 8-byte offsets is supported";
        return false;
    }
    const uint64_t root = f.u(56 + 8, 8);
    std::vector<Msg> msgs;
    if (!header_messages(f, root, msgs, err))
        return false;
    uint64_t btree = UNDEF, heap = UNDEF;
    for (const Msg &m : msgs)
        if (m.type == 0x11 && m.size >= 16) {
            btree = f.u(m.off, 8);
            heap = f.u(m.off + 8, 8);
        }
    if (btree == UNDEF || !f.in(heap, 32) || memcmp(&f.b[heap], "HEAP", 4) != 0) {
        err = "root group has no symbol table";
        return false;
    }
    const uint64_t heap_size = f.u(heap + 8, 8), heap_data = f.u(heap + 24, 8);
    std::vector<std::pair<uint64_t, uint64_t>> ents;
    if (!group_entries(f, btree, ents, err))
        return false;
    for (auto &e : ents) {
        if (e.first >= heap_size || !f.in(heap_data + e.first, 1))
            continue;
        const char *nm = (const char *) &f.b[heap_data + e.first];
        const uint64_t room = std::min<uint64_t>(heap_size - e.first, f.b.size() - (heap_data + e.first));
        const size_t nlen = strnlen(nm, (size_t) room);
        if (nlen == room)
            continue;  // unterminated name
        std::string name(nm, nlen);
        std::vector<Msg> dm;
        if (!header_messages(f, e.second, dm, err))
            return false;
        Dataset ds;
        int cls = -1, size = 0, layout = -1;
        bool is_signed = true, have_space = false;
        uint64_t data_addr = UNDEF, data_size = 0;
        ChunkInfo ci{};
        const Msg *pipeline = nullptr;
        for (const Msg &m : dm) {
            if (m.type == 0x1) {
                if (m.size < 8) {
                    err = "truncated dataspace of " + name;
                    return false;
                }
                const int ver = f.b[m.off], nd = f.b[m.off + 1];
                const uint64_t d0 = m.off + (ver == 1 ? 8 : 4);
                if (d0 + 8 * (uint64_t) nd > m.off + m.size || !f.in(d0, 8 * (uint64_t) nd)) {
                    err = "truncated dataspace of " + name;
                    return false;
                }
                for (int i = 0; i < nd; i++)
                    ds.dims.push_back(f.u(d0 + 8 * (uint64_t) i, 8));
                have_space = true;
            } else if (m.type == 0x3) {
                if (m.size < 8) {
                    err = "truncated datatype of " + name;
                    return false;
                }
                cls = f.b[m.off] & 0x0f;
                size = (int) f.u(m.off + 4, 4);
                if (cls == 0)
                    is_signed = (f.b[m.off + 1] & 0x08) != 0;
                if ((f.b[m.off + 1] & 0x01) != 0) {
                    err = "big-endian datasets are not supported (" + name + ")";
                    return false;
                }
            } else if (m.type == 0xB) {
                pipeline = &m;
            } else if (m.type == 0x8) {
                if (m.size < 2 || f.b[m.off] != 3)
                    continue;  // only layout message version 3
                layout = f.b[m.off + 1];
                if (layout == 1 && m.size >= 18) {  // contiguous: address, size
                    data_addr = f.u(m.off + 2, 8);
                    data_size = f.u(m.off + 10, 8);
                } else if (layout == 0 && m.size >= 4) {  // compact: size, raw data
                    data_size = f.u(m.off + 2, 2);
                    if (4 + data_size > m.size) {
                        err = "truncated compact data of " + name;
                        return false;
                    }
                    data_addr = m.off + 4;
                } else if (layout == 2 && m.size >= 3) {  // chunked: rank + 1, B-tree, dims
                    const int cnd = f.b[m.off + 2];
                    if (cnd < 2 || 11 + 4 * (uint64_t) cnd > m.size) {
                        err = "truncated chunked layout of " + name;
                        return false;
                    }
                    data_addr = f.u(m.off + 3, 8);
                    ci.nd = cnd - 1;
                    for (int i = 0; i < cnd; i++)
                        ci.cd.push_back(f.u(m.off + 11 + 4 * (uint64_t) i, 4));
                    ci.elem = (int) ci.cd.back();
                    ci.cd.pop_back();
                } else {
                    layout = -1;
                }
            }
        }
        if (!have_space || layout < 0 || cls < 0)
            continue;  // groups, external or virtual layouts are not read
        if (!(cls == 1 && (size == 8 || size == 4)) && !(cls == 0 && (size == 4 || size == 8)))
            continue;
        uint64_t count = 1;
        for (uint64_t d : ds.dims)
            count *= d;
        std::vector<uint8_t> chunked;
        if (layout == 2) {
            if ((size_t) ci.nd != ds.dims.size() || ci.elem != size) {
                err = "chunk shape of " + name + " does not match its dataspace";
                return false;
            }
            for (uint64_t c : ci.cd)
                if (c == 0) {
                    err = "zero chunk dimension in " + name;
                    return false;
                }
            if (pipeline && !filter_pipeline(f, *pipeline, ci.filters, err))
                return false;
            chunked.assign(count * (uint64_t) size, 0);  // unwritten chunks read as 0
            if (data_addr != UNDEF && count &&
                !read_chunks(f, data_addr, ci, ds.dims, chunked.data(), err)) {
                err += " (" + name + ")";
                return false;
            }
        } else if (data_addr == UNDEF) {
            count = 0;  // never written: empty
        } else if (!f.in(data_addr, count * (uint64_t) size) || data_size < count * (uint64_t) size) {
            err = "dataset " + name + " extends past the end of the file";
            return false;
        }
        const uint8_t *src = !count ? nullptr : (layout == 2 ? chunked.data() : &f.b[data_addr]);
        if (cls == 1 && (size == 8 || size == 4)) {
            ds.f64.resize(count);
            for (uint64_t i = 0; i < count; i++) {
                if (size == 8) {
                    double v;
                    memcpy(&v, src + 8 * i, 8);
                    ds.f64[i] = v;
                } else {
                    float v;
                    memcpy(&v, src + 4 * i, 4);
                    ds.f64[i] = v;
                }
            }
        } else if (cls == 0 && (size == 4 || size == 8)) {
            ds.is_int = true;
            ds.i64.resize(count);
            for (uint64_t i = 0; i < count; i++) {
                if (size == 4) {
                    int32_t v;
                    memcpy(&v, src + 4 * i, 4);
                    ds.i64[i] = is_signed ? v : (int64_t) (uint32_t) v;
                } else {
                    int64_t v;
                    memcpy(&v, src + 8 * i, 8);
                    ds.i64[i] = v;
                }
            }
        } else {
            continue;
        }
        out[name] = std::move(ds);
    }
    return true;
}

// ---------------------------------------------------------------------------
// writer
// ---------------------------------------------------------------------------
void Writer::add_f64(const std::string &name, const std::vector<uint64_t> &dims,
                     const double *data)
{
    Item it{name, dims, false, {}};
    uint64_t n = 1;
    for (uint64_t d : dims)
        n *= d;
    it.bytes.resize(n * 8);
    if (n)
        memcpy(it.bytes.data(), data, n * 8);
    items_.push_back(std::move(it));
}

void Writer::add_i32(const std::string &name, const std::vector<uint64_t> &dims,
                     const int32_t *data)
{
    Item it{name, dims, true, {}};
    uint64_t n = 1;
    for (uint64_t d : dims)
        n *= d;
    it.bytes.resize(n * 4);
    if (n)
        memcpy(it.bytes.data(), data, n * 4);
    items_.push_back(std::move(it));
}

namespace {

struct Out {
    std::vector<uint8_t> b;
    void put(uint64_t v, int n)
    {
        for (int i = 0; i < n; i++)
            b.push_back((uint8_t) (v >> (8 * i)));
    }
    void set(uint64_t off, uint64_t v, int n)
    {
        for (int i = 0; i < n; i++)
            b[off + i] = (uint8_t) (v >> (8 * i));
    }
    void bytes(const void *p, size_t n)
    {
        const uint8_t *q = (const uint8_t *) p;
        b.insert(b.end(), q, q + n);
    }
    void pad8()
    {
        while (b.size() % 8)
            b.push_back(0);
    }
};

// one header message: type, size (padded to 8), flags, body
void message(Out &o, int type, const std::vector<uint8_t> &body, int flags = 0)
{
    size_t sz = (body.size() + 7) & ~(size_t) 7;
    o.put(type, 2);
    o.put(sz, 2);
    o.put(flags, 1);
    o.put(0, 3);
    o.bytes(body.data(), body.size());
    for (size_t i = body.size(); i < sz; i++)
        o.b.push_back(0);
}

}  // namespace

bool Writer::write(const std::string &path, std::string &err) const
{
    constexpr int LEAF_K = 32, INTERNAL_K = 16;  // one symbol node holds 2*LEAF_K entries
    if (items_.size() > (size_t) 2 * LEAF_K) {
        err = "too many datasets for one symbol table node";
        return false;
    }
    std::vector<const Item *> sorted;
    for (const Item &it : items_)
        sorted.push_back(&it);
    std::sort(sorted.begin(), sorted.end(),
              [](const Item *a, const Item *b) { return a->name < b->name; });

    Out o;
    // --- superblock (version 0), root symbol table entry patched later
    static const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    o.bytes(sig, 8);
    o.put(0, 1);  // superblock version
    o.put(0, 1);  // free-space version
    o.put(0, 1);  // root group symbol table entry version
    o.put(0, 1);
    o.put(0, 1);  // shared header message version
    o.put(8, 1);  // size of offsets
    o.put(8, 1);  // size of lengths
    o.put(0, 1);
    o.put(LEAF_K, 2);
    o.put(INTERNAL_K, 2);
    o.put(0, 4);      // consistency flags
    o.put(0, 8);      // base address
    o.put(UNDEF, 8);  // free-space info
    const uint64_t eof_at = o.b.size();
    o.put(0, 8);      // end of file address
    o.put(UNDEF, 8);  // driver info
    const uint64_t root_ste = o.b.size();
    o.put(0, 8);   // link name offset
    o.put(0, 8);   // object header address (patched)
    o.put(1, 4);   // cache type 1: scratch holds B-tree and heap addresses
    o.put(0, 4);
    o.put(0, 8);   // B-tree address (patched)
    o.put(0, 8);   // heap address (patched)

    // --- local heap: "" at offset 0, then the names
    std::vector<uint64_t> name_off;
    std::vector<uint8_t> heap_data(8, 0);
    for (const Item *it : sorted) {
        name_off.push_back(heap_data.size());
        heap_data.insert(heap_data.end(), it->name.begin(), it->name.end());
        heap_data.push_back(0);
        while (heap_data.size() % 8)
            heap_data.push_back(0);
    }
    o.pad8();
    const uint64_t heap_addr = o.b.size();
    o.bytes("HEAP", 4);
    o.put(0, 1);
    o.put(0, 3);
    o.put(heap_data.size(), 8);
    o.put(UNDEF, 8);  // no free list
    const uint64_t heap_data_addr = o.b.size() + 8;
    o.put(heap_data_addr, 8);
    o.bytes(heap_data.data(), heap_data.size());

    // --- dataset object headers and data
    std::vector<uint64_t> obj_addr;
    for (const Item *it : sorted) {
        o.pad8();
        const uint64_t hdr = o.b.size();
        obj_addr.push_back(hdr);
        Out m;
        // dataspace, version 1
        std::vector<uint8_t> ds{1, (uint8_t) it->dims.size(), 0, 0, 0, 0, 0, 0};
        for (uint64_t d : it->dims)
            for (int i = 0; i < 8; i++)
                ds.push_back((uint8_t) (d >> (8 * i)));
        message(m, 0x1, ds, 1);
        // datatype
        std::vector<uint8_t> dt;
        if (it->is_int) {
            dt = {0x10, 0x08, 0, 0, 4, 0, 0, 0, 0, 0, 32, 0};
        } else {
            dt = {0x11, 0x20, 0x3f, 0, 8, 0, 0, 0, 0, 0, 64, 0, 52, 11, 0, 52, 0xff, 0x03, 0, 0};
        }
        message(m, 0x3, dt, 1);
        // fill value, version 2: allocation late, write if set, undefined
        message(m, 0x5, {2, 2, 2, 0}, 1);
        // layout, version 3, contiguous (address patched below)
        std::vector<uint8_t> lay(18, 0);
        lay[0] = 3;
        lay[1] = 1;
        const uint64_t layout_body = m.b.size() + 8;
        message(m, 0x8, lay, 0);
        // prefix
        o.put(1, 1);
        o.put(0, 1);
        o.put(4, 2);           // messages
        o.put(1, 4);           // reference count
        o.put(m.b.size(), 4);  // header size
        o.put(0, 4);           // pad to 8
        const uint64_t msgs_at = o.b.size();
        o.bytes(m.b.data(), m.b.size());
        o.pad8();
        const uint64_t data_addr = o.b.size();
        o.bytes(it->bytes.data(), it->bytes.size());
        o.set(msgs_at + layout_body + 2, it->bytes.empty() ? UNDEF : data_addr, 8);
        o.set(msgs_at + layout_body + 10, it->bytes.size(), 8);
    }

    // --- symbol table node (one, sorted)
    o.pad8();
    const uint64_t snod = o.b.size();
    o.bytes("SNOD", 4);
    o.put(1, 1);
    o.put(0, 1);
    o.put(sorted.size(), 2);
    for (int e = 0; e < 2 * LEAF_K; e++) {
        if (e < (int) sorted.size()) {
            o.put(name_off[e], 8);
            o.put(obj_addr[e], 8);
        } else {
            o.put(0, 8);
            o.put(0, 8);
        }
        o.put(0, 4);
        o.put(0, 4);
        o.put(0, 16);
    }

    // --- group B-tree (version 1, type 0), one leaf child
    o.pad8();
    const uint64_t btree = o.b.size();
    o.bytes("TREE", 4);
    o.put(0, 1);  // node type: group
    o.put(0, 1);  // level
    o.put(1, 2);  // entries used
    o.put(UNDEF, 8);
    o.put(UNDEF, 8);
    o.put(0, 8);  // key 0: the empty name
    o.put(snod, 8);
    o.put(sorted.empty() ? 0 : name_off.back(), 8);  // key 1: largest name
    for (int i = 1; i < 2 * INTERNAL_K; i++) {
        o.put(0, 8);
        o.put(0, 8);
    }

    // --- root group object header: symbol table message
    o.pad8();
    const uint64_t root_hdr = o.b.size();
    Out m;
    std::vector<uint8_t> stm(16, 0);
    for (int i = 0; i < 8; i++) {
        stm[i] = (uint8_t) (btree >> (8 * i));
        stm[8 + i] = (uint8_t) (heap_addr >> (8 * i));
    }
    message(m, 0x11, stm, 0);
    o.put(1, 1);
    o.put(0, 1);
    o.put(1, 2);
    o.put(1, 4);
    o.put(m.b.size(), 4);
    o.put(0, 4);
    o.bytes(m.b.data(), m.b.size());
    o.pad8();

    o.set(root_ste + 8, root_hdr, 8);
    o.set(root_ste + 24, btree, 8);
    o.set(root_ste + 32, heap_addr, 8);
    o.set(eof_at, o.b.size(), 8);

    std::ofstream out(path, std::ios::binary | std::ios::trunc);
    if (!out) {
        err = "cannot create " + path;
        return false;
    }
    out.write((const char *) o.b.data(), (std::streamsize) o.b.size());
    if (!out) {
        err = "write failed: " + path;
        return false;
    }
    return true;
}

}  // namespace h5lite
