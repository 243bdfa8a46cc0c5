// host_hdf5.cpp -- Gadget-2 initial conditions from HDF5 files, without
// libhdf5 (absent here).
//
// grav_sim's galaxy-collision example reads its initial conditions through
// libhdf5 (examples/galaxy_collision/c/galaxy_collision.c:109-293): the
// attributes Header/NumPart_ThisFile and Units/"Unit length|mass|time in cgs
// (U_L|U_M|U_t)", and the datasets Masses, Coordinates, Velocities of
// PartType1 then PartType2 into one System.  load_gadget2_ic does the same
// by parsing the file directly, following the published HDF5 file format
// specification for the structures such files use: the version-0 superblock,
// version-1 object headers (with continuation blocks), groups stored as
// symbol tables (version-1 B-tree of group nodes, local heap, symbol table
// nodes), and dataspace, datatype (IEEE float, little-endian integers), data
// layout (contiguous or compact) and attribute messages.  Anything else
// (version-2 object headers, chunked or filtered datasets, big-endian data)
// is reported as an error rather than guessed at.  Every offset read from
// the file is checked against its size.
#include "gs_internal.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace gs {
namespace {

struct H5 {
    std::vector<unsigned char> d;
    int so = 8;   // size of offsets
    int sl = 8;   // size of lengths
    uint64_t base = 0;

    bool has(uint64_t off, uint64_t n) const { return off <= d.size() && n <= d.size() - off; }
    uint64_t u(uint64_t off, int n) const   // little-endian unsigned; caller checked has()
    {
        uint64_t v = 0;
        for (int k = n - 1; k >= 0; --k) v = (v << 8) | d[off + k];
        return v;
    }
};

#define H5_NEED(f, off, n)                                                                  \
    do {                                                                                    \
        if (!(f).has((off), (n)))                                                           \
            return GS_RAISE(GRAV_VALUE_ERROR, "HDF5 file truncated or corrupt at offset %llu", \
                            (unsigned long long)(off));                                     \
    } while (0)

ErrorStatus open_h5(const char *path, H5 &f)
{
    std::FILE *fp = std::fopen(path, "rb");
    if (!fp) return GS_RAISE(GRAV_OS_ERROR, "Failed to open initial condition file: \"%s\"", path);
    std::fseek(fp, 0, SEEK_END);
    const long len = std::ftell(fp);
    std::fseek(fp, 0, SEEK_SET);
    if (len < 0) {
        std::fclose(fp);
        return GS_RAISE(GRAV_OS_ERROR, "Failed to read initial condition file: \"%s\"", path);
    }
    f.d.resize((size_t)len);
    const size_t got = len > 0 ? std::fread(f.d.data(), 1, (size_t)len, fp) : 0;
    std::fclose(fp);
    if (got != (size_t)len)
        return GS_RAISE(GRAV_OS_ERROR, "Failed to read initial condition file: \"%s\"", path);
    static const unsigned char sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    if (!f.has(0, 96) || std::memcmp(f.d.data(), sig, 8) != 0)
        return GS_RAISE(GRAV_VALUE_ERROR, "\"%s\" is not an HDF5 file", path);
    if (f.d[8] != 0 && f.d[8] != 1)
        return GS_RAISE(GRAV_VALUE_ERROR,
                        "HDF5 superblock version %d is not supported (0 and 1 are)", f.d[8]);
    f.so = f.d[13];
    f.sl = f.d[14];
    if (f.so != 8 || f.sl != 8)
        return GS_RAISE(GRAV_VALUE_ERROR, "HDF5 offsets of %d and lengths of %d bytes are not supported",
                        f.so, f.sl);
    f.base = f.u(24, 8);
    return ok();
}

// Root group object header: the root symbol table entry of the superblock
// (version 0 at byte 56; version 1 has 4 more bytes before it).
ErrorStatus root_header(const H5 &f, uint64_t *ohdr)
{
    const uint64_t entry = f.d[8] == 0 ? 56 : 60;
    H5_NEED(f, entry, 40);
    *ohdr = f.base + f.u(entry + 8, 8);
    return ok();
}

struct Msg {
    int type;
    uint64_t off;   // message data
    uint64_t size;
};

// Messages of a version-1 object header, continuation blocks followed.
ErrorStatus header_messages(const H5 &f, uint64_t ohdr, std::vector<Msg> &out)
{
    out.clear();
    H5_NEED(f, ohdr, 16);
    if (f.d[ohdr] != 1)
        return GS_RAISE(GRAV_VALUE_ERROR,
                        "HDF5 object header version %d is not supported (1 is)", f.d[ohdr]);
    const uint64_t hsize = f.u(ohdr + 8, 4);
    std::vector<std::pair<uint64_t, uint64_t>> blocks{{ohdr + 16, hsize}};
    for (size_t b = 0; b < blocks.size() && b < 64; ++b) {
        uint64_t p = blocks[b].first;
        const uint64_t end = blocks[b].first + blocks[b].second;
        H5_NEED(f, blocks[b].first, blocks[b].second);
        while (p + 8 <= end) {
            const int type = (int)f.u(p, 2);
            const uint64_t size = f.u(p + 2, 2);
            if (p + 8 + size > end)
                return GS_RAISE(GRAV_VALUE_ERROR, "HDF5 object header message overruns its block");
            if (type == 0x10) {   // continuation: (offset, length)
                if (size < 16) return GS_RAISE(GRAV_VALUE_ERROR, "bad HDF5 continuation message");
                blocks.push_back({f.base + f.u(p + 8, 8), f.u(p + 16, 8)});
            } else if (type != 0) {
                out.push_back({type, p + 8, size});
            }
            p += 8 + size;
        }
    }
    return ok();
}

// Name of a local-heap entry.
ErrorStatus heap_name(const H5 &f, uint64_t heap, uint64_t name_off, std::string &name)
{
    H5_NEED(f, heap, 32);
    if (std::memcmp(&f.d[heap], "HEAP", 4) != 0)
        return GS_RAISE(GRAV_VALUE_ERROR, "HDF5 local heap signature missing");
    const uint64_t size = f.u(heap + 8, 8);
    const uint64_t data = f.base + f.u(heap + 24, 8);
    if (name_off >= size) return GS_RAISE(GRAV_VALUE_ERROR, "HDF5 heap offset out of range");
    H5_NEED(f, data, size);
    const unsigned char *s = &f.d[data + name_off];
    const size_t maxlen = (size_t)(size - name_off);
    const size_t len = strnlen(reinterpret_cast<const char *>(s), maxlen);
    name.assign(reinterpret_cast<const char *>(s), len);
    return ok();
}

// Search a version-1 B-tree of group nodes for `name`.
ErrorStatus btree_find(const H5 &f, uint64_t node, uint64_t heap, const std::string &name,
                       uint64_t *ohdr, bool *found, int depth)
{
    if (depth > 32) return GS_RAISE(GRAV_VALUE_ERROR, "HDF5 B-tree too deep");
    H5_NEED(f, node, 24);
    if (std::memcmp(&f.d[node], "TREE", 4) != 0 || f.d[node + 4] != 0)
        return GS_RAISE(GRAV_VALUE_ERROR, "HDF5 group B-tree node expected");
    const int level = f.d[node + 5];
    const int used = (int)f.u(node + 6, 2);
    // keys and children alternate after the two sibling addresses
    const uint64_t kc = node + 24;
    H5_NEED(f, kc, (uint64_t)(2 * used + 1) * 8);
    for (int c = 0; c < used && !*found; ++c) {
        const uint64_t child = f.base + f.u(kc + 8 + (uint64_t)c * 16, 8);
        if (level > 0) {
            GS_TRY(btree_find(f, child, heap, name, ohdr, found, depth + 1));
            continue;
        }
        H5_NEED(f, child, 8);
        if (std::memcmp(&f.d[child], "SNOD", 4) != 0)
            return GS_RAISE(GRAV_VALUE_ERROR, "HDF5 symbol table node expected");
        const int nsym = (int)f.u(child + 6, 2);
        H5_NEED(f, child + 8, (uint64_t)nsym * 40);
        for (int e = 0; e < nsym; ++e) {
            const uint64_t ent = child + 8 + (uint64_t)e * 40;
            std::string nm;
            GS_TRY(heap_name(f, heap, f.u(ent, 8), nm));
            if (nm == name) {
                *ohdr = f.base + f.u(ent + 8, 8);
                *found = true;
                break;
            }
        }
    }
    return ok();
}

ErrorStatus group_child(const H5 &f, uint64_t group, const std::string &name, uint64_t *child)
{
    std::vector<Msg> ms;
    GS_TRY(header_messages(f, group, ms));
    for (const Msg &m : ms) {
        if (m.type != 0x11) continue;   // symbol table message
        if (m.size < 16) return GS_RAISE(GRAV_VALUE_ERROR, "bad HDF5 symbol table message");
        const uint64_t bt = f.base + f.u(m.off, 8), heap = f.base + f.u(m.off + 8, 8);
        bool found = false;
        GS_TRY(btree_find(f, bt, heap, name, child, &found, 0));
        if (!found) return GS_RAISE(GRAV_OS_ERROR, "HDF5 object \"%s\" not found", name.c_str());
        return ok();
    }
    return GS_RAISE(GRAV_VALUE_ERROR,
                    "HDF5 group without a symbol table (only symbol-table groups are supported)");
}

ErrorStatus lookup(const H5 &f, const char *path, uint64_t *ohdr)
{
    GS_TRY(root_header(f, ohdr));
    std::string p(path);
    size_t at = 0;
    while (at < p.size()) {
        if (p[at] == '/') {
            ++at;
            continue;
        }
        const size_t end = p.find('/', at);
        const std::string part = p.substr(at, end == std::string::npos ? std::string::npos : end - at);
        GS_TRY(group_child(f, *ohdr, part, ohdr));
        if (end == std::string::npos) break;
        at = end + 1;
    }
    return ok();
}

struct Dtype {
    int cls = -1;     // 0 fixed point, 1 floating point
    int size = 0;
    bool sign = false;
};

ErrorStatus parse_dtype(const H5 &f, uint64_t off, uint64_t size, Dtype &t)
{
    if (size < 8) return GS_RAISE(GRAV_VALUE_ERROR, "bad HDF5 datatype message");
    H5_NEED(f, off, 8);
    t.cls = f.d[off] & 0x0f;
    const unsigned bits = (unsigned)f.u(off + 1, 3);
    t.size = (int)f.u(off + 4, 4);
    if (t.cls != 0 && t.cls != 1)
        return GS_RAISE(GRAV_VALUE_ERROR, "HDF5 datatype class %d is not supported (numbers only)",
                        t.cls);
    if (bits & 1u) return GS_RAISE(GRAV_VALUE_ERROR, "big-endian HDF5 data is not supported");
    if (t.cls == 1 && (bits & 0x40u))
        return GS_RAISE(GRAV_VALUE_ERROR, "VAX-order HDF5 floats are not supported");
    if (t.cls == 1 && t.size != 4 && t.size != 8)
        return GS_RAISE(GRAV_VALUE_ERROR, "HDF5 float of %d bytes is not supported", t.size);
    if (t.cls == 0 && t.size != 1 && t.size != 2 && t.size != 4 && t.size != 8)
        return GS_RAISE(GRAV_VALUE_ERROR, "HDF5 integer of %d bytes is not supported", t.size);
    t.sign = (bits & 0x08u) != 0;
    return ok();
}

// Number of elements of a dataspace message (scalar = 1).
ErrorStatus parse_space(const H5 &f, uint64_t off, uint64_t size, uint64_t *count,
                        std::vector<uint64_t> *dims)
{
    H5_NEED(f, off, 8);
    if (size < 4) return GS_RAISE(GRAV_VALUE_ERROR, "bad HDF5 dataspace message");
    const int ver = f.d[off], rank = f.d[off + 1];
    uint64_t first = 0;
    if (ver == 1) {
        first = off + 8;
    } else if (ver == 2) {
        if (f.d[off + 3] == 2) {   // null dataspace
            *count = 0;
            return ok();
        }
        first = off + 4;
    } else {
        return GS_RAISE(GRAV_VALUE_ERROR, "HDF5 dataspace version %d is not supported", ver);
    }
    H5_NEED(f, first, (uint64_t)rank * 8);
    uint64_t n = 1;
    if (dims) dims->clear();
    for (int k = 0; k < rank; ++k) {
        const uint64_t dk = f.u(first + (uint64_t)k * 8, 8);
        if (dims) dims->push_back(dk);
        if (dk > ((uint64_t)1 << 36) || (n *= dk) > ((uint64_t)1 << 36))
            return GS_RAISE(GRAV_VALUE_ERROR, "HDF5 dataspace too large");
    }
    *count = n;
    return ok();
}

// Convert count elements of type t at raw to double.
ErrorStatus convert(const H5 &f, uint64_t raw, const Dtype &t, uint64_t count,
                    std::vector<double> &out)
{
    H5_NEED(f, raw, count * (uint64_t)t.size);
    out.resize(count);
    const unsigned char *p = &f.d[raw];
    for (uint64_t i = 0; i < count; ++i, p += t.size) {
        if (t.cls == 1 && t.size == 8) {
            double v;
            std::memcpy(&v, p, 8);
            out[i] = v;
        } else if (t.cls == 1) {
            float v;
            std::memcpy(&v, p, 4);
            out[i] = v;
        } else {
            uint64_t v = 0;
            for (int k = t.size - 1; k >= 0; --k) v = (v << 8) | p[k];
            if (t.sign && t.size < 8 && (v >> (8 * t.size - 1)) & 1u) v |= ~0ull << (8 * t.size);
            out[i] = t.sign ? (double)(int64_t)v : (double)v;
        }
    }
    return ok();
}

ErrorStatus read_attribute(const H5 &f, uint64_t ohdr, const char *name, std::vector<double> &out)
{
    std::vector<Msg> ms;
    GS_TRY(header_messages(f, ohdr, ms));
    for (const Msg &m : ms) {
        if (m.type != 0x0c) continue;
        H5_NEED(f, m.off, 8);
        const int ver = f.d[m.off];
        const uint64_t nsz = f.u(m.off + 2, 2), tsz = f.u(m.off + 4, 2), ssz = f.u(m.off + 6, 2);
        uint64_t p = m.off + 8;
        if (ver == 3) ++p;   // character set encoding
        else if (ver != 1 && ver != 2)
            return GS_RAISE(GRAV_VALUE_ERROR, "HDF5 attribute version %d is not supported", ver);
        auto pad = [ver](uint64_t n) { return ver == 1 ? (n + 7) / 8 * 8 : n; };
        H5_NEED(f, p, nsz);
        const std::string nm(reinterpret_cast<const char *>(&f.d[p]),
                             strnlen(reinterpret_cast<const char *>(&f.d[p]), (size_t)nsz));
        p += pad(nsz);
        if (nm != name) continue;
        Dtype t;
        GS_TRY(parse_dtype(f, p, tsz, t));
        p += pad(tsz);
        uint64_t count = 0;
        GS_TRY(parse_space(f, p, ssz, &count, nullptr));
        p += pad(ssz);
        return convert(f, p, t, count, out);
    }
    return GS_RAISE(GRAV_OS_ERROR, "HDF5 attribute \"%s\" not found", name);
}

ErrorStatus read_dataset(const H5 &f, uint64_t ohdr, std::vector<double> &out,
                         std::vector<uint64_t> &dims)
{
    std::vector<Msg> ms;
    GS_TRY(header_messages(f, ohdr, ms));
    Dtype t;
    uint64_t count = 0;
    bool have_t = false, have_s = false;
    uint64_t raw = 0, raw_size = 0;
    bool have_l = false;
    for (const Msg &m : ms) {
        if (m.type == 0x03) {
            GS_TRY(parse_dtype(f, m.off, m.size, t));
            have_t = true;
        } else if (m.type == 0x01) {
            GS_TRY(parse_space(f, m.off, m.size, &count, &dims));
            have_s = true;
        } else if (m.type == 0x0b) {
            return GS_RAISE(GRAV_VALUE_ERROR, "filtered (compressed) HDF5 datasets are not supported");
        } else if (m.type == 0x08) {
            H5_NEED(f, m.off, 2);
            const int ver = f.d[m.off];
            if (ver == 3 || ver == 4) {
                const int cls = f.d[m.off + 1];
                if (cls == 0) {   // compact: size, data
                    H5_NEED(f, m.off + 2, 2);
                    raw_size = f.u(m.off + 2, 2);
                    raw = m.off + 4;
                } else if (cls == 1) {   // contiguous: address, size
                    H5_NEED(f, m.off + 2, 16);
                    raw = f.base + f.u(m.off + 2, 8);
                    raw_size = f.u(m.off + 10, 8);
                } else {
                    return GS_RAISE(GRAV_VALUE_ERROR,
                                    "chunked HDF5 datasets are not supported (layout class %d)", cls);
                }
            } else if (ver == 1 || ver == 2) {
                H5_NEED(f, m.off, 8);
                const int rank = f.d[m.off + 1], cls = f.d[m.off + 2];
                if (cls != 1)
                    return GS_RAISE(GRAV_VALUE_ERROR, "HDF5 layout class %d is not supported", cls);
                H5_NEED(f, m.off + 8, 8 + (uint64_t)rank * 4);
                raw = f.base + f.u(m.off + 8, 8);
                raw_size = ~0ull;
            } else {
                return GS_RAISE(GRAV_VALUE_ERROR, "HDF5 layout version %d is not supported", ver);
            }
            have_l = true;
        }
    }
    if (!have_t || !have_s || !have_l)
        return GS_RAISE(GRAV_VALUE_ERROR, "HDF5 dataset lacks a datatype, dataspace or layout");
    if (raw_size != ~0ull && raw_size < count * (uint64_t)t.size)
        return GS_RAISE(GRAV_VALUE_ERROR, "HDF5 dataset storage smaller than its dataspace");
    return convert(f, raw, t, count, out);
}

ErrorStatus read_part_type(const H5 &f, const char *group, uint64_t n, double *m, double *x,
                           double *v)
{
    const char *names[3] = {"Masses", "Coordinates", "Velocities"};
    double *dst[3] = {m, x, v};
    const uint64_t want[3] = {n, 3 * n, 3 * n};
    for (int k = 0; k < 3; ++k) {
        const std::string path = std::string(group) + "/" + names[k];
        uint64_t oh = 0;
        GS_TRY(lookup(f, path.c_str(), &oh));
        std::vector<double> buf;
        std::vector<uint64_t> dims;
        GS_TRY(read_dataset(f, oh, buf, dims));
        if (buf.size() != want[k])
            return GS_RAISE(GRAV_VALUE_ERROR, "%s holds %llu values, %llu expected", path.c_str(),
                            (unsigned long long)buf.size(), (unsigned long long)want[k]);
        std::memcpy(dst[k], buf.data(), buf.size() * sizeof(double));
    }
    return ok();
}

// ---- writer ----------------------------------------------------------
// Snapshot files in the layout of grav_sim's HDF5 output
// (src/output.c:483-695): group /Header with the int attributes
// NumFilesPerSnapshot, NumPart_ThisFile, NumPart_Total and the double
// attribute Time (each a one-element simple dataspace), and group
// /PartType0 with the datasets ParticleIDs (int32 [N]), Masses ([N]),
// Coordinates ([N][3]) and Velocities ([N][3]), FP32 or FP64 as the
// output dtypes say.  The file is built in memory with the same structures
// the reader above follows (version-0 superblock, version-1 object headers,
// symbol-table groups with one B-tree node and one symbol table node each,
// contiguous little-endian data) and written in one piece.

constexpr uint64_t H5_UNDEF = ~0ull;
constexpr int H5_LEAF_K = 4;       // symbol table node: 2K entries
constexpr int H5_INTERNAL_K = 16;  // group B-tree node: 2K children

class H5Builder {
  public:
    std::vector<unsigned char> b;

    uint64_t alloc(size_t n)
    {
        const uint64_t at = (b.size() + 7) & ~(uint64_t)7;
        b.resize(at + n, 0);
        return at;
    }
    void put(uint64_t at, uint64_t v, int n)
    {
        for (int k = 0; k < n; ++k) b[at + k] = (unsigned char)(v >> (8 * k));
    }
    void put_bytes(uint64_t at, const void *src, size_t n) { std::memcpy(&b[at], src, n); }
};

using Bytes = std::vector<unsigned char>;

void le(Bytes &o, uint64_t v, int n)
{
    for (int k = 0; k < n; ++k) o.push_back((unsigned char)(v >> (8 * k)));
}

void pad8(Bytes &o)
{
    while (o.size() % 8) o.push_back(0);
}

// Datatype message (version 1): little-endian int32, FP32 or FP64.
Bytes h5_dtype(int kind)
{
    Bytes o;
    if (kind == 0) {   // int32, signed
        o = {0x10, 0x08, 0x00, 0x00};
        le(o, 4, 4);
        le(o, 0, 2);    // bit offset
        le(o, 32, 2);   // precision
    } else if (kind == 1) {   // IEEE binary32
        o = {0x11, 0x20, 31, 0x00};
        le(o, 4, 4);
        le(o, 0, 2);
        le(o, 32, 2);
        o.push_back(23);   // exponent location
        o.push_back(8);    // exponent size
        o.push_back(0);    // mantissa location
        o.push_back(23);   // mantissa size
        le(o, 127, 4);     // exponent bias
    } else {   // IEEE binary64
        o = {0x11, 0x20, 63, 0x00};
        le(o, 8, 4);
        le(o, 0, 2);
        le(o, 64, 2);
        o.push_back(52);
        o.push_back(11);
        o.push_back(0);
        o.push_back(52);
        le(o, 1023, 4);
    }
    return o;
}

// Dataspace (version 1): simple with the given dimensions, scalar when none.
Bytes h5_space(const std::vector<uint64_t> &dims)
{
    Bytes o = {1, (unsigned char)dims.size(), 0, 0, 0, 0, 0, 0};
    for (uint64_t d : dims) le(o, d, 8);
    return o;
}

struct H5Msg {
    int type;
    Bytes data;
};

// Version-1 object header holding the messages (each padded to 8 bytes).
uint64_t h5_object_header(H5Builder &w, const std::vector<H5Msg> &msgs)
{
    size_t body = 0;
    for (const H5Msg &m : msgs) body += 8 + ((m.data.size() + 7) & ~(size_t)7);
    const uint64_t at = w.alloc(16 + body);
    w.put(at, 1, 1);   // version
    w.put(at + 2, msgs.size(), 2);
    w.put(at + 4, 1, 4);   // reference count
    w.put(at + 8, body, 4);
    uint64_t p = at + 16;
    for (const H5Msg &m : msgs) {
        const size_t sz = (m.data.size() + 7) & ~(size_t)7;
        w.put(p, (uint64_t)m.type, 2);
        w.put(p + 2, sz, 2);
        if (!m.data.empty()) w.put_bytes(p + 8, m.data.data(), m.data.size());
        p += 8 + sz;
    }
    return at;
}

struct H5Child {
    std::string name;   // children in ascending name order
    uint64_t ohdr;
    bool group;
    uint64_t btree, heap;   // a group's symbol table
};

// A group's local heap, B-tree node and symbol table node; returns the
// (B-tree, heap) addresses of its symbol table message.
void h5_symbol_table(H5Builder &w, const std::vector<H5Child> &kids, uint64_t *btree,
                     uint64_t *heap)
{
    Bytes data(8, 0);   // offset 0: the empty name
    std::vector<uint64_t> name_off;
    for (const H5Child &c : kids) {
        name_off.push_back(data.size());
        data.insert(data.end(), c.name.begin(), c.name.end());
        data.push_back(0);
        pad8(data);
    }
    const uint64_t hd = w.alloc(data.size());
    w.put_bytes(hd, data.data(), data.size());
    *heap = w.alloc(32);
    w.put_bytes(*heap, "HEAP", 4);
    w.put(*heap + 8, data.size(), 8);
    w.put(*heap + 16, H5_UNDEF, 8);   // no free block
    w.put(*heap + 24, hd, 8);
    uint64_t snod = 0;
    if (!kids.empty()) {
        snod = w.alloc(8 + 2 * H5_LEAF_K * 40);
        w.put_bytes(snod, "SNOD", 4);
        w.put(snod + 4, 1, 1);
        w.put(snod + 6, kids.size(), 2);
        for (size_t k = 0; k < kids.size(); ++k) {
            const uint64_t e = snod + 8 + 40 * k;
            w.put(e, name_off[k], 8);
            w.put(e + 8, kids[k].ohdr, 8);
            if (kids[k].group) {
                w.put(e + 16, 1, 4);   // cache type 1: the symbol table's addresses
                w.put(e + 24, kids[k].btree, 8);
                w.put(e + 32, kids[k].heap, 8);
            }
        }
    }
    *btree = w.alloc(24 + 8 * (2 * H5_INTERNAL_K + 1) + 8 * (2 * H5_INTERNAL_K));
    w.put_bytes(*btree, "TREE", 4);
    w.put(*btree + 4, 0, 1);   // group node
    w.put(*btree + 5, 0, 1);   // leaf level
    w.put(*btree + 6, kids.empty() ? 0 : 1, 2);
    w.put(*btree + 8, H5_UNDEF, 8);
    w.put(*btree + 16, H5_UNDEF, 8);
    if (!kids.empty()) {
        w.put(*btree + 24, 0, 8);                       // key 0: the empty name
        w.put(*btree + 32, snod, 8);                    // child 0
        w.put(*btree + 40, name_off.back(), 8);         // key 1: the last name
    }
}

H5Msg h5_symbol_table_msg(uint64_t btree, uint64_t heap)
{
    Bytes o;
    le(o, btree, 8);
    le(o, heap, 8);
    return {0x11, o};
}

// Attribute message (version 1) holding one value: a one-element simple
// dataspace, or a scalar one.
H5Msg h5_attribute(const char *name, int kind, const void *value, bool scalar = false)
{
    Bytes nm(name, name + std::strlen(name) + 1);
    const Bytes t = h5_dtype(kind), sp = scalar ? h5_space({}) : h5_space({1});
    Bytes o = {1, 0};
    le(o, nm.size(), 2);
    le(o, t.size(), 2);
    le(o, sp.size(), 2);
    o.insert(o.end(), nm.begin(), nm.end());
    pad8(o);
    o.insert(o.end(), t.begin(), t.end());
    pad8(o);
    o.insert(o.end(), sp.begin(), sp.end());
    pad8(o);
    const int vsize = kind == 2 ? 8 : 4;
    const unsigned char *v = static_cast<const unsigned char *>(value);
    o.insert(o.end(), v, v + vsize);
    return {0x0c, o};
}

// A contiguous dataset: its raw data, then its object header.
uint64_t h5_dataset(H5Builder &w, int kind, const std::vector<uint64_t> &dims, const void *raw,
                    size_t raw_bytes)
{
    const uint64_t data = w.alloc(raw_bytes);
    if (raw_bytes) w.put_bytes(data, raw, raw_bytes);
    Bytes fill = {2, 2, 2, 0};   // fill value (v2): late allocation, never written, undefined
    Bytes layout = {3, 1};       // data layout (v3): contiguous
    le(layout, data, 8);
    le(layout, raw_bytes, 8);
    return h5_object_header(w, {{0x01, h5_space(dims)}, {0x03, h5_dtype(kind)}, {0x05, fill},
                                {0x08, layout}});
}

}  // namespace

ErrorStatus write_snapshot_hdf5(const char *path, int n, const int *ids, const double *x,
                                const double *v, const double *m, double t, bool x_float,
                                bool v_float, bool m_float, const CosmologyHeader *cosmo)
{
    if (n < 0) return GS_RAISE(GRAV_VALUE_ERROR, "negative particle count %d", n);
    const size_t N = (size_t)n;
    H5Builder w;
    w.alloc(96);   // superblock, filled last
    // /PartType0 datasets
    std::vector<float> f32;
    auto dataset = [&](bool as_float, const double *src, size_t count,
                       std::vector<uint64_t> dims) -> uint64_t {
        if (as_float) {
            f32.resize(count);
            for (size_t i = 0; i < count; ++i) f32[i] = (float)src[i];
            return h5_dataset(w, 1, dims, f32.data(), count * 4);
        }
        return h5_dataset(w, 2, dims, src, count * 8);
    };
    const uint64_t d_coord = dataset(x_float, x, 3 * N, {N, 3});
    const uint64_t d_mass = dataset(m_float, m, N, {N});
    const uint64_t d_ids = h5_dataset(w, 0, {N}, ids, N * 4);
    const uint64_t d_vel = dataset(v_float, v, 3 * N, {N, 3});
    uint64_t pt_bt = 0, pt_heap = 0;
    h5_symbol_table(w,
                    {{"Coordinates", d_coord, false, 0, 0}, {"Masses", d_mass, false, 0, 0},
                     {"ParticleIDs", d_ids, false, 0, 0}, {"Velocities", d_vel, false, 0, 0}},
                    &pt_bt, &pt_heap);
    const uint64_t pt = h5_object_header(w, {h5_symbol_table_msg(pt_bt, pt_heap)});
    // /Header: an empty group with four attributes; a cosmological snapshot
    // (src/output.c:697-900) has a scalar Time and Redshift = 1/a - 1,
    // Omega0 and OmegaLambda besides
    uint64_t hd_bt = 0, hd_heap = 0;
    h5_symbol_table(w, {}, &hd_bt, &hd_heap);
    const int one = 1;
    std::vector<H5Msg> hmsg = {h5_symbol_table_msg(hd_bt, hd_heap),
                               h5_attribute("NumFilesPerSnapshot", 0, &one),
                               h5_attribute("NumPart_ThisFile", 0, &n),
                               h5_attribute("NumPart_Total", 0, &n),
                               h5_attribute("Time", 2, &t, cosmo != nullptr)};
    const double z = 1.0 / t - 1.0;
    if (cosmo) {
        hmsg.push_back(h5_attribute("Redshift", 2, &z, true));
        hmsg.push_back(h5_attribute("Omega0", 2, &cosmo->omega_m, true));
        hmsg.push_back(h5_attribute("OmegaLambda", 2, &cosmo->omega_lambda, true));
    }
    const uint64_t hdr = h5_object_header(w, hmsg);
    std::vector<H5Child> root_kids = {{"Header", hdr, true, hd_bt, hd_heap},
                                      {"PartType0", pt, true, pt_bt, pt_heap}};
    if (cosmo) {
        // /Units: the cgs units, current and temperature 1
        uint64_t un_bt = 0, un_heap = 0;
        h5_symbol_table(w, {}, &un_bt, &un_heap);
        const double unity = 1.0;
        const uint64_t un = h5_object_header(
            w, {h5_symbol_table_msg(un_bt, un_heap),
                h5_attribute("Unit current in cgs (U_I)", 2, &unity, true),
                h5_attribute("Unit length in cgs (U_L)", 2, &cosmo->unit_length, true),
                h5_attribute("Unit mass in cgs (U_M)", 2, &cosmo->unit_mass, true),
                h5_attribute("Unit time in cgs (U_t)", 2, &cosmo->unit_time, true),
                h5_attribute("Unit temperature in cgs (U_T)", 2, &unity, true)});
        root_kids.push_back({"Units", un, true, un_bt, un_heap});
    }
    // root group
    uint64_t rt_bt = 0, rt_heap = 0;
    h5_symbol_table(w, root_kids, &rt_bt, &rt_heap);
    const uint64_t root = h5_object_header(w, {h5_symbol_table_msg(rt_bt, rt_heap)});
    // superblock (version 0)
    static const unsigned char sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    w.put_bytes(0, sig, 8);
    w.put(13, 8, 1);   // size of offsets
    w.put(14, 8, 1);   // size of lengths
    w.put(16, H5_LEAF_K, 2);
    w.put(18, H5_INTERNAL_K, 2);
    w.put(24, 0, 8);          // base address
    w.put(32, H5_UNDEF, 8);   // free-space info
    w.put(40, w.b.size(), 8); // end of file
    w.put(48, H5_UNDEF, 8);   // driver information
    w.put(56, 0, 8);          // root entry: name offset
    w.put(64, root, 8);
    w.put(72, 1, 4);          // cache type 1
    w.put(80, rt_bt, 8);
    w.put(88, rt_heap, 8);
    std::FILE *fp = std::fopen(path, "wb");
    if (!fp)
        return GS_RAISE(GRAV_OS_ERROR, "Failed to create HDF5 file for storing snapshots: \"%s\".",
                        path);
    const size_t wrote = std::fwrite(w.b.data(), 1, w.b.size(), fp);
    const bool bad = wrote != w.b.size() || std::ferror(fp) != 0;
    std::fclose(fp);
    if (bad) return GS_RAISE(GRAV_OS_ERROR, "Failed to write snapshot file: \"%s\".", path);
    return ok();
}

namespace {

// The values of one dataset or attribute of a file, by path (a test and
// reading aid for the snapshots above).
ErrorStatus read_path(const char *path, const char *object, const char *attribute,
                      std::vector<double> &out, std::vector<uint64_t> &dims)
{
    H5 f;
    GS_TRY(open_h5(path, f));
    uint64_t oh = 0;
    GS_TRY(lookup(f, object, &oh));
    if (attribute) {
        dims.clear();
        GS_TRY(read_attribute(f, oh, attribute, out));
        dims.push_back(out.size());
        return ok();
    }
    return read_dataset(f, oh, out, dims);
}

}  // namespace
}  // namespace gs

extern "C" {

int gsgpu_hdf5_read(const char *path, const char *object, const char *attribute, double *out,
                    long long capacity, long long *count)
{
    if (!path || !object || !count) return GRAV_POINTER_ERROR;
    std::vector<double> v;
    std::vector<uint64_t> dims;
    ErrorStatus st = gs::read_path(path, object, attribute, v, dims);
    if (st.return_code != GRAV_SUCCESS) {
        print_and_free_traceback(&st);
        return st.return_code;
    }
    *count = (long long)v.size();
    if (out) {
        if ((long long)v.size() > capacity) return GRAV_VALUE_ERROR;
        std::memcpy(out, v.data(), v.size() * sizeof(double));
    }
    return GRAV_SUCCESS;
}

int gsgpu_write_snapshot_hdf5(const char *path, int num_particles, const int *ids,
                              const double *x, const double *v, const double *m, double t,
                              int coordinate_output_dtype, int velocity_output_dtype,
                              int mass_output_dtype)
{
    if (!path || (num_particles > 0 && (!ids || !x || !v || !m))) return GRAV_POINTER_ERROR;
    ErrorStatus st = gs::write_snapshot_hdf5(
        path, num_particles, ids, x, v, m, t, coordinate_output_dtype == OUTPUT_DTYPE_FLOAT,
        velocity_output_dtype == OUTPUT_DTYPE_FLOAT, mass_output_dtype == OUTPUT_DTYPE_FLOAT,
        nullptr);
    if (st.return_code != GRAV_SUCCESS) {
        print_and_free_traceback(&st);
        return st.return_code;
    }
    return GRAV_SUCCESS;
}

// src/system.c: free_system releases the four arrays of a System.
void free_system(System *system)
{
    if (!system) return;
    std::free(system->particle_ids);
    std::free(system->x);
    std::free(system->v);
    std::free(system->m);
    system->particle_ids = nullptr;
    system->x = system->v = system->m = nullptr;
}

ErrorStatus load_gadget2_ic(const char *path, System *system, double *unit_length,
                            double *unit_mass, double *unit_time)
{
    using namespace gs;
    if (!path || !system) return GS_RAISE(GRAV_POINTER_ERROR, "NULL argument");
    H5 f;
    GS_TRY(open_h5(path, f));
    uint64_t header = 0, units = 0;
    GS_TRY(lookup(f, "/Header", &header));
    GS_TRY(lookup(f, "/Units", &units));
    std::vector<double> np;
    GS_TRY(read_attribute(f, header, "NumPart_ThisFile", np));
    if (np.size() < 3) return GS_RAISE(GRAV_VALUE_ERROR, "NumPart_ThisFile has %zu entries", np.size());
    const uint64_t n1 = (uint64_t)np[1], n2 = (uint64_t)np[2];
    if (n1 + n2 == 0 || n1 + n2 > 0x7fffffffull)
        return GS_RAISE(GRAV_VALUE_ERROR, "NumPart_ThisFile gives %llu particles of types 1 and 2",
                        (unsigned long long)(n1 + n2));
    const char *unit_names[3] = {"Unit length in cgs (U_L)", "Unit mass in cgs (U_M)",
                                 "Unit time in cgs (U_t)"};
    double *unit_out[3] = {unit_length, unit_mass, unit_time};
    double units_v[3];
    for (int k = 0; k < 3; ++k) {
        std::vector<double> u;
        GS_TRY(read_attribute(f, units, unit_names[k], u));
        if (u.size() != 1) return GS_RAISE(GRAV_VALUE_ERROR, "%s is not a scalar", unit_names[k]);
        units_v[k] = u[0];
    }
    const int n = (int)(n1 + n2);
    System s = get_new_system();
    s.num_particles = n;
    s.particle_ids = static_cast<int *>(std::malloc((size_t)n * sizeof(int)));
    s.x = static_cast<double *>(std::calloc((size_t)n * 3, sizeof(double)));
    s.v = static_cast<double *>(std::calloc((size_t)n * 3, sizeof(double)));
    s.m = static_cast<double *>(std::calloc((size_t)n, sizeof(double)));
    if (!s.particle_ids || !s.x || !s.v || !s.m) {
        free_system(&s);
        return GS_RAISE(GRAV_MEMORY_ERROR, "Failed to allocate memory for system");
    }
    for (int i = 0; i < n; ++i) s.particle_ids[i] = i;
    ErrorStatus st = read_part_type(f, "/PartType1", n1, s.m, s.x, s.v);
    if (st.return_code == GRAV_SUCCESS)
        st = read_part_type(f, "/PartType2", n2, s.m + n1, s.x + 3 * n1, s.v + 3 * n1);
    if (st.return_code != GRAV_SUCCESS) {
        free_system(&s);
        return gs::traceback(st, "read_part_type(...)", __FILE__, __LINE__, __func__);
    }
    for (int k = 0; k < 3; ++k)
        if (unit_out[k]) *unit_out[k] = units_v[k];
    *system = s;
    return ok();
}

}  // extern "C"
