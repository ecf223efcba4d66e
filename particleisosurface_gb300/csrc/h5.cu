// Host formats: HDF5 particle files and XDMF frame lists.
//
// The reference reads a frame with the HDF5 library (readShonDyParticleData,
// src/main.cpp:281-327, with size / readDouble of src/hdf5Utils.cpp:60-90):
// the dataset "position" (3N doubles) and, for per-particle radii,
// "particleRadius" (N doubles), each double converted to float.  Its frame
// list comes from an XDMF file (readShonDyParticleXDMF, src/hdf5Utils.cpp:
// 7-47): the text of Xdmf/Domain/Grid/Grid/Geometry/DataItem up to the first
// ':' names each frame's file.
//
// The HDF5 library is not part of this build, so the file format is read
// here, following the published HDF5 File Format Specification (version 3.0),
// for the structures such files use:
//   - superblock versions 0-3, found at 0, 512, 1024, ... (user block);
//   - object headers version 1 and 2 ("OHDR") with continuation blocks;
//   - groups by symbol table (version 1 B-tree of "SNOD" nodes with a local
//     heap of names) or by link messages (compact groups); groups stored in
//     a fractal heap are reported as unsupported;
//   - datasets with a simple dataspace, fixed-point or IEEE floating-point
//     element types of either byte order, converted to double as H5Dread
//     does into H5T_NATIVE_DOUBLE;
//   - compact, contiguous and chunked layouts (layout message versions 1-4;
//     chunks indexed by a version 1 B-tree, or a single chunk), with the
//     deflate (RFC 1950/1951 stream, decoded here), shuffle and Fletcher-32
//     filters.
// Anything else raises an error naming the structure.
#include <cstdint>
#include <cstring>
#include <fstream>
#include <functional>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "internal.h"

namespace pisurf {
namespace {

struct FormatError : std::invalid_argument {
  explicit FormatError(const std::string& s) : std::invalid_argument("HDF5: " + s) {}
};

// ---------------------------------------------------------------------------
// DEFLATE decoder (RFC 1951) for zlib streams (RFC 1950): canonical Huffman
// codes decoded bit by bit from per-length counts, LSB-first bit order.
// ---------------------------------------------------------------------------
class Inflater {
 public:
  Inflater(const uint8_t* p, size_t n) : in_(p), n_(n) {}

  std::vector<uint8_t> zlib(size_t expect) {
    if (n_ < 2) throw FormatError("deflate stream too short");
    const int cmf = in_[0], flg = in_[1];
    if ((cmf & 15) != 8 || ((cmf << 8) | flg) % 31 != 0) throw FormatError("not a zlib deflate stream");
    if (flg & 0x20) throw FormatError("deflate stream with a preset dictionary");
    pos_ = 2;
    out_.reserve(expect);
    int last = 0;
    while (!last) {
      last = bits(1);
      const int type = bits(2);
      if (type == 0) {
        stored();
      } else if (type == 1) {
        fixed_tables();
        codes();
      } else if (type == 2) {
        dynamic_tables();
        codes();
      } else {
        throw FormatError("invalid deflate block type");
      }
    }
    return std::move(out_);
  }

 private:
  struct Huff {
    int count[16];
    int symbol[320];
  };
  const uint8_t* in_;
  size_t n_, pos_ = 0;
  uint32_t bitbuf_ = 0;
  int bitcnt_ = 0;
  std::vector<uint8_t> out_;
  Huff lit_, dist_;

  int bits(int need) {
    uint32_t v = bitbuf_;
    while (bitcnt_ < need) {
      if (pos_ >= n_) throw FormatError("deflate stream truncated");
      v |= (uint32_t)in_[pos_++] << bitcnt_;
      bitcnt_ += 8;
    }
    bitbuf_ = v >> need;
    bitcnt_ -= need;
    return (int)(v & ((1u << need) - 1u));
  }

  void stored() {
    bitbuf_ = 0;
    bitcnt_ = 0;
    if (pos_ + 4 > n_) throw FormatError("deflate stream truncated");
    const unsigned len = in_[pos_] | (in_[pos_ + 1] << 8);
    const unsigned nlen = in_[pos_ + 2] | (in_[pos_ + 3] << 8);
    pos_ += 4;
    if (len != (~nlen & 0xffffu)) throw FormatError("deflate stored block length check");
    if (pos_ + len > n_) throw FormatError("deflate stream truncated");
    out_.insert(out_.end(), in_ + pos_, in_ + pos_ + len);
    pos_ += len;
  }

  // counts and symbols of the canonical code with the given code lengths
  static void build(Huff& h, const uint8_t* len, int n) {
    for (int i = 0; i < 16; ++i) h.count[i] = 0;
    for (int s = 0; s < n; ++s) h.count[len[s]]++;
    int offs[16];
    offs[1] = 0;
    for (int i = 1; i < 15; ++i) offs[i + 1] = offs[i] + h.count[i];
    for (int s = 0; s < n; ++s)
      if (len[s]) h.symbol[offs[len[s]]++] = s;
  }

  int decode(const Huff& h) {
    int code = 0, first = 0, index = 0;
    for (int len = 1; len < 16; ++len) {
      code |= bits(1);
      const int cnt = h.count[len];
      if (code - cnt < first) return h.symbol[index + (code - first)];
      index += cnt;
      first = (first + cnt) << 1;
      code <<= 1;
    }
    throw FormatError("invalid deflate code");
  }

  void fixed_tables() {
    uint8_t len[288];
    int s = 0;
    for (; s < 144; ++s) len[s] = 8;
    for (; s < 256; ++s) len[s] = 9;
    for (; s < 280; ++s) len[s] = 7;
    for (; s < 288; ++s) len[s] = 8;
    build(lit_, len, 288);
    for (s = 0; s < 30; ++s) len[s] = 5;
    build(dist_, len, 30);
  }

  void dynamic_tables() {
    const int nlen = bits(5) + 257, ndist = bits(5) + 1, ncode = bits(4) + 4;
    if (nlen > 286 || ndist > 30) throw FormatError("invalid deflate table sizes");
    static const int order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
    uint8_t len[320] = {0};
    for (int i = 0; i < ncode; ++i) len[order[i]] = (uint8_t)bits(3);
    Huff lens;
    build(lens, len, 19);
    int i = 0;
    while (i < nlen + ndist) {
      const int sym = decode(lens);
      if (sym < 16) {
        len[i++] = (uint8_t)sym;
        continue;
      }
      int rep, val = 0;
      if (sym == 16) {
        if (i == 0) throw FormatError("deflate repeat with no previous length");
        val = len[i - 1];
        rep = 3 + bits(2);
      } else if (sym == 17) {
        rep = 3 + bits(3);
      } else {
        rep = 11 + bits(7);
      }
      if (i + rep > nlen + ndist) throw FormatError("deflate code lengths overrun");
      while (rep--) len[i++] = (uint8_t)val;
    }
    build(lit_, len, nlen);
    build(dist_, len + nlen, ndist);
  }

  void codes() {
    static const int lbase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                                  31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
    static const int lext[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
    static const int dbase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                  193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
    static const int dext[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
    for (;;) {
      int sym = decode(lit_);
      if (sym < 256) {
        out_.push_back((uint8_t)sym);
      } else if (sym == 256) {
        return;
      } else {
        sym -= 257;
        if (sym >= 29) throw FormatError("invalid deflate length code");
        const int len = lbase[sym] + bits(lext[sym]);
        const int ds = decode(dist_);
        if (ds >= 30) throw FormatError("invalid deflate distance code");
        const size_t dist = (size_t)(dbase[ds] + bits(dext[ds]));
        if (dist > out_.size()) throw FormatError("deflate distance beyond the output");
        const size_t from = out_.size() - dist;
        for (int k = 0; k < len; ++k) out_.push_back(out_[from + k]);
      }
    }
  }
};

// ---------------------------------------------------------------------------
// HDF5 structures
// ---------------------------------------------------------------------------
constexpr uint64_t kUndef = ~0ull;

struct Msg {
  int type;
  const uint8_t* p;
  size_t n;
};

struct Dataset {
  std::vector<uint64_t> dims;
  int cls = -1, size = 0, big = 0, sign = 0;
  int layout = -1;  // 0 compact, 1 contiguous, 2 chunked
  uint64_t addr = kUndef, bytes = 0;
  const uint8_t* compact = nullptr;
  std::vector<uint64_t> chunk;  // chunk dims (rank entries)
  int chunk_index = 0;          // 0: version 1 B-tree, 1: single chunk
  uint64_t single_size = 0;
  uint32_t single_mask = 0;
  std::vector<int> filters;
};

class H5 {
 public:
  explicit H5(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::invalid_argument("cannot read hdf5 file: " + path);
    f.seekg(0, std::ios::end);
    const std::streamoff n = f.tellg();
    f.seekg(0);
    buf_.resize((size_t)n);
    if (n > 0) f.read(reinterpret_cast<char*>(buf_.data()), n);
    if (!f) throw std::invalid_argument("cannot read hdf5 file: " + path);
    superblock();
  }

  // values of the dataset at `path` (a name in the root group, or a path of
  // group names separated by '/'), converted to double, and its dims
  std::vector<double> read(const std::string& path, std::vector<uint64_t>* dims_out) {
    uint64_t oh = root_;
    size_t s = 0;
    while (s < path.size()) {
      while (s < path.size() && path[s] == '/') ++s;
      size_t e = path.find('/', s);
      if (e == std::string::npos) e = path.size();
      if (e > s) oh = lookup(oh, path.substr(s, e - s));
      s = e;
    }
    Dataset d = dataset(oh, path);
    if (dims_out) *dims_out = d.dims;
    return values(d);
  }

 private:
  std::vector<uint8_t> buf_;
  uint64_t base_ = 0, root_ = kUndef;
  int so_ = 8, sl_ = 8;

  const uint8_t* at(uint64_t abs, uint64_t n) const {
    if (abs > buf_.size() || n > buf_.size() - abs) throw FormatError("structure outside the file");
    return buf_.data() + abs;
  }
  static uint64_t le(const uint8_t* p, int n) {
    uint64_t v = 0;
    for (int i = n - 1; i >= 0; --i) v = (v << 8) | p[i];
    return v;
  }
  // an address field (relative to the base address) as an absolute offset
  uint64_t addr(const uint8_t* p) const {
    const uint64_t v = le(p, so_);
    if (so_ < 8 && v == ((1ull << (8 * so_)) - 1ull)) return kUndef;
    return v == kUndef ? kUndef : v + base_;
  }

  void superblock() {
    static const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    uint64_t off = 0;
    for (;;) {
      if (off + 8 > buf_.size()) throw FormatError("no superblock signature (not an HDF5 file)");
      if (std::memcmp(buf_.data() + off, sig, 8) == 0) break;
      off = off ? off * 2 : 512;
    }
    const uint8_t* p = at(off, 12);
    const int ver = p[8];
    if (ver <= 1) {
      p = at(off, 24);
      so_ = p[13];
      sl_ = p[14];
      const uint64_t fixed = ver == 0 ? 24 : 28;
      const uint8_t* q = at(off + fixed, 4 * (uint64_t)so_ + 2 * (uint64_t)so_ + 24);
      base_ = le(q, so_);
      // the root group's symbol table entry follows the four addresses
      const uint8_t* e = q + 4 * so_;
      root_ = le(e + so_, so_) + base_;
    } else if (ver <= 3) {
      so_ = p[9];
      sl_ = p[10];
      const uint8_t* q = at(off + 12, 4 * (uint64_t)so_);
      base_ = le(q, so_);
      root_ = le(q + 3 * so_, so_) + base_;
    } else {
      throw FormatError("superblock version " + std::to_string(ver));
    }
    if (so_ < 2 || so_ > 8 || sl_ < 2 || sl_ > 8) throw FormatError("unsupported size of offsets or lengths");
  }

  // the messages of the object header at absolute offset oh
  std::vector<Msg> header(uint64_t oh) const {
    const uint8_t* p = at(oh, 16);
    std::vector<std::pair<uint64_t, uint64_t>> blocks;  // (start, length) of message blocks
    bool v2 = false;
    if (std::memcmp(p, "OHDR", 4) == 0) {
      v2 = true;
      const int flags = p[5];
      uint64_t o = oh + 6;
      if (flags & 0x20) o += 16;
      if (flags & 0x10) o += 4;
      const int w = 1 << (flags & 3);
      const uint64_t size = le(at(o, w), w);
      o += w;
      blocks.push_back({o, size});
      return walk(blocks, v2, flags);
    }
    if (p[0] != 1) throw FormatError("object header version " + std::to_string(p[0]));
    const uint64_t size = le(p + 8, 4);
    blocks.push_back({oh + 16, size});
    return walk(blocks, v2, 0);
  }

  std::vector<Msg> walk(std::vector<std::pair<uint64_t, uint64_t>> blocks, bool v2, int flags) const {
    std::vector<Msg> out;
    for (size_t b = 0; b < blocks.size(); ++b) {
      uint64_t o = blocks[b].first;
      uint64_t end = o + blocks[b].second;
      if (v2 && b > 0) {  // continuation chunk: "OCHK", messages, checksum
        if (std::memcmp(at(o, 4), "OCHK", 4) != 0) throw FormatError("bad object header continuation");
        o += 4;
        end -= 4;
      }
      const uint64_t hdr = v2 ? ((flags & 4) ? 6 : 4) : 8;
      while (o + hdr <= end) {
        const uint8_t* m = at(o, hdr);
        const int type = v2 ? m[0] : (int)le(m, 2);
        const uint64_t n = v2 ? le(m + 1, 2) : le(m + 2, 2);
        const uint8_t* data = at(o + hdr, n);
        if (type == 0x10) {
          blocks.push_back({addr(data), le(data + so_, sl_)});
        } else if (type != 0) {
          out.push_back({type, data, (size_t)n});
        }
        o += hdr + n;
      }
    }
    return out;
  }

  // object header of the link `name` in the group whose header is at oh
  uint64_t lookup(uint64_t oh, const std::string& name) const {
    for (const Msg& m : header(oh)) {
      if (m.type == 0x11) {  // symbol table: B-tree (version 1, group nodes) and local heap
        const uint64_t tree = addr(m.p), heap = addr(m.p + so_);
        const uint8_t* h = at(heap, 8 + 2 * (uint64_t)sl_ + so_);
        if (std::memcmp(h, "HEAP", 4) != 0) throw FormatError("bad local heap");
        const uint64_t data = addr(h + 8 + 2 * sl_);
        uint64_t found = kUndef;
        group_tree(tree, [&](uint64_t name_off, uint64_t obj) {
          const char* s = reinterpret_cast<const char*>(at(data + name_off, 1));
          const size_t maxlen = buf_.size() - (data + name_off);
          if (strnlen(s, maxlen) == name.size() && std::memcmp(s, name.data(), name.size()) == 0) found = obj;
        });
        if (found != kUndef) return found;
      } else if (m.type == 0x06) {  // link message
        const uint8_t* p = m.p;
        const int flags = p[1];
        size_t o = 2;
        int ltype = 0;
        if (flags & 0x08) ltype = p[o++];
        if (flags & 0x04) o += 8;
        if (flags & 0x10) o += 1;
        const int w = 1 << (flags & 3);
        const uint64_t len = le(p + o, w);
        o += w;
        if (o + len > m.n) throw FormatError("bad link message");
        if (ltype == 0 && len == name.size() && std::memcmp(p + o, name.data(), len) == 0) return addr(p + o + len);
      } else if (m.type == 0x02) {
        const uint8_t* p = m.p;
        const uint64_t heap = addr(p + 2 + ((p[1] & 1) ? 8 : 0));
        if (heap != kUndef) throw FormatError("groups in dense link storage (fractal heap) are not supported");
      }
    }
    throw std::invalid_argument("hdf5 file has no object '" + name + "'");
  }

  // every (name offset, object header) of a group's version 1 B-tree
  void group_tree(uint64_t node, const std::function<void(uint64_t, uint64_t)>& fn) const {
    const uint8_t* p = at(node, 8 + 2 * (uint64_t)so_);
    if (std::memcmp(p, "TREE", 4) != 0 || p[4] != 0) throw FormatError("bad group B-tree node");
    const int level = p[5];
    const int used = (int)le(p + 6, 2);
    const uint64_t kids = node + 8 + 2 * so_;
    for (int i = 0; i < used; ++i) {
      const uint64_t child = addr(at(kids + (uint64_t)i * (sl_ + so_) + sl_, so_));
      if (level > 0) {
        group_tree(child, fn);
        continue;
      }
      const uint8_t* s = at(child, 8);
      if (std::memcmp(s, "SNOD", 4) != 0) throw FormatError("bad symbol table node");
      const int nsym = (int)le(s + 6, 2);
      const uint64_t esz = 2 * (uint64_t)so_ + 24;
      for (int k = 0; k < nsym; ++k) {
        const uint8_t* e = at(child + 8 + k * esz, esz);
        fn(le(e, so_), addr(e + so_));
      }
    }
  }

  Dataset dataset(uint64_t oh, const std::string& name) const {
    Dataset d;
    for (const Msg& m : header(oh)) {
      const uint8_t* p = m.p;
      if (m.type == 0x01) {  // dataspace
        const int ver = p[0], rank = p[1], flags = p[2];
        size_t o = ver == 1 ? 8 : 4;
        d.dims.clear();
        for (int i = 0; i < rank; ++i) d.dims.push_back(le(p + o + (size_t)i * sl_, sl_));
        if (ver == 2 && p[3] == 2) d.dims.assign(1, 0);  // null dataspace: no elements
        (void)flags;
      } else if (m.type == 0x03) {  // datatype
        d.cls = p[0] & 15;
        d.big = p[1] & 1;
        d.sign = (p[1] >> 3) & 1;
        d.size = (int)le(p + 4, 4);
      } else if (m.type == 0x08) {  // data layout
        layout(p, m.n, d);
      } else if (m.type == 0x0B) {  // filter pipeline
        const int ver = p[0], nf = p[1];
        size_t o = ver == 1 ? 8 : 2;
        for (int i = 0; i < nf; ++i) {
          const int id = (int)le(p + o, 2);
          size_t namelen = (ver == 1 || id >= 256) ? le(p + o + 2, 2) : 0;
          o += (ver == 1 || id >= 256) ? 4 : 2;
          const int nvals = (int)le(p + o + 2, 2);
          o += 4;
          if (ver == 1) namelen = (namelen + 7) / 8 * 8;
          o += namelen + 4 * (size_t)nvals;
          if (ver == 1 && (nvals & 1)) o += 4;
          d.filters.push_back(id);
        }
      }
    }
    if (d.cls < 0 || d.layout < 0) throw std::invalid_argument("hdf5 object '" + name + "' is not a dataset");
    if (d.cls != 0 && d.cls != 1) throw FormatError("dataset '" + name + "': element class " + std::to_string(d.cls));
    if (d.cls == 1 && d.size != 4 && d.size != 8) throw FormatError("dataset '" + name + "': float size");
    if (d.cls == 0 && d.size != 1 && d.size != 2 && d.size != 4 && d.size != 8)
      throw FormatError("dataset '" + name + "': integer size");
    for (int id : d.filters)
      if (id != 1 && id != 2 && id != 3) throw FormatError("dataset '" + name + "': filter " + std::to_string(id));
    return d;
  }

  void layout(const uint8_t* p, size_t n, Dataset& d) const {
    const int ver = p[0];
    if (ver == 1 || ver == 2) {
      const int rank = p[1];
      d.layout = p[2];
      size_t o = 8;
      if (d.layout != 0) {
        d.addr = addr(p + o);
        o += so_;
      }
      if (d.layout == 1) d.bytes = kUndef;  // not recorded: the extent decides
      std::vector<uint64_t> dd;
      for (int i = 0; i < rank; ++i) dd.push_back(le(p + o + 4 * (size_t)i, 4));
      o += 4 * (size_t)rank;
      if (d.layout == 2) {
        d.chunk.assign(dd.begin(), dd.end() - 1);
      } else if (d.layout == 0) {
        d.bytes = le(p + o, 4);
        d.compact = p + o + 4;
      }
      return;
    }
    if (ver != 3 && ver != 4) throw FormatError("data layout version " + std::to_string(ver));
    d.layout = p[1];
    if (d.layout == 0) {
      d.bytes = le(p + 2, 2);
      d.compact = p + 4;
    } else if (d.layout == 1) {
      d.addr = addr(p + 2);
      d.bytes = le(p + 2 + so_, sl_);
    } else if (d.layout == 2 && ver == 3) {
      const int rank = p[2];
      d.addr = addr(p + 3);
      for (int i = 0; i + 1 < rank; ++i) d.chunk.push_back(le(p + 3 + so_ + 4 * (size_t)i, 4));
    } else if (d.layout == 2) {
      const int flags = p[2], rank = p[3], w = p[4];
      size_t o = 5;
      for (int i = 0; i + 1 < rank; ++i) d.chunk.push_back(le(p + o + (size_t)i * w, w));
      o += (size_t)rank * w;
      const int index = p[o++];
      if (index != 1) throw FormatError("chunk index type " + std::to_string(index) + " (only a single chunk)");
      d.chunk_index = 1;
      if (flags & 2) {
        d.single_size = le(p + o, sl_);
        d.single_mask = (uint32_t)le(p + o + sl_, 4);
        o += sl_ + 4;
      }
      d.addr = addr(p + o);
    } else {
      throw FormatError("layout class " + std::to_string(d.layout));
    }
    (void)n;
  }

  static uint64_t count(const std::vector<uint64_t>& dims) {
    uint64_t c = 1;
    for (uint64_t x : dims) c *= x;
    return c;
  }

  double element(const uint8_t* e, const Dataset& d) const {
    uint8_t b[8];
    for (int i = 0; i < d.size; ++i) b[i] = e[d.big ? d.size - 1 - i : i];
    if (d.cls == 1) {
      if (d.size == 4) {
        float f;
        std::memcpy(&f, b, 4);
        return (double)f;
      }
      double v;
      std::memcpy(&v, b, 8);
      return v;
    }
    const uint64_t u = le(b, d.size);
    if (!d.sign) return (double)u;
    const int sh = 64 - 8 * d.size;
    return (double)((int64_t)(u << sh) >> sh);
  }

  // raw chunk bytes through the filter pipeline (reversed), `expect` bytes
  std::vector<uint8_t> unfilter(const uint8_t* p, uint64_t n, uint32_t mask, const Dataset& d,
                                uint64_t expect) const {
    std::vector<uint8_t> v(p, p + n);
    for (int i = (int)d.filters.size() - 1; i >= 0; --i) {
      if (mask & (1u << i)) continue;
      const int id = d.filters[i];
      if (id == 1) {
        v = Inflater(v.data(), v.size()).zlib(expect);
      } else if (id == 2) {
        const size_t es = (size_t)d.size, ne = v.size() / es;
        std::vector<uint8_t> o(v.size());
        for (size_t k = 0; k < es; ++k)
          for (size_t e = 0; e < ne; ++e) o[e * es + k] = v[k * ne + e];
        std::copy(v.begin() + ne * es, v.end(), o.begin() + ne * es);
        v.swap(o);
      } else if (id == 3) {
        if (v.size() < 4) throw FormatError("Fletcher-32 chunk too short");
        v.resize(v.size() - 4);
      }
    }
    if (v.size() < expect) throw FormatError("chunk shorter than its extent");
    return v;
  }

  // copies a decoded chunk at element offsets `origin` into out (row-major)
  void place(const std::vector<uint8_t>& c, const std::vector<uint64_t>& origin, const Dataset& d,
             std::vector<double>& out) const {
    const size_t rank = d.dims.size();
    const uint64_t total = count(d.chunk);
    std::vector<uint64_t> idx(rank, 0);
    for (uint64_t k = 0; k < total; ++k) {
      uint64_t lin = 0;
      bool in = true;
      for (size_t a = 0; a < rank; ++a) {
        const uint64_t g = origin[a] + idx[a];
        if (g >= d.dims[a]) in = false;
        lin = lin * d.dims[a] + g;
      }
      if (in) out[lin] = element(c.data() + k * d.size, d);
      for (size_t a = rank; a-- > 0;) {
        if (++idx[a] < d.chunk[a]) break;
        idx[a] = 0;
      }
    }
  }

  void chunk_tree(uint64_t node, const Dataset& d, std::vector<double>& out) const {
    const size_t rank = d.dims.size();
    const uint8_t* p = at(node, 8 + 2 * (uint64_t)so_);
    if (std::memcmp(p, "TREE", 4) != 0 || p[4] != 1) throw FormatError("bad chunk B-tree node");
    const int level = p[5];
    const int used = (int)le(p + 6, 2);
    const uint64_t ksz = 8 + 8 * (uint64_t)(rank + 1);
    uint64_t o = node + 8 + 2 * so_;
    const uint64_t expect = count(d.chunk) * d.size;
    for (int i = 0; i < used; ++i) {
      const uint8_t* key = at(o, ksz + so_);
      const uint64_t size = le(key, 4);
      const uint32_t mask = (uint32_t)le(key + 4, 4);
      std::vector<uint64_t> origin(rank);
      for (size_t a = 0; a < rank; ++a) origin[a] = le(key + 8 + 8 * a, 8);
      const uint64_t child = addr(key + ksz);
      if (level > 0) {
        chunk_tree(child, d, out);
      } else {
        place(unfilter(at(child, size), size, mask, d, expect), origin, d, out);
      }
      o += ksz + so_;
    }
  }

  std::vector<double> values(const Dataset& d) const {
    const uint64_t n = count(d.dims);
    std::vector<double> out(n, 0.0);  // unwritten chunks read as the fill value 0
    if (n == 0) return out;
    if (d.layout == 0 || d.layout == 1) {
      if (d.layout == 1 && d.addr == kUndef) return out;
      if (d.bytes < n * d.size) throw FormatError("dataset storage shorter than its extent");
      const uint8_t* p = d.layout == 0 ? d.compact : at(d.addr, n * d.size);
      for (uint64_t i = 0; i < n; ++i) out[i] = element(p + i * d.size, d);
      return out;
    }
    if (d.chunk.size() != d.dims.size()) throw FormatError("chunk rank differs from the dataspace rank");
    if (d.addr == kUndef) return out;
    if (d.chunk_index == 1) {
      const uint64_t expect = count(d.chunk) * d.size;
      const uint64_t size = d.filters.empty() ? expect : d.single_size;
      place(unfilter(at(d.addr, size), size, d.single_mask, d, expect), std::vector<uint64_t>(d.dims.size(), 0), d,
            out);
    } else {
      chunk_tree(d.addr, d, out);
    }
    return out;
  }
};

// ---------------------------------------------------------------------------
// XML, as much as an XDMF frame list needs: elements, attributes (skipped),
// character data with the predefined and numeric entities, CDATA, comments,
// processing instructions and a DOCTYPE; line ends normalised to '\n';
// whitespace-only character data dropped and other character data kept as
// written (pugixml's default parse, which the reference uses).
// ---------------------------------------------------------------------------
struct XNode {
  std::string name;
  std::vector<XNode> kids;
  std::vector<std::string> text;  // character data children, in order
  const XNode* child(const std::string& n) const {
    for (const XNode& k : kids)
      if (k.name == n) return &k;
    return nullptr;
  }
};

class Xml {
 public:
  explicit Xml(std::string s) {
    for (size_t i = 0; i < s.size(); ++i)
      if (s[i] == '\r') {
        if (i + 1 < s.size() && s[i + 1] == '\n')
          s.erase(i, 1);
        else
          s[i] = '\n';
      }
    s_ = std::move(s);
    root_.name = "#document";
    parse_children(root_, "");
  }
  const XNode& root() const { return root_; }

 private:
  std::string s_;
  size_t i_ = 0;
  XNode root_;

  [[noreturn]] static void bad(const char* what) { throw std::invalid_argument(std::string("xdmf: ") + what); }

  bool starts(const char* t) const { return s_.compare(i_, std::strlen(t), t) == 0; }

  void skip_past(const char* t) {
    const size_t e = s_.find(t, i_);
    if (e == std::string::npos) bad("unterminated markup");
    i_ = e + std::strlen(t);
  }

  static bool blank(const std::string& t) {
    for (char c : t)
      if (c != ' ' && c != '\t' && c != '\n') return false;
    return true;
  }

  static std::string unescape(const std::string& t) {
    std::string o;
    for (size_t k = 0; k < t.size(); ++k) {
      if (t[k] != '&') {
        o += t[k];
        continue;
      }
      const size_t e = t.find(';', k);
      if (e == std::string::npos) {
        o += t[k];
        continue;
      }
      const std::string ent = t.substr(k + 1, e - k - 1);
      unsigned long cp = 0;
      bool ok = true;
      if (ent == "lt") cp = '<';
      else if (ent == "gt") cp = '>';
      else if (ent == "amp") cp = '&';
      else if (ent == "apos") cp = '\'';
      else if (ent == "quot") cp = '"';
      else if (ent.size() > 1 && ent[0] == '#') cp = ent[1] == 'x' ? std::strtoul(ent.c_str() + 2, nullptr, 16)
                                                                   : std::strtoul(ent.c_str() + 1, nullptr, 10);
      else ok = false;
      if (!ok) {
        o += t[k];
        continue;
      }
      if (cp < 0x80) {
        o += (char)cp;
      } else if (cp < 0x800) {
        o += (char)(0xC0 | (cp >> 6));
        o += (char)(0x80 | (cp & 0x3F));
      } else if (cp < 0x10000) {
        o += (char)(0xE0 | (cp >> 12));
        o += (char)(0x80 | ((cp >> 6) & 0x3F));
        o += (char)(0x80 | (cp & 0x3F));
      } else {
        o += (char)(0xF0 | (cp >> 18));
        o += (char)(0x80 | ((cp >> 12) & 0x3F));
        o += (char)(0x80 | ((cp >> 6) & 0x3F));
        o += (char)(0x80 | (cp & 0x3F));
      }
      k = e;
    }
    return o;
  }

  void parse_children(XNode& parent, const std::string& close) {
    while (i_ < s_.size()) {
      if (s_[i_] != '<') {
        const size_t e = s_.find('<', i_);
        const std::string t = s_.substr(i_, e == std::string::npos ? std::string::npos : e - i_);
        i_ = e == std::string::npos ? s_.size() : e;
        if (!blank(t)) parent.text.push_back(unescape(t));
        continue;
      }
      if (starts("<!--")) {
        skip_past("-->");
      } else if (starts("<![CDATA[")) {
        i_ += 9;
        const size_t e = s_.find("]]>", i_);
        if (e == std::string::npos) bad("unterminated CDATA");
        parent.text.push_back(s_.substr(i_, e - i_));
        i_ = e + 3;
      } else if (starts("<?")) {
        skip_past("?>");
      } else if (starts("<!")) {
        skip_past(">");
      } else if (starts("</")) {
        const size_t e = s_.find('>', i_);
        if (e == std::string::npos) bad("unterminated end tag");
        std::string name = s_.substr(i_ + 2, e - i_ - 2);
        while (!name.empty() && (name.back() == ' ' || name.back() == '\t' || name.back() == '\n')) name.pop_back();
        if (name != close) bad("mismatched end tag");
        i_ = e + 1;
        return;
      } else {
        size_t k = i_ + 1;
        while (k < s_.size() && !std::strchr(" \t\n/>", s_[k])) ++k;
        XNode node;
        node.name = s_.substr(i_ + 1, k - i_ - 1);
        // attributes: skipped, quotes respected
        char q = 0;
        while (k < s_.size() && (q || s_[k] != '>')) {
          if (q) {
            if (s_[k] == q) q = 0;
          } else if (s_[k] == '"' || s_[k] == '\'') {
            q = s_[k];
          }
          ++k;
        }
        if (k >= s_.size()) bad("unterminated start tag");
        const bool empty = s_[k - 1] == '/';
        i_ = k + 1;
        if (!empty) parse_children(node, node.name);
        parent.kids.push_back(std::move(node));
      }
    }
    if (!close.empty()) bad("unterminated element");
  }
};

}  // namespace

long long load_hdf5(const char* path, float* xyz, float* radius, long long cap, bool want_radius,
                    long long* n_out) {
  H5 h(path);
  std::vector<uint64_t> dims;
  const std::vector<double> pos = h.read("position", &dims);
  // the reference sizes the frame from the first dimension divided by 3 and
  // reads all values (a flat 3N array); an (N, 3) array is taken as N rows
  const long long n = dims.size() == 2 && dims[1] == 3 ? (long long)dims[0]
                                                       : (dims.empty() ? 0 : (long long)(dims[0] / 3));
  std::vector<double> rad;
  if (want_radius) {
    rad = h.read("particleRadius", nullptr);
    if ((long long)rad.size() < n) throw std::invalid_argument("hdf5 particleRadius holds fewer values than particles");
  }
  *n_out = n;
  if (!xyz) return n;
  if (n > cap) throw std::length_error("particle buffer too small");
  for (long long i = 0; i < 3 * n; ++i) xyz[i] = (float)pos[(size_t)i];
  if (want_radius && radius)
    for (long long i = 0; i < n; ++i) radius[i] = (float)rad[(size_t)i];
  return n;
}

std::vector<double> load_hdf5_dataset(const char* path, const char* name, std::vector<uint64_t>* dims) {
  H5 h(path);
  return h.read(name, dims);
}

std::vector<std::string> load_xdmf(const char* dir, const char* file, int target_frame) {
  const std::string p = std::string(dir) + "/" + file;
  std::ifstream f(p, std::ios::binary);
  if (!f) throw std::invalid_argument("cannot find xdmf file: " + p);
  std::string s((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  Xml x(std::move(s));
  std::vector<std::string> out;
  const XNode* xd = x.root().child("Xdmf");
  const XNode* dom = xd ? xd->child("Domain") : nullptr;
  const XNode* grid = dom ? dom->child("Grid") : nullptr;
  if (!grid) return out;
  int nframes = 0;
  for (const XNode& k : grid->kids)
    if (k.name == "Grid") ++nframes;
  int index = 0;
  for (const XNode& k : grid->kids) {
    if (k.name != "Grid") continue;
    ++index;
    const XNode* geo = k.child("Geometry");
    const XNode* item = geo ? geo->child("DataItem") : nullptr;
    std::string v = item && !item->text.empty() ? item->text[0] : std::string();
    v = v.substr(0, v.find_first_of(':'));
    if (target_frame > 0 && target_frame <= nframes) {
      if (target_frame == index) out.push_back(v);
    } else {
      out.push_back(v);
    }
  }
  return out;
}

}  // namespace pisurf
