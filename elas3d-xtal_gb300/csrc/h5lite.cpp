// Minimal HDF5 reader / writer (see h5lite.h).  Every structure below follows
// the HDF5 file-format specification, section by section: superblock (format
// signature, version 0 or 1), symbol-table entries, version-1 object headers
// and their messages (dataspace 0x0001, datatype 0x0003, fill value 0x0005,
// data layout 0x0008, attribute 0x000C, continuation 0x0010, symbol table
// 0x0011), the version-1 B-tree of a group (node type 0), local heaps and
// symbol-table nodes.  Host code only: no HDF5 library is involved.
#include "h5lite.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <limits>

namespace h5lite {

namespace {

constexpr uint64_t kUndef = ~0ull;
constexpr uint8_t kSig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
constexpr int kLeafK = 4;       // symbols per symbol-table node: 2K
constexpr int kInternalK = 16;  // children per group B-tree node: 2K

uint64_t pad8(uint64_t n) { return (n + 7) & ~7ull; }

// Little-endian byte sink with random-access patching.
struct Buf {
  std::vector<uint8_t> b;
  uint64_t size() const { return b.size(); }
  void u8(uint64_t v) { b.push_back((uint8_t)v); }
  void le(uint64_t v, int n) {
    for (int i = 0; i < n; ++i) b.push_back((uint8_t)(v >> (8 * i)));
  }
  void bytes(const void* p, size_t n) {
    const uint8_t* q = static_cast<const uint8_t*>(p);
    b.insert(b.end(), q, q + n);
  }
  void zeros(uint64_t n) { b.insert(b.end(), (size_t)n, 0); }
  void align8() { zeros(pad8(size()) - size()); }
  void put(uint64_t at, uint64_t v, int n) {
    for (int i = 0; i < n; ++i) b[(size_t)at + i] = (uint8_t)(v >> (8 * i));
  }
};

// Datatype message body (version 1) of a little-endian int32 or IEEE float64,
// padded to eight bytes; returns the unpadded length.
int datatype_body(Buf& o, Type t) {
  const uint64_t start = o.size();
  if (t == Type::I32) {
    o.u8(0x10);  // version 1, class 0 (fixed-point)
    o.u8(0x08);  // little endian, zero padding, signed
    o.u8(0);
    o.u8(0);
    o.le(4, 4);   // size
    o.le(0, 2);   // bit offset
    o.le(32, 2);  // bit precision
  } else {
    o.u8(0x11);  // version 1, class 1 (floating-point)
    o.u8(0x20);  // little endian, mantissa normalised with an implied leading 1
    o.u8(63);    // sign bit
    o.u8(0);
    o.le(8, 4);     // size
    o.le(0, 2);     // bit offset
    o.le(64, 2);    // bit precision
    o.u8(52);       // exponent location
    o.u8(11);       // exponent size
    o.u8(0);        // mantissa location
    o.u8(52);       // mantissa size
    o.le(1023, 4);  // exponent bias
  }
  const int len = (int)(o.size() - start);
  o.align8();
  return len;
}

// Dataspace message body (version 1, simple); returns its length (a multiple of 8).
int dataspace_body(Buf& o, const std::vector<uint64_t>& dims) {
  o.u8(1);
  o.u8((uint8_t)dims.size());
  o.u8(0);  // no maximum dimensions
  o.u8(0);
  o.le(0, 4);
  for (uint64_t d : dims) o.le(d, 8);
  return 8 + 8 * (int)dims.size();
}

struct Msg {
  uint16_t type;
  uint8_t flags;
  std::vector<uint8_t> body;  // padded to eight bytes
};

// Object header (version 1) with the given messages at o's end; returns its address.
uint64_t object_header(Buf& o, const std::vector<Msg>& msgs) {
  o.align8();
  const uint64_t at = o.size();
  uint64_t body = 0;
  for (const Msg& m : msgs) body += 8 + m.body.size();
  o.u8(1);  // version
  o.u8(0);
  o.le(msgs.size(), 2);
  o.le(1, 4);  // reference count
  o.le(body, 4);
  o.zeros(4);  // messages start eight-byte aligned
  for (const Msg& m : msgs) {
    o.le(m.type, 2);
    o.le(m.body.size(), 2);
    o.u8(m.flags);
    o.zeros(3);
    o.bytes(m.body.data(), m.body.size());
  }
  return at;
}

}  // namespace

int write_file(const std::string& path, const std::vector<DatasetOut>& sets_in) {
  std::vector<DatasetOut> sets = sets_in;
  std::sort(sets.begin(), sets.end(), [](const DatasetOut& a, const DatasetOut& b) { return a.name < b.name; });
  if (sets.size() > (size_t)(2 * kLeafK)) return -1;  // one symbol-table node holds them all
  Buf o;
  // ---- superblock, version 0 (addresses patched below)
  o.bytes(kSig, 8);
  o.u8(0);  // superblock version
  o.u8(0);  // free-space storage version
  o.u8(0);  // root group symbol table entry version
  o.u8(0);
  o.u8(0);  // shared header message format version
  o.u8(8);  // size of offsets
  o.u8(8);  // size of lengths
  o.u8(0);
  o.le(kLeafK, 2);
  o.le(kInternalK, 2);
  o.le(0, 4);  // file consistency flags
  o.le(0, 8);  // base address
  o.le(kUndef, 8);  // free-space info
  const uint64_t at_eof = o.size();
  o.le(0, 8);       // end of file address (patched)
  o.le(kUndef, 8);  // driver information block
  // root group symbol table entry
  o.le(0, 8);  // link name offset
  const uint64_t at_root_oh = o.size();
  o.le(0, 8);  // object header address (patched)
  o.le(1, 4);  // cache type 1: the scratch pad holds the B-tree and heap addresses
  o.le(0, 4);
  const uint64_t at_scratch = o.size();
  o.le(0, 8);
  o.le(0, 8);
  // ---- root group object header: symbol table message
  Msg stab{0x0011, 0, std::vector<uint8_t>(16, 0)};
  const uint64_t root_oh = object_header(o, {stab});
  const uint64_t at_stab = root_oh + 16 + 8;  // body of the only message
  o.put(at_root_oh, root_oh, 8);
  // ---- local heap with the link names ("" at offset 0)
  Buf names;
  names.zeros(8);
  std::vector<uint64_t> name_off;
  for (const DatasetOut& d : sets) {
    name_off.push_back(names.size());
    names.bytes(d.name.c_str(), d.name.size() + 1);
    names.align8();
  }
  o.align8();
  const uint64_t heap = o.size();
  o.bytes("HEAP", 4);
  o.u8(0);
  o.zeros(3);
  o.le(names.size(), 8);
  o.le(kUndef, 8);  // no free block
  o.le(heap + 32, 8);
  o.bytes(names.b.data(), names.size());
  // ---- group B-tree: one leaf-level node pointing at one symbol-table node
  o.align8();
  const uint64_t btree = o.size();
  o.bytes("TREE", 4);
  o.u8(0);  // group node
  o.u8(0);  // level 0
  o.le(sets.empty() ? 0 : 1, 2);
  o.le(kUndef, 8);
  o.le(kUndef, 8);
  const uint64_t at_keys = o.size();
  o.zeros((2 * kInternalK + 1) * 8 + 2 * kInternalK * 8);
  // ---- symbol-table node (entries patched once the datasets are placed)
  o.align8();
  const uint64_t snod = o.size();
  o.bytes("SNOD", 4);
  o.u8(1);
  o.u8(0);
  o.le(sets.size(), 2);
  const uint64_t at_entries = o.size();
  o.zeros(2 * kLeafK * 40);
  if (!sets.empty()) {
    o.put(at_keys, 0, 8);                          // key 0: "" (below every name)
    o.put(at_keys + 8, snod, 8);                   // child 0
    o.put(at_keys + 16, name_off.back(), 8);       // key 1: the largest name in the child
  }
  o.put(at_scratch, btree, 8);
  o.put(at_scratch + 8, heap, 8);
  o.put(at_stab, btree, 8);
  o.put(at_stab + 8, heap, 8);
  // ---- datasets
  for (size_t i = 0; i < sets.size(); ++i) {
    const DatasetOut& d = sets[i];
    uint64_t count = 1;
    for (uint64_t v : d.dims) count *= v;
    const uint64_t esz = d.type == Type::I32 ? 4 : 8;
    std::vector<Msg> msgs;
    {
      Buf b;
      dataspace_body(b, d.dims);
      msgs.push_back({0x0001, 0, b.b});
    }
    {
      Buf b;
      datatype_body(b, d.type);
      msgs.push_back({0x0003, 1, b.b});  // constant
    }
    {
      Buf b;  // fill value, version 2: allocated late, written if set, none defined
      b.u8(2);
      b.u8(2);
      b.u8(2);
      b.u8(0);
      b.align8();
      msgs.push_back({0x0005, 1, b.b});
    }
    const size_t layout_idx = msgs.size();
    {
      Buf b;  // data layout, version 3, contiguous (address patched)
      b.u8(3);
      b.u8(1);
      b.le(0, 8);
      b.le(count * esz, 8);
      b.align8();
      msgs.push_back({0x0008, 0, b.b});
    }
    if (!d.attr_name.empty()) {
      Buf b;  // attribute, version 1: name, datatype, dataspace, data
      Buf t, s;
      const int tlen = datatype_body(t, Type::I32);
      const int slen = dataspace_body(s, {(uint64_t)d.attr.size()});
      b.u8(1);
      b.u8(0);
      b.le(d.attr_name.size() + 1, 2);
      b.le(tlen, 2);
      b.le(slen, 2);
      b.bytes(d.attr_name.c_str(), d.attr_name.size() + 1);
      b.align8();
      b.bytes(t.b.data(), t.size());
      b.bytes(s.b.data(), s.size());
      for (int32_t v : d.attr) b.le((uint32_t)v, 4);
      b.align8();
      msgs.push_back({0x000C, 0, b.b});
    }
    const uint64_t oh = object_header(o, msgs);
    // the layout message's address field: header prefix, earlier messages, message header, version + class
    uint64_t at_addr = oh + 16;
    for (size_t m = 0; m < layout_idx; ++m) at_addr += 8 + msgs[m].body.size();
    at_addr += 8 + 2;
    o.align8();
    const uint64_t data = o.size();
    o.put(at_addr, data, 8);
    o.bytes(d.data, count * esz);
    // symbol table entry
    const uint64_t e = at_entries + 40 * i;
    o.put(e, name_off[i], 8);
    o.put(e + 8, oh, 8);
  }
  o.put(at_eof, o.size(), 8);
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) return -1;
  const bool ok = std::fwrite(o.b.data(), 1, o.b.size(), f) == o.b.size();
  return (std::fclose(f) == 0 && ok) ? 0 : -1;
}

// ============================================================== reader

Reader::Reader(const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) {
    io_error_ = true;
    fail("cannot open " + path);
    return;
  }
  std::fseek(f, 0, SEEK_END);
  const long n = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  if (n > 0) {
    file_.resize((size_t)n);
    if (std::fread(file_.data(), 1, (size_t)n, f) != (size_t)n) file_.clear();
  }
  std::fclose(f);
  if (file_.empty()) {
    io_error_ = true;
    fail("cannot read " + path);
    return;
  }
  ok_ = parse_superblock();
}

bool Reader::fail(const std::string& why) {
  if (err_.empty()) err_ = why;
  return false;
}

bool Reader::rd(uint64_t addr, void* dst, uint64_t n) {
  const uint64_t a = base_ + addr;
  if (addr == kUndef || a < base_ || a > file_.size() || n > file_.size() - a)
    return fail("address outside the file");
  std::memcpy(dst, file_.data() + a, (size_t)n);
  return true;
}

uint64_t Reader::u(const uint8_t* p, int nbytes) const {
  uint64_t v = 0;
  for (int i = 0; i < nbytes; ++i) v |= (uint64_t)p[i] << (8 * i);
  // an address of all ones is the undefined address, whatever its width
  if (nbytes == so_ && nbytes < 8 && v == ((1ull << (8 * nbytes)) - 1)) return kUndef;
  return v;
}

bool Reader::parse_superblock() {
  // The signature sits at 0 or after a user block of 512, 1024, 2048, ... bytes.
  uint64_t at = kUndef;
  for (uint64_t off = 0; off + 8 <= file_.size(); off = off ? off * 2 : 512)
    if (std::memcmp(file_.data() + off, kSig, 8) == 0) {
      at = off;
      break;
    }
  if (at == kUndef) return fail("not an HDF5 file (no format signature)");
  base_ = at;
  uint8_t h[24];
  if (!rd(0, h, sizeof h)) return false;
  const int ver = h[8];
  if (ver > 1) return fail("superblock version " + std::to_string(ver) + " is not supported (versions 0 and 1 are)");
  so_ = h[13];
  sl_ = h[14];
  if ((so_ != 4 && so_ != 8) || (sl_ != 4 && sl_ != 8)) return fail("unsupported address or length size");
  uint64_t p = 24 + (ver == 1 ? 4 : 0);
  p += 4 * (uint64_t)so_;  // base, free-space, end of file and driver addresses
  // root group symbol table entry
  std::vector<uint8_t> e(2 * so_ + 24);
  if (!rd(p, e.data(), e.size())) return false;
  const uint64_t root_oh = u(e.data() + so_, so_);
  const uint32_t cache = (uint32_t)u(e.data() + 2 * so_, 4);
  uint64_t btree = kUndef, heap = kUndef;
  if (cache == 1) {
    btree = u(e.data() + 2 * so_ + 8, so_);
    heap = u(e.data() + 2 * so_ + 8 + so_, so_);
  } else {
    DatasetInfo dummy;  // the root group's own header carries the symbol table message
    uint8_t pre[16];
    if (!rd(root_oh, pre, 16)) return false;
    if (pre[0] != 1) return fail("root group: object header version " + std::to_string(pre[0]) + " is not supported");
    const uint64_t len = u(pre + 8, 4);
    std::vector<uint8_t> body(len);
    if (!rd(root_oh + 16, body.data(), len)) return false;
    for (uint64_t q = 0; q + 8 <= len;) {
      const uint16_t type = (uint16_t)u(body.data() + q, 2);
      const uint16_t sz = (uint16_t)u(body.data() + q + 2, 2);
      if (q + 8 + sz > len) break;
      if (type == 0x0011) {
        btree = u(body.data() + q + 8, so_);
        heap = u(body.data() + q + 8 + so_, so_);
      }
      q += 8 + sz;
    }
  }
  if (btree == kUndef || heap == kUndef) return fail("root group has no symbol table");
  std::vector<uint8_t> hh(8 + 2 * sl_ + so_);
  if (!rd(heap, hh.data(), hh.size())) return false;
  if (std::memcmp(hh.data(), "HEAP", 4) != 0) return fail("bad local heap signature");
  const uint64_t heap_data = u(hh.data() + 8 + 2 * sl_, so_);
  return walk_btree(btree, heap_data, 0);
}

bool Reader::walk_btree(uint64_t addr, uint64_t heap_data, int depth) {
  if (depth > 32) return fail("group B-tree too deep");
  std::vector<uint8_t> h(8 + 2 * so_);
  if (!rd(addr, h.data(), h.size())) return false;
  if (std::memcmp(h.data(), "TREE", 4) != 0) return fail("bad B-tree signature");
  if (h[4] != 0) return fail("not a group B-tree node");
  const int level = h[5];
  const int used = (int)u(h.data() + 6, 2);
  const uint64_t kv = 8 + 2 * (uint64_t)so_;  // keys and children follow the siblings
  for (int i = 0; i < used; ++i) {
    uint8_t c[8];
    if (!rd(addr + kv + sl_ + (uint64_t)i * (sl_ + so_), c, so_)) return false;
    const uint64_t child = u(c, so_);
    if (level > 0) {
      if (!walk_btree(child, heap_data, depth + 1)) return false;
      continue;
    }
    uint8_t sh[8];
    if (!rd(child, sh, 8)) return false;
    if (std::memcmp(sh, "SNOD", 4) != 0) return fail("bad symbol-table node signature");
    const int nsym = (int)u(sh + 6, 2);
    const uint64_t esz = 2 * (uint64_t)so_ + 24;
    for (int s = 0; s < nsym; ++s) {
      std::vector<uint8_t> e(esz);
      if (!rd(child + 8 + s * esz, e.data(), esz)) return false;
      const uint64_t noff = u(e.data(), so_);
      const uint64_t oh = u(e.data() + so_, so_);
      std::string name;
      for (uint64_t q = heap_data + noff;; ++q) {
        char ch;
        if (!rd(q, &ch, 1)) return false;
        if (!ch) break;
        name.push_back(ch);
        if (name.size() > 4096) return fail("link name too long");
      }
      links_.emplace_back(name, oh);
    }
  }
  return true;
}

std::vector<std::string> Reader::names() const {
  std::vector<std::string> out;
  for (const auto& l : links_) out.push_back(l.first);
  return out;
}

namespace {

// Datatype message: class, size, byte order, sign.
bool parse_datatype(const uint8_t* p, uint64_t len, DatasetInfo& d) {
  if (len < 8) return false;
  d.klass = p[0] & 0x0f;
  d.size = (int)(p[4] | (p[5] << 8) | (p[6] << 16) | ((uint32_t)p[7] << 24));
  if (d.klass == 0) {
    d.big_endian = (p[1] & 0x01) != 0;
    d.is_signed = (p[1] & 0x08) != 0;
    return d.size == 1 || d.size == 2 || d.size == 4 || d.size == 8;
  }
  if (d.klass == 1) {
    if (p[1] & 0x40) return false;  // VAX byte order
    d.big_endian = (p[1] & 0x01) != 0;
    return d.size == 4 || d.size == 8;
  }
  return false;
}

}  // namespace

bool Reader::parse_messages(const uint8_t* p, uint64_t len, DatasetInfo& d,
                            std::vector<std::pair<uint64_t, uint64_t>>& cont, bool& have_space, bool& have_type,
                            bool& have_layout) {
  for (uint64_t q = 0; q + 8 <= len;) {
    const uint16_t type = (uint16_t)u(p + q, 2);
    const uint16_t sz = (uint16_t)u(p + q + 2, 2);
    const uint8_t flags = p[q + 4];
    const uint8_t* m = p + q + 8;
    if (q + 8 + sz > len) return fail("object header message runs past its block");
    if ((flags & 0x02) && (type == 0x0001 || type == 0x0003)) return fail("shared dataspace or datatype messages are not supported");
    if (type == 0x0001) {  // dataspace
      const int ver = m[0], nd = m[1];
      if (ver != 1 && ver != 2) return fail("dataspace version " + std::to_string(ver));
      if (ver == 2 && m[3] == 2) return fail("null dataspace");
      const uint64_t off = ver == 1 ? 8 : 4;  // a scalar (version 2, type 0) has no dimensions
      if (off + (uint64_t)nd * sl_ > sz) return fail("dataspace message too short");
      d.dims.clear();
      for (int i = 0; i < nd; ++i) d.dims.push_back(u(m + off + (uint64_t)i * sl_, sl_));
      have_space = true;
    } else if (type == 0x0003) {
      if (!parse_datatype(m, sz, d)) return fail("unsupported element type");
      have_type = true;
    } else if (type == 0x0008) {  // data layout
      const int ver = m[0];
      if (ver == 3 || ver == 4) {
        const int cls = m[1];
        if (cls == 0) {
          const uint64_t n = u(m + 2, 2);
          if (4 + n > sz) return fail("compact data runs past its message");
          d.layout = 0;
          d.nbytes = n;
          d.compact.assign(m + 4, m + 4 + n);
        } else if (cls == 1) {
          if (2 + (uint64_t)so_ + sl_ > sz) return fail("data layout message too short");
          d.layout = 1;
          d.addr = u(m + 2, so_);
          d.nbytes = u(m + 2 + so_, sl_);
        } else {
          return fail("chunked or virtual storage is not supported");
        }
      } else if (ver == 1 || ver == 2) {
        const int nd = m[1], cls = m[2];
        uint64_t off = 8;
        if (off + so_ + 4 * (uint64_t)nd + 4 > sz) return fail("data layout message too short");
        if (cls == 1) {
          d.layout = 1;
          d.addr = u(m + off, so_);
          off += so_;
          uint64_t n = 1;
          for (int i = 0; i < nd; ++i) n *= u(m + off + 4 * (uint64_t)i, 4);  // the last one is the element size
          d.nbytes = n;
        } else if (cls == 0) {
          off += 4 * (uint64_t)nd;
          const uint64_t n = u(m + off, 4);
          if (off + 4 + n > sz) return fail("compact data runs past its message");
          d.layout = 0;
          d.nbytes = n;
          d.compact.assign(m + off + 4, m + off + 4 + n);
        } else {
          return fail("chunked storage is not supported");
        }
      } else {
        return fail("data layout version " + std::to_string(ver));
      }
      have_layout = true;
    } else if (type == 0x000C && sz >= 8) {  // attribute: only the int32 "dimensions" is read
      const int ver = m[0];
      const uint64_t nl = u(m + 2, 2), tl = u(m + 4, 2), sl = u(m + 6, 2);
      const bool padded = ver == 1;
      uint64_t off = ver == 3 ? 9 : 8;
      const uint64_t at_name = off;
      off += padded ? pad8(nl) : nl;
      const uint64_t at_type = off;
      off += padded ? pad8(tl) : tl;
      const uint64_t at_space = off;
      off += padded ? pad8(sl) : sl;
      if (off > sz || nl < 1 || tl < 8 || sl < 4) {
        q += 8 + sz;
        continue;  // malformed or empty: skip it
      }
      const std::string name(reinterpret_cast<const char*>(m + at_name), nl - 1);
      DatasetInfo t;
      const bool tok = parse_datatype(m + at_type, tl, t);
      const uint8_t* s = m + at_space;
      if (name == "dimensions" && tok && t.klass == 0 && t.size == 4 && !t.big_endian && (s[0] == 1 || s[0] == 2)) {
        const int nd = s[1];
        uint64_t cnt = 1;
        const uint64_t soff = s[0] == 1 ? 8 : 4;
        const bool fits = soff + (uint64_t)nd * sl_ <= sl;
        for (int i = 0; fits && i < nd; ++i) cnt *= u(s + soff + (uint64_t)i * sl_, sl_);
        if (fits && cnt <= (sz - off) / 4) {
          d.dimensions_attr.clear();
          for (uint64_t i = 0; i < cnt; ++i) d.dimensions_attr.push_back((int32_t)u(m + off + 4 * i, 4));
        }
      }
    } else if (type == 0x0010) {  // continuation
      if ((uint64_t)so_ + sl_ > sz) return fail("continuation message too short");
      cont.emplace_back(u(m, so_), u(m + so_, sl_));
    }
    q += 8 + sz;
  }
  return true;
}

bool Reader::parse_object_header(uint64_t addr, DatasetInfo& d) {
  uint8_t pre[16];
  if (!rd(addr, pre, 16)) return false;
  if (pre[0] != 1) return fail("object header version " + std::to_string(pre[0]) + " is not supported");
  std::vector<std::pair<uint64_t, uint64_t>> blocks{{addr + 16, u(pre + 8, 4)}};
  bool hs = false, ht = false, hl = false;
  for (size_t i = 0; i < blocks.size(); ++i) {
    if (blocks.size() > 1024) return fail("too many object header blocks");
    std::vector<uint8_t> body(blocks[i].second);
    if (!rd(blocks[i].first, body.data(), body.size())) return false;
    if (!parse_messages(body.data(), body.size(), d, blocks, hs, ht, hl)) return false;
  }
  if (!hs || !ht || !hl) return fail("not a dataset (missing dataspace, datatype or layout)");
  return true;
}

bool Reader::info(const std::string& name, DatasetInfo& out) {
  if (!ok_) return false;
  for (const auto& l : links_)
    if (l.first == name) {
      out = DatasetInfo{};
      return parse_object_header(l.second, out);
    }
  return fail("no dataset named \"" + name + "\"");
}

bool Reader::raw(const DatasetInfo& d, std::vector<uint8_t>& bytes) {
  for (uint64_t v : d.dims)
    if (v > (1ull << 40)) return fail("dataspace too large");
  if (d.count() > (1ull << 40)) return fail("dataspace too large");
  const uint64_t need = d.count() * (uint64_t)d.size;
  if (d.layout == 0) {
    if (d.compact.size() < need) return fail("compact data shorter than the dataspace");
    bytes.assign(d.compact.begin(), d.compact.begin() + (size_t)need);
    return true;
  }
  if (d.addr == kUndef) {  // storage never allocated: the default fill value, zero
    bytes.assign((size_t)need, 0);
    return true;
  }
  if (d.nbytes < need) return fail("stored data shorter than the dataspace");
  bytes.resize((size_t)need);
  return rd(d.addr, bytes.data(), need);
}

namespace {

uint64_t load(const uint8_t* p, int n, bool be) {
  uint64_t v = 0;
  for (int i = 0; i < n; ++i) v |= (uint64_t)p[be ? n - 1 - i : i] << (8 * i);
  return v;
}

bool to_i64(const uint8_t* p, const DatasetInfo& d, long long& out) {
  const uint64_t v = load(p, d.size, d.big_endian);
  if (d.klass != 0) return false;
  if (d.is_signed) {
    const int sh = 64 - 8 * d.size;
    out = sh ? ((long long)(v << sh)) >> sh : (long long)v;
  } else {
    if (d.size == 8 && v > (uint64_t)std::numeric_limits<long long>::max()) return false;
    out = (long long)v;
  }
  return true;
}

double to_f64(const uint8_t* p, const DatasetInfo& d) {
  const uint64_t v = load(p, d.size, d.big_endian);
  if (d.klass == 1) {
    if (d.size == 8) {
      double x;
      std::memcpy(&x, &v, 8);
      return x;
    }
    const uint32_t w = (uint32_t)v;
    float x;
    std::memcpy(&x, &w, 4);
    return x;
  }
  long long i = 0;
  to_i64(p, d, i);
  return (double)i;
}

}  // namespace

bool Reader::read_i32(const std::string& name, int32_t* out, uint64_t n) {
  DatasetInfo d;
  if (!info(name, d)) return false;
  if (d.count() != n) return fail("\"" + name + "\" holds " + std::to_string(d.count()) + " values, not " + std::to_string(n));
  if (d.klass != 0) return fail("\"" + name + "\" is not an integer dataset");
  std::vector<uint8_t> b;
  if (!raw(d, b)) return false;
  for (uint64_t i = 0; i < n; ++i) {
    long long v = 0;
    if (!to_i64(b.data() + i * d.size, d, v) || v < std::numeric_limits<int32_t>::min() ||
        v > std::numeric_limits<int32_t>::max())
      return fail("\"" + name + "\" holds a value outside the int32 range");
    out[i] = (int32_t)v;
  }
  return true;
}

bool Reader::read_f64(const std::string& name, double* out, uint64_t n) {
  DatasetInfo d;
  if (!info(name, d)) return false;
  if (d.count() != n) return fail("\"" + name + "\" holds " + std::to_string(d.count()) + " values, not " + std::to_string(n));
  std::vector<uint8_t> b;
  if (!raw(d, b)) return false;
  for (uint64_t i = 0; i < n; ++i) out[i] = to_f64(b.data() + i * d.size, d);
  return true;
}

}  // namespace h5lite
