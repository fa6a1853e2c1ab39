// h5lite implementation. Structures and field orders follow the public HDF5 File Format
// Specification; see h5lite.h for the supported subset.
#include "h5lite.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>

namespace h5l {

static const uint64_t UNDEF = ~0ull;
static const uint8_t SIGNATURE[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
// Group B-tree ("internal node K") and symbol-table-node ("leaf node K") parameters written in
// the superblock: a B-tree node holds up to 2*IK children, a symbol table node 2*LK entries.
static const int LK = 4;
static const int IK = 16;
static const size_t SNOD_SIZE = 8 + 2 * LK * 40;
static const size_t BTREE_SIZE = 24 + 2 * IK * 8 + (2 * IK + 1) * 8;
// libhdf5 marks the end of a local heap's free list with the offset value 1.
static const uint64_t HEAP_FREE_NULL = 1;

size_t dtype_size(DType t) {
  switch (t) {
    case DType::F64: return 8;
    case DType::F32: return 4;
    case DType::U32: return 4;
    case DType::I32: return 4;
    case DType::U64: return 8;
    case DType::I64: return 8;
    case DType::U8: return 1;
  }
  return 0;
}

uint64_t DatasetInfo::nelem() const {
  uint64_t n = 1;
  for (auto d : dims) n *= d;
  return n;
}

// =============================================================================================
// Writer
// =============================================================================================
struct Writer::Node {
  bool is_group = true;
  std::map<std::string, std::unique_ptr<Node>> children;  // std::string order == strcmp order
  DType t = DType::F64;
  std::vector<uint64_t> dims;
  std::vector<uint8_t> data;
  const uint8_t* ext = nullptr;  // borrowed data (add_dataset_ref), ext_bytes long
  size_t ext_bytes = 0;
  size_t nbytes() const { return ext ? ext_bytes : data.size(); }
  const uint8_t* bytes() const { return ext ? ext : data.data(); }
};

Writer::Writer() : root_(new Node) {}
Writer::~Writer() {}

static std::vector<std::string> split_path(const std::string& p) {
  std::vector<std::string> out;
  std::string cur;
  for (char c : p) {
    if (c == '/') {
      if (!cur.empty()) out.push_back(cur);
      cur.clear();
    } else {
      cur.push_back(c);
    }
  }
  if (!cur.empty()) out.push_back(cur);
  return out;
}

Writer::Node* Writer::make_group(const std::string& path) {
  Node* n = root_.get();
  for (auto& part : split_path(path)) {
    auto it = n->children.find(part);
    if (it == n->children.end()) {
      it = n->children.emplace(part, std::unique_ptr<Node>(new Node)).first;
    }
    if (!it->second->is_group) return nullptr;
    n = it->second.get();
  }
  return n;
}

void Writer::create_group(const std::string& path) { make_group(path); }

bool Writer::add_dataset(const std::string& path, DType t, const std::vector<uint64_t>& dims,
                         const void* data) {
  return add(path, t, dims, data, true);
}

bool Writer::add_dataset_ref(const std::string& path, DType t, const std::vector<uint64_t>& dims,
                             const void* data) {
  return add(path, t, dims, data, false);
}

bool Writer::add(const std::string& path, DType t, const std::vector<uint64_t>& dims, const void* data,
                 bool copy) {
  auto parts = split_path(path);
  if (parts.empty()) return false;
  std::string leaf = parts.back();
  std::string parent;
  for (size_t i = 0; i + 1 < parts.size(); ++i) parent += "/" + parts[i];
  Node* g = make_group(parent);
  if (!g || g->children.count(leaf)) return false;
  std::unique_ptr<Node> d(new Node);
  d->is_group = false;
  d->t = t;
  d->dims = dims;
  uint64_t n = 1;
  for (auto x : dims) n *= x;
  size_t bytes = (size_t)n * dtype_size(t);
  if (copy || !bytes) {
    d->data.resize(bytes);
    if (bytes) std::memcpy(d->data.data(), data, bytes);
  } else {
    d->ext = static_cast<const uint8_t*>(data);
    d->ext_bytes = bytes;
  }
  g->children.emplace(leaf, std::move(d));
  return true;
}

namespace {
// The file image: metadata bytes in `b`, with the borrowed dataset bytes as holes that are only
// read when the file is written. pos() is the file offset; put64 patches the superblock, which
// precedes every hole.
struct Buf {
  struct Hole {
    size_t at;  // offset in b where the hole sits
    const uint8_t* p;
    size_t n;
  };
  std::vector<uint8_t> b;
  std::vector<Hole> holes;
  uint64_t skipped = 0;
  uint64_t pos() const { return b.size() + skipped; }
  void hole(const uint8_t* p, size_t n) {
    holes.push_back({b.size(), p, n});
    skipped += n;
  }
  void u8(uint8_t v) { b.push_back(v); }
  void u16(uint16_t v) { for (int i = 0; i < 2; ++i) b.push_back((v >> (8 * i)) & 0xff); }
  void u32(uint32_t v) { for (int i = 0; i < 4; ++i) b.push_back((v >> (8 * i)) & 0xff); }
  void u64(uint64_t v) { for (int i = 0; i < 8; ++i) b.push_back((v >> (8 * i)) & 0xff); }
  void bytes(const void* p, size_t n) {
    const uint8_t* c = (const uint8_t*)p;
    b.insert(b.end(), c, c + n);
  }
  void zeros(size_t n) { b.insert(b.end(), n, 0); }
  void pad8() { while (pos() % 8) b.push_back(0); }
  void put64(uint64_t at, uint64_t v) { for (int i = 0; i < 8; ++i) b[at + i] = (v >> (8 * i)) & 0xff; }
};

struct Msg {
  uint16_t type;
  uint8_t flags;
  std::vector<uint8_t> data;
};

// Object header version 1: 16-byte prefix, then messages with 8-byte headers and data padded
// to a multiple of 8 bytes.
uint64_t emit_ohdr_v1(Buf& B, const std::vector<Msg>& msgs) {
  uint64_t addr = B.pos();
  uint32_t size = 0;
  for (auto& m : msgs) size += 8 + (uint32_t)((m.data.size() + 7) / 8 * 8);
  B.u8(1);
  B.u8(0);
  B.u16((uint16_t)msgs.size());
  B.u32(1);
  B.u32(size);
  B.u32(0);
  for (auto& m : msgs) {
    size_t dsz = (m.data.size() + 7) / 8 * 8;
    B.u16(m.type);
    B.u16((uint16_t)dsz);
    B.u8(m.flags);
    B.zeros(3);
    B.bytes(m.data.data(), m.data.size());
    B.zeros(dsz - m.data.size());
  }
  return addr;
}

void le(std::vector<uint8_t>& v, uint64_t x, int n) {
  for (int i = 0; i < n; ++i) v.push_back((x >> (8 * i)) & 0xff);
}

Msg dataspace_msg(const std::vector<uint64_t>& dims) {
  Msg m{0x0001, 0, {}};
  m.data.push_back(1);                    // version
  m.data.push_back((uint8_t)dims.size()); // dimensionality
  m.data.push_back(0);                    // flags: no max dims
  m.data.push_back(0);                    // reserved
  le(m.data, 0, 4);                       // reserved
  for (auto d : dims) le(m.data, d, 8);
  return m;
}

Msg datatype_msg(DType t) {
  Msg m{0x0003, 1, {}};  // flag bit 0: constant message
  auto& d = m.data;
  if (t == DType::F64 || t == DType::F32) {
    bool dbl = (t == DType::F64);
    d.push_back(0x10 | 1);           // version 1, class floating point
    d.push_back(0x20);               // little endian, mantissa normalization: implied msb
    d.push_back(dbl ? 63 : 31);      // sign bit location
    d.push_back(0);
    le(d, dbl ? 8 : 4, 4);           // size
    le(d, 0, 2);                     // bit offset
    le(d, dbl ? 64 : 32, 2);         // bit precision
    d.push_back(dbl ? 52 : 23);      // exponent location
    d.push_back(dbl ? 11 : 8);       // exponent size
    d.push_back(0);                  // mantissa location
    d.push_back(dbl ? 52 : 23);      // mantissa size
    le(d, dbl ? 1023 : 127, 4);      // exponent bias
  } else {
    bool sgn = (t == DType::I32 || t == DType::I64);
    uint32_t sz = (uint32_t)dtype_size(t);
    d.push_back(0x10 | 0);           // version 1, class fixed point
    d.push_back(sgn ? 0x08 : 0x00);  // little endian, zero padding, signedness
    d.push_back(0);
    d.push_back(0);
    le(d, sz, 4);
    le(d, 0, 2);                     // bit offset
    le(d, sz * 8, 2);                // bit precision
  }
  return m;
}

Msg layout_msg(uint64_t addr, uint64_t size) {
  Msg m{0x0008, 0, {}};
  m.data.push_back(3);  // version 3
  m.data.push_back(1);  // contiguous
  le(m.data, addr, 8);
  le(m.data, size, 8);
  return m;
}

struct GroupRefs {
  uint64_t ohdr, btree, heap;
};

struct Emitter {
  Buf B;

  uint64_t emit_dataset(const Writer::Node& n) {
    uint64_t daddr = UNDEF;
    if (n.nbytes()) {
      B.pad8();
      daddr = B.pos();
      if (n.ext)
        B.hole(n.ext, n.ext_bytes);
      else
        B.bytes(n.data.data(), n.data.size());
    }
    B.pad8();
    std::vector<Msg> msgs;
    msgs.push_back(dataspace_msg(n.dims));
    msgs.push_back(datatype_msg(n.t));
    msgs.push_back(layout_msg(daddr, n.nbytes()));
    return emit_ohdr_v1(B, msgs);
  }

  GroupRefs emit_group(const Writer::Node& g) {
    struct Ent {
      std::string name;
      bool is_group;
      GroupRefs refs;
      uint64_t heap_off;
    };
    std::vector<Ent> ents;
    for (auto& kv : g.children) {
      Ent e;
      e.name = kv.first;
      e.is_group = kv.second->is_group;
      if (e.is_group) {
        e.refs = emit_group(*kv.second);
      } else {
        e.refs = {emit_dataset(*kv.second), UNDEF, UNDEF};
      }
      ents.push_back(e);
    }
    // Local heap: offset 0 holds the empty string; names are NUL-terminated, 8-byte padded.
    std::vector<uint8_t> heapdata(8, 0);
    for (auto& e : ents) {
      e.heap_off = heapdata.size();
      heapdata.insert(heapdata.end(), e.name.begin(), e.name.end());
      heapdata.push_back(0);
      while (heapdata.size() % 8) heapdata.push_back(0);
    }
    B.pad8();
    uint64_t heap_addr = B.pos();
    B.bytes("HEAP", 4);
    B.u8(0);
    B.zeros(3);
    B.u64(heapdata.size());
    B.u64(HEAP_FREE_NULL);
    B.u64(heap_addr + 32);
    B.bytes(heapdata.data(), heapdata.size());

    // Symbol table nodes, 2*LK entries each.
    struct Child {
      uint64_t addr;
      uint64_t right_key;  // heap offset of the largest name below this child
    };
    std::vector<Child> level;
    for (size_t s = 0; s < ents.size(); s += 2 * LK) {
      size_t e_end = std::min(ents.size(), s + 2 * LK);
      B.pad8();
      uint64_t a = B.pos();
      B.bytes("SNOD", 4);
      B.u8(1);
      B.u8(0);
      B.u16((uint16_t)(e_end - s));
      for (size_t i = s; i < e_end; ++i) {
        const Ent& e = ents[i];
        B.u64(e.heap_off);
        B.u64(e.refs.ohdr);
        if (e.is_group) {
          B.u32(1);
          B.u32(0);
          B.u64(e.refs.btree);
          B.u64(e.refs.heap);
        } else {
          B.u32(0);
          B.u32(0);
          B.zeros(16);
        }
      }
      B.zeros(SNOD_SIZE - 8 - (e_end - s) * 40);
      level.push_back({a, ents[e_end - 1].heap_off});
    }
    // B-tree levels, bottom-up. Child i of a node holds names in (key_i, key_{i+1}].
    uint64_t root_btree = UNDEF;
    int lvl = 0;
    if (level.empty()) {
      B.pad8();
      root_btree = B.pos();
      B.bytes("TREE", 4);
      B.u8(0);
      B.u8(0);
      B.u16(0);
      B.u64(UNDEF);
      B.u64(UNDEF);
      B.u64(0);  // key 0
      B.zeros(BTREE_SIZE - 32);
    }
    while (!level.empty()) {
      size_t nnodes = (level.size() + 2 * IK - 1) / (2 * IK);
      std::vector<uint64_t> addrs(nnodes);
      B.pad8();
      uint64_t first = B.pos();
      for (size_t k = 0; k < nnodes; ++k) addrs[k] = first + k * BTREE_SIZE;
      std::vector<Child> next;
      uint64_t left_key = 0;
      for (size_t k = 0; k < nnodes; ++k) {
        size_t c0 = k * 2 * IK, c1 = std::min(level.size(), c0 + 2 * IK);
        uint64_t start = B.pos();
        B.bytes("TREE", 4);
        B.u8(0);
        B.u8((uint8_t)lvl);
        B.u16((uint16_t)(c1 - c0));
        B.u64(k > 0 ? addrs[k - 1] : UNDEF);
        B.u64(k + 1 < nnodes ? addrs[k + 1] : UNDEF);
        B.u64(left_key);
        for (size_t c = c0; c < c1; ++c) {
          B.u64(level[c].addr);
          B.u64(level[c].right_key);
        }
        B.zeros(BTREE_SIZE - (B.pos() - start));
        next.push_back({addrs[k], level[c1 - 1].right_key});
        left_key = level[c1 - 1].right_key;
      }
      if (next.size() == 1) {
        root_btree = next[0].addr;
        break;
      }
      level.swap(next);
      ++lvl;
    }
    B.pad8();
    Msg stab{0x0011, 0, {}};
    le(stab.data, root_btree, 8);
    le(stab.data, heap_addr, 8);
    uint64_t oh = emit_ohdr_v1(B, {stab});
    return {oh, root_btree, heap_addr};
  }
};
}  // namespace

namespace {
// Metadata with holes, superblock patched.
void emit_file(const Writer::Node& root, Buf* out);
}  // namespace

std::vector<uint8_t> Writer::serialize() const {
  Buf B;
  emit_file(*root_, &B);
  std::vector<uint8_t> f;
  f.reserve(B.pos());
  size_t at = 0;
  for (const auto& h : B.holes) {
    f.insert(f.end(), B.b.begin() + at, B.b.begin() + h.at);
    f.insert(f.end(), h.p, h.p + h.n);
    at = h.at;
  }
  f.insert(f.end(), B.b.begin() + at, B.b.end());
  return f;
}

bool Writer::write(const std::string& filename) const {
  Buf B;
  emit_file(*root_, &B);
  FILE* f = std::fopen(filename.c_str(), "wb");
  if (!f) return false;
  bool ok = true;
  size_t at = 0;
  for (const auto& h : B.holes) {
    ok = ok && std::fwrite(B.b.data() + at, 1, h.at - at, f) == h.at - at;
    ok = ok && std::fwrite(h.p, 1, h.n, f) == h.n;
    at = h.at;
  }
  ok = ok && std::fwrite(B.b.data() + at, 1, B.b.size() - at, f) == B.b.size() - at;
  int c = std::fclose(f);
  return ok && c == 0;
}

namespace {
void emit_file(const Writer::Node& root, Buf* out) {
  Emitter E;
  E.B.zeros(96);
  GroupRefs r = E.emit_group(root);
  E.B.pad8();
  Buf& B = E.B;
  uint64_t eof = B.pos();
  std::memcpy(B.b.data(), SIGNATURE, 8);
  uint8_t* s = B.b.data();
  s[8] = 0; s[9] = 0; s[10] = 0; s[11] = 0; s[12] = 0; s[13] = 8; s[14] = 8; s[15] = 0;
  s[16] = LK & 0xff; s[17] = (LK >> 8) & 0xff;
  s[18] = IK & 0xff; s[19] = (IK >> 8) & 0xff;
  B.put64(24, 0);      // base address
  B.put64(32, UNDEF);  // free-space info
  B.put64(40, eof);    // end of file
  B.put64(48, UNDEF);  // driver info
  B.put64(56, 0);      // root entry: link name offset
  B.put64(64, r.ohdr);
  s[72] = 1; s[73] = 0; s[74] = 0; s[75] = 0;  // cache type 1: symbol table info cached
  B.put64(80, r.btree);
  B.put64(88, r.heap);
  *out = std::move(B);
}
}  // namespace

// =============================================================================================
// Reader
// =============================================================================================
struct Reader::Impl {
  std::vector<uint8_t> f;
  uint64_t base = 0;
  int so = 8, sl = 8;
  uint64_t root_ohdr = UNDEF;
  std::string* err = nullptr;

  bool fail(const std::string& m) {
    if (err) *err = m;
    return false;
  }
  bool have(uint64_t a, uint64_t n) const { return a <= f.size() && n <= f.size() - a; }
  uint64_t rd(uint64_t a, int n) const {
    uint64_t v = 0;
    for (int i = 0; i < n; ++i) v |= (uint64_t)f[a + i] << (8 * i);
    return v;
  }
  uint64_t rdo(uint64_t a) const {
    uint64_t v = rd(a, so);
    if (so < 8 && v == ((1ull << (8 * so)) - 1)) return UNDEF;
    return v;
  }
  uint64_t addr(uint64_t rel) const { return rel == UNDEF ? UNDEF : rel + base; }

  bool parse_superblock() {
    // The superblock may sit at 0, 512, 1024, ... (user block).
    uint64_t at = UNDEF;
    for (uint64_t p = 0; p + 8 <= f.size(); p = (p == 0 ? 512 : p * 2)) {
      if (std::memcmp(&f[p], SIGNATURE, 8) == 0) { at = p; break; }
    }
    if (at == UNDEF) return fail("not an HDF5 file (no signature)");
    if (!have(at, 16)) return fail("truncated superblock");
    int ver = f[at + 8];
    if (ver == 0 || ver == 1) {
      so = f[at + 13];
      sl = f[at + 14];
      if (so < 2 || so > 8 || sl < 2 || sl > 8) return fail("unsupported offset/length size");
      uint64_t p = at + 24;
      if (ver == 1) p += 4;
      if (!have(p, 4 * so + 8 + 2 * so + 16)) return fail("truncated superblock");
      base = rd(p, so);
      p += 4 * so;  // base, free-space, EOF, driver info
      // root group symbol table entry
      p += so;      // link name offset
      root_ohdr = addr(rdo(p));
    } else if (ver == 2 || ver == 3) {
      so = f[at + 9];
      sl = f[at + 10];
      uint64_t p = at + 12;
      base = rd(p, so);
      p += 3 * so;  // base, superblock extension, EOF
      root_ohdr = addr(rdo(p));
    } else {
      return fail("unsupported superblock version " + std::to_string(ver));
    }
    return true;
  }

  struct M {
    int type;
    uint64_t off, size;
  };

  bool messages(uint64_t oh, std::vector<M>* out) {
    if (!have(oh, 16)) return fail("object header out of range");
    struct Chunk {
      uint64_t a, n;
    };
    std::vector<Chunk> chunks;
    if (std::memcmp(&f[oh], "OHDR", 4) == 0) {
      int flags = f[oh + 5];
      uint64_t p = oh + 6;
      if (flags & 0x20) p += 16;
      if (flags & 0x10) p += 4;
      int csz = 1 << (flags & 3);
      uint64_t n = rd(p, csz);
      p += csz;
      chunks.push_back({p, n});
      bool track_order = (flags & 0x04) != 0;
      for (size_t ci = 0; ci < chunks.size(); ++ci) {
        uint64_t q = chunks[ci].a, end = chunks[ci].a + chunks[ci].n;
        if (!have(chunks[ci].a, chunks[ci].n)) return fail("object header chunk out of range");
        int hdr = track_order ? 6 : 4;
        while (q + hdr <= end) {
          int type = f[q];
          uint64_t sz = rd(q + 1, 2);
          q += hdr;
          if (q + sz > end) break;
          if (type == 0x10) {
            uint64_t ca = addr(rdo(q)), cl = rd(q + so, sl);
            if (!have(ca, cl) || cl < 8 || std::memcmp(&f[ca], "OCHK", 4) != 0)
              return fail("bad continuation chunk");
            chunks.push_back({ca + 4, cl - 8});
          } else {
            out->push_back({type, q, sz});
          }
          q += sz;
        }
      }
      return true;
    }
    if (f[oh] != 1) return fail("unsupported object header version " + std::to_string(f[oh]));
    uint64_t nm = rd(oh + 2, 2);
    uint64_t sz = rd(oh + 8, 4);
    chunks.push_back({oh + 16, sz});
    uint64_t seen = 0;
    for (size_t ci = 0; ci < chunks.size() && seen < nm; ++ci) {
      uint64_t q = chunks[ci].a, end = chunks[ci].a + chunks[ci].n;
      if (!have(chunks[ci].a, chunks[ci].n)) return fail("object header chunk out of range");
      while (q + 8 <= end && seen < nm) {
        int type = (int)rd(q, 2);
        uint64_t msz = rd(q + 2, 2);
        q += 8;
        if (q + msz > end) return fail("object header message overruns chunk");
        ++seen;
        if (type == 0x10) {
          chunks.push_back({addr(rdo(q)), rd(q + so, sl)});
        } else {
          out->push_back({type, q, msz});
        }
        q += msz;
      }
    }
    return true;
  }

  bool heap_name(uint64_t heap, uint64_t off, std::string* s) {
    if (!have(heap, 8 + 2 * sl + so) || std::memcmp(&f[heap], "HEAP", 4) != 0)
      return fail("bad local heap");
    uint64_t dsz = rd(heap + 8, sl);
    uint64_t da = addr(rdo(heap + 8 + 2 * sl));
    if (off >= dsz || !have(da, dsz)) return fail("bad heap offset");
    const char* c = (const char*)&f[da + off];
    size_t n = strnlen(c, dsz - off);
    s->assign(c, n);
    return true;
  }

  bool btree_collect(uint64_t node, uint64_t heap, std::map<std::string, uint64_t>* out,
                     int depth) {
    if (depth > 64) return fail("B-tree too deep");
    if (!have(node, 8 + 2 * so) || std::memcmp(&f[node], "TREE", 4) != 0)
      return fail("bad B-tree node");
    if (f[node + 4] != 0) return fail("not a group B-tree");
    int level = f[node + 5];
    uint64_t n = rd(node + 6, 2);
    uint64_t p = node + 8 + 2 * so + sl;  // past header and key 0
    for (uint64_t i = 0; i < n; ++i) {
      if (!have(p, so + sl)) return fail("B-tree node out of range");
      uint64_t child = addr(rdo(p));
      p += so + sl;
      if (level > 0) {
        if (!btree_collect(child, heap, out, depth + 1)) return false;
      } else {
        if (!have(child, 8) || std::memcmp(&f[child], "SNOD", 4) != 0)
          return fail("bad symbol table node");
        uint64_t ns = rd(child + 6, 2);
        uint64_t e = child + 8;
        uint64_t esz = so + so + 4 + 4 + 16;
        for (uint64_t k = 0; k < ns; ++k, e += esz) {
          if (!have(e, esz)) return fail("symbol table entry out of range");
          std::string name;
          if (!heap_name(heap, rd(e, sl), &name)) return false;
          (*out)[name] = addr(rdo(e + sl));
        }
      }
    }
    return true;
  }

  bool members(uint64_t oh, std::map<std::string, uint64_t>* out) {
    std::vector<M> ms;
    if (!messages(oh, &ms)) return false;
    bool is_group = false;
    for (auto& m : ms) {
      if (m.type == 0x11) {
        uint64_t bt = addr(rdo(m.off)), hp = addr(rdo(m.off + so));
        if (!btree_collect(bt, hp, out, 0)) return false;
        is_group = true;
      } else if (m.type == 0x06) {
        // Link message (compact link storage)
        uint64_t p = m.off;
        int flags = f[p + 1];
        p += 2;
        int ltype = 0;
        if (flags & 0x08) ltype = f[p++];
        if (flags & 0x04) p += 8;
        if (flags & 0x10) p += 1;
        int lsz = 1 << (flags & 3);
        uint64_t nlen = rd(p, lsz);
        p += lsz;
        std::string name((const char*)&f[p], nlen);
        p += nlen;
        if (ltype == 0) (*out)[name] = addr(rdo(p));
        is_group = true;
      } else if (m.type == 0x02) {
        uint64_t p = m.off + 1;
        int flags = f[p++];
        if (flags & 1) p += 8;
        uint64_t fheap = rdo(p);
        if (fheap != UNDEF) return fail("dense link storage (fractal heap) is not supported");
        is_group = true;
      }
    }
    if (!is_group) return fail("object is not a group");
    return true;
  }

  // member tables of the groups resolved so far, by object header address (the file is read-only)
  std::map<uint64_t, std::map<std::string, uint64_t>> member_cache;

  bool resolve(const std::string& path, uint64_t* oh) {
    uint64_t cur = root_ohdr;
    for (auto& part : split_path(path)) {
      auto c = member_cache.find(cur);
      if (c == member_cache.end()) {
        std::map<std::string, uint64_t> mem;
        if (!members(cur, &mem)) return false;
        c = member_cache.emplace(cur, std::move(mem)).first;
      }
      auto it = c->second.find(part);
      if (it == c->second.end()) return fail("no such object: " + path);
      cur = it->second;
    }
    *oh = cur;
    return true;
  }

  bool dataset(uint64_t oh, DatasetInfo* d) {
    std::vector<M> ms;
    if (!messages(oh, &ms)) return false;
    bool has_space = false, has_type = false, has_layout = false;
    for (auto& m : ms) {
      uint64_t p = m.off;
      if (m.type == 0x01) {
        int ver = f[p];
        int rank = f[p + 1];
        d->dims.clear();
        if (ver == 1) {
          p += 8;
        } else if (ver == 2) {
          p += 4;
        } else {
          return fail("unsupported dataspace version");
        }
        for (int i = 0; i < rank; ++i) d->dims.push_back(rd(p + (uint64_t)i * sl, sl));
        has_space = true;
      } else if (m.type == 0x03) {
        d->type_class = f[p] & 0x0f;
        int bits0 = f[p + 1];
        d->type_size = (uint32_t)rd(p + 4, 4);
        d->big_endian = (bits0 & 1) != 0;
        d->is_signed = (d->type_class == 0) && (bits0 & 0x08);
        if (d->type_class != 0 && d->type_class != 1)
          return fail("unsupported datatype class " + std::to_string(d->type_class));
        has_type = true;
      } else if (m.type == 0x08) {
        int ver = f[p];
        if (ver == 3 || ver == 4) {
          int cls = f[p + 1];
          if (cls == 1) {
            d->data_addr = addr(rdo(p + 2));
            d->data_size = rd(p + 2 + so, sl);
            d->compact = false;
          } else if (cls == 0) {
            uint64_t n = rd(p + 2, 2);
            d->compact = true;
            d->compact_data.assign(f.begin() + p + 4, f.begin() + p + 4 + n);
            d->data_size = n;
          } else {
            return fail("chunked/virtual dataset layout is not supported");
          }
        } else if (ver == 1 || ver == 2) {
          int nd = f[p + 1];
          int cls = f[p + 2];
          p += 8;
          if (cls == 1) {
            d->data_addr = addr(rdo(p));
            p += so;
            d->compact = false;
            d->data_size = UNDEF;
          } else if (cls == 0) {
            p += 4 * (uint64_t)nd;
            uint64_t n = rd(p, 4);
            d->compact = true;
            d->compact_data.assign(f.begin() + p + 4, f.begin() + p + 4 + n);
            d->data_size = n;
          } else {
            return fail("chunked dataset layout is not supported");
          }
        } else {
          return fail("unsupported layout version");
        }
        has_layout = true;
      } else if (m.type == 0x0B) {
        return fail("filtered (compressed) datasets are not supported");
      }
    }
    if (!has_space || !has_type || !has_layout) return fail("object is not a dataset");
    return true;
  }
};

Reader::Reader() : impl_(new Impl) { impl_->err = &err_; }
Reader::~Reader() {}

bool Reader::open(const std::string& filename) {
  FILE* fp = std::fopen(filename.c_str(), "rb");
  if (!fp) {
    err_ = "cannot open " + filename;
    return false;
  }
  std::vector<uint8_t> bytes;
  std::fseek(fp, 0, SEEK_END);
  long n = std::ftell(fp);
  std::fseek(fp, 0, SEEK_SET);
  if (n < 0) {
    std::fclose(fp);
    err_ = "cannot size " + filename;
    return false;
  }
  bytes.resize((size_t)n);
  size_t got = n ? std::fread(bytes.data(), 1, (size_t)n, fp) : 0;
  std::fclose(fp);
  if (got != (size_t)n) {
    err_ = "short read on " + filename;
    return false;
  }
  return open_memory(std::move(bytes));
}

bool Reader::open_memory(std::vector<uint8_t> bytes) {
  impl_->f = std::move(bytes);
  impl_->member_cache.clear();
  return impl_->parse_superblock();
}

bool Reader::info(const std::string& path, DatasetInfo* out) {
  uint64_t oh;
  if (!impl_->resolve(path, &oh)) return false;
  *out = DatasetInfo();
  return impl_->dataset(oh, out);
}

bool Reader::exists(const std::string& path) {
  uint64_t oh;
  std::string keep = err_;
  bool ok = impl_->resolve(path, &oh);
  err_ = keep;
  return ok;
}

bool Reader::list(const std::string& path, std::vector<std::string>* names) {
  uint64_t oh;
  if (!impl_->resolve(path, &oh)) return false;
  std::map<std::string, uint64_t> mem;
  if (!impl_->members(oh, &mem)) return false;
  names->clear();
  for (auto& kv : mem) names->push_back(kv.first);
  return true;
}

namespace {
template <class T>
T clamp_from_i(int64_t v) {
  if (v < (int64_t)std::numeric_limits<T>::lowest()) return std::numeric_limits<T>::lowest();
  if (std::numeric_limits<T>::is_integer && sizeof(T) < 8 &&
      v > (int64_t)std::numeric_limits<T>::max())
    return std::numeric_limits<T>::max();
  return (T)v;
}
template <class T>
T clamp_from_u(uint64_t v) {
  if (std::numeric_limits<T>::is_integer && v > (uint64_t)std::numeric_limits<T>::max())
    return std::numeric_limits<T>::max();
  return (T)v;
}
template <class T>
T clamp_from_f(double v) {
  if (!std::numeric_limits<T>::is_integer) return (T)v;
  if (std::isnan(v)) return 0;
  if (v <= (double)std::numeric_limits<T>::lowest()) return std::numeric_limits<T>::lowest();
  if (v >= (double)std::numeric_limits<T>::max()) return std::numeric_limits<T>::max();
  return (T)v;
}
template <class T>
void store(uint8_t* dst, T v) {
  std::memcpy(dst, &v, sizeof(T));
}
}  // namespace

bool Reader::read(const std::string& path, DType want, std::vector<uint64_t>* dims,
                  std::vector<uint8_t>* out) {
  DatasetInfo d;
  if (!info(path, &d)) return false;
  if (dims) *dims = d.dims;
  uint64_t n = d.nelem();
  uint32_t es = d.type_size;
  if (!(es == 1 || es == 2 || es == 4 || es == 8) || (d.type_class == 1 && es < 4)) {
    err_ = "unsupported element size in " + path;
    return false;
  }
  const uint8_t* src = nullptr;
  std::vector<uint8_t> zeros;
  if (d.compact) {
    if (d.compact_data.size() < n * es) {
      err_ = "compact data too small in " + path;
      return false;
    }
    src = d.compact_data.data();
  } else if (d.data_addr == UNDEF) {
    zeros.assign(n * es, 0);  // never written: default fill value 0
    src = zeros.data();
  } else {
    if (!impl_->have(d.data_addr, n * es)) {
      err_ = "dataset data out of range in " + path;
      return false;
    }
    src = &impl_->f[d.data_addr];
  }
  size_t osz = dtype_size(want);
  // fast paths (same results as the element loop below): little-endian data already in the wanted
  // representation is copied; signed 64-bit integers (h5py's default) to uint32 clamp in one loop
  const bool want_float = want == DType::F64 || want == DType::F32;
  const bool want_signed = want == DType::I32 || want == DType::I64;
  if (!d.big_endian && es == osz &&
      (d.type_class == 1 ? want_float : (!want_float && want_signed == d.is_signed))) {
    out->assign(src, src + n * es);
    return true;
  }
  if (!d.big_endian && d.type_class == 0 && d.is_signed && es == 8 && want == DType::U32) {
    out->assign(n * 4, 0);
    uint32_t* o = reinterpret_cast<uint32_t*>(out->data());
    for (uint64_t i = 0; i < n; ++i) {
      int64_t sv;
      std::memcpy(&sv, src + i * 8, 8);
      const uint32_t v = sv < 0 ? 0u : clamp_from_u<uint32_t>((uint64_t)sv);
      std::memcpy(o + i, &v, 4);
    }
    return true;
  }
  out->assign(n * osz, 0);
  for (uint64_t i = 0; i < n; ++i) {
    uint8_t e[8];
    for (uint32_t k = 0; k < es; ++k) e[k] = src[i * es + (d.big_endian ? (es - 1 - k) : k)];
    uint8_t* o = out->data() + i * osz;
    if (d.type_class == 1) {
      double v;
      if (es == 8) {
        std::memcpy(&v, e, 8);
      } else {
        float fv;
        std::memcpy(&fv, e, 4);
        v = fv;
      }
      switch (want) {
        case DType::F64: store(o, v); break;
        case DType::F32: store(o, (float)v); break;
        case DType::U32: store(o, clamp_from_f<uint32_t>(v)); break;
        case DType::I32: store(o, clamp_from_f<int32_t>(v)); break;
        case DType::U64: store(o, clamp_from_f<uint64_t>(v)); break;
        case DType::I64: store(o, clamp_from_f<int64_t>(v)); break;
        case DType::U8: store(o, clamp_from_f<uint8_t>(v)); break;
      }
    } else {
      uint64_t raw = 0;
      for (uint32_t k = 0; k < es; ++k) raw |= (uint64_t)e[k] << (8 * k);
      if (d.is_signed) {
        int64_t sv;
        if (es < 8 && (raw >> (8 * es - 1)) & 1) raw |= ~0ull << (8 * es);
        std::memcpy(&sv, &raw, 8);
        switch (want) {
          case DType::F64: store(o, (double)sv); break;
          case DType::F32: store(o, (float)sv); break;
          case DType::U32: store(o, sv < 0 ? 0u : clamp_from_u<uint32_t>((uint64_t)sv)); break;
          case DType::I32: store(o, clamp_from_i<int32_t>(sv)); break;
          case DType::U64: store(o, sv < 0 ? (uint64_t)0 : (uint64_t)sv); break;
          case DType::I64: store(o, sv); break;
          case DType::U8: store(o, sv < 0 ? (uint8_t)0 : clamp_from_u<uint8_t>((uint64_t)sv)); break;
        }
      } else {
        switch (want) {
          case DType::F64: store(o, (double)raw); break;
          case DType::F32: store(o, (float)raw); break;
          case DType::U32: store(o, clamp_from_u<uint32_t>(raw)); break;
          case DType::I32: store(o, clamp_from_u<int32_t>(raw)); break;
          case DType::U64: store(o, raw); break;
          case DType::I64: store(o, clamp_from_u<int64_t>(raw)); break;
          case DType::U8: store(o, clamp_from_u<uint8_t>(raw)); break;
        }
      }
    }
  }
  return true;
}

}  // namespace h5l
