// HDF5 checkpoint and record files of the reference, read and written
// without libhdf5 (host code only).
//
// The reference writes its snapshots with the HDF5 Fortran API
// (big_periodic_3D.f90:593-651: h5fcreate_f, h5ltset_attribute_*_f,
// h5ltmake_dataset_double_f), its per-step sub-block records in groups
// "t_%.4f" (:664-712, h5gcreate_f), and restarts from a snapshot
// (:296-324, h5ltread_dataset_double_f).  This file implements the part of the
// published HDF5 File Format Specification that those calls produce with the
// library's default property lists:
//   - a version 0 superblock (8-byte offsets and lengths, group K 4 / 16);
//   - version 1 object headers, with continuation blocks on reading;
//   - groups as symbol tables: a local heap of names, a version 1 B-tree
//     (any depth) and symbol table nodes;
//   - datasets: version 1 dataspace, IEEE little-endian double datatype,
//     version 1 fill value, contiguous version 3 layout (reading also takes
//     version 1-3 compact and contiguous layouts and other numeric types);
//   - attributes: version 1 messages (reading takes versions 1-3) of 32-bit
//     integers, doubles and null-terminated fixed strings.
// Chunked or compressed datasets, version 2 object headers and link-message
// groups are reported as NS_ERR_IO ("outside the subset").
//
// A file is an in-memory tree of object-header messages over the raw data on
// disk.  Raw data goes to the end of the file when a dataset is written; a
// flush writes every object header, heap, B-tree and symbol table node anew at
// the end of the file and then the superblock, so the file on disk is
// complete after every flush (the metadata of an earlier flush stays behind
// as unused bytes).  Opening an existing file for writing reads its tree and
// keeps every message it does not regenerate (attributes, dataspaces,
// layouts) byte for byte.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <set>
#include <string>
#include <vector>

#include "../../include/ns_gpu.h"
#include "ns_session.cuh"

namespace {

constexpr uint64_t kUndef = ~0ull;
constexpr int kLeafK = 4;   // symbol table nodes hold 2 * kLeafK entries
constexpr int kNodeK = 16;  // B-tree nodes hold 2 * kNodeK children
constexpr unsigned char kSig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
constexpr int kMaxDepth = 64;

enum : uint16_t {
  MSG_NIL = 0x0000,
  MSG_DATASPACE = 0x0001,
  MSG_DATATYPE = 0x0003,
  MSG_FILL = 0x0005,
  MSG_LAYOUT = 0x0008,
  MSG_ATTR = 0x000C,
  MSG_CONT = 0x0010,
  MSG_STAB = 0x0011,
};

using Bytes = std::vector<uint8_t>;

inline uint64_t pad8(uint64_t n) { return (n + 7) & ~7ull; }

void put(Bytes& b, uint64_t v, int n) {
  for (int i = 0; i < n; ++i) b.push_back((uint8_t)(v >> (8 * i)));
}
void put_bytes(Bytes& b, const void* p, size_t n) {
  const uint8_t* s = static_cast<const uint8_t*>(p);
  b.insert(b.end(), s, s + n);
}
void pad_to8(Bytes& b) {
  while (b.size() % 8) b.push_back(0);
}
uint64_t get(const uint8_t* p, int n) {
  uint64_t v = 0;
  for (int i = 0; i < n; ++i) v |= (uint64_t)p[i] << (8 * i);
  return v;
}

struct Msg {
  uint16_t type;
  uint8_t flags;
  Bytes data;
};

// One object: a group (children by name, strcmp order as in a symbol table)
// or a dataset; msgs holds every message but a group's symbol table.
struct Node {
  bool group = false;
  std::vector<Msg> msgs;
  std::map<std::string, std::unique_ptr<Node>> kids;
};

struct IoError {
  std::string what;
};

}  // namespace

struct ns_h5 {
  std::FILE* fp = nullptr;
  bool writable = false;
  uint64_t base = 0;  // absolute position of the superblock; addresses are relative to it
  uint64_t end = 0;   // relative end of the file (next allocation)
  Node root;
  bool dirty = false;
  std::string err;
};

namespace {

// ---------------------------------------------------------------------------
// low-level file access
// ---------------------------------------------------------------------------
void read_at(ns_h5* f, uint64_t rel, void* dst, size_t n) {
  if (rel == kUndef || rel > f->end || n > f->end - rel) throw IoError{"address past the end of the file"};
  if (fseeko(f->fp, (off_t)(f->base + rel), SEEK_SET) != 0 || std::fread(dst, 1, n, f->fp) != n)
    throw IoError{"read failed"};
}
Bytes read_bytes(ns_h5* f, uint64_t rel, size_t n) {
  Bytes b(n);
  if (n) read_at(f, rel, b.data(), n);
  return b;
}
// Append n bytes at the end of the file; returns their address.
uint64_t append(ns_h5* f, const void* src, size_t n) {
  const uint64_t a = f->end;
  if (n) {
    if (fseeko(f->fp, (off_t)(f->base + a), SEEK_SET) != 0 || std::fwrite(src, 1, n, f->fp) != n)
      throw IoError{"write failed"};
  }
  f->end += n;
  return a;
}
uint64_t append(ns_h5* f, const Bytes& b) { return append(f, b.data(), b.size()); }

// ---------------------------------------------------------------------------
// reading the tree
// ---------------------------------------------------------------------------
// Messages of the version 1 object header at addr (continuations followed).
std::vector<Msg> read_messages(ns_h5* f, uint64_t addr) {
  uint8_t pre[16];
  read_at(f, addr, pre, 16);
  if (pre[0] != 1) throw IoError{"object header version " + std::to_string(pre[0]) + " is outside the subset"};
  const uint64_t nmsg = get(pre + 2, 2);
  const uint64_t size = get(pre + 8, 4);
  std::vector<std::pair<uint64_t, uint64_t>> chunks = {{addr + 16, size}};
  std::vector<Msg> out;
  for (size_t c = 0; c < chunks.size() && out.size() < nmsg; ++c) {
    if (c > 4096) throw IoError{"too many object header continuations"};
    const Bytes blk = read_bytes(f, chunks[c].first, chunks[c].second);
    size_t p = 0;
    while (p + 8 <= blk.size() && out.size() < nmsg) {
      Msg m;
      m.type = (uint16_t)get(&blk[p], 2);
      const size_t ms = (size_t)get(&blk[p + 2], 2);
      m.flags = blk[p + 4];
      if (p + 8 + ms > blk.size()) throw IoError{"object header message past its block"};
      m.data.assign(blk.begin() + p + 8, blk.begin() + p + 8 + ms);
      if (m.type == MSG_CONT) {
        if (ms < 16) throw IoError{"short continuation message"};
        chunks.push_back({get(&m.data[0], 8), get(&m.data[8], 8)});
      }
      out.push_back(std::move(m));
      p += 8 + ms;
    }
  }
  return out;
}

std::string heap_name(ns_h5* f, uint64_t seg, uint64_t seg_size, uint64_t off) {
  if (off >= seg_size) throw IoError{"name offset outside the local heap"};
  const Bytes b = read_bytes(f, seg + off, (size_t)std::min<uint64_t>(seg_size - off, 1024));
  const auto z = std::find(b.begin(), b.end(), 0);
  if (z == b.end()) throw IoError{"unterminated name in the local heap"};
  return std::string(b.begin(), z);
}

void read_btree(ns_h5* f, uint64_t node, uint64_t seg, uint64_t seg_size, int depth,
                std::vector<std::pair<std::string, uint64_t>>& out) {
  if (depth > kMaxDepth) throw IoError{"group B-tree too deep"};
  uint8_t hd[24];
  read_at(f, node, hd, 24);
  if (std::memcmp(hd, "TREE", 4) != 0) throw IoError{"bad B-tree node signature"};
  if (hd[4] != 0) throw IoError{"not a group B-tree"};
  const int level = hd[5];
  const int used = (int)get(hd + 6, 2);
  if (used > 2 * 1024) throw IoError{"B-tree node with too many entries"};
  const Bytes kv = read_bytes(f, node + 24, (size_t)used * 16 + 8);
  for (int i = 0; i < used; ++i) {
    const uint64_t child = get(&kv[8 + 16 * i], 8);
    if (level > 0) {
      read_btree(f, child, seg, seg_size, depth + 1, out);
      continue;
    }
    uint8_t sh[8];
    read_at(f, child, sh, 8);
    if (std::memcmp(sh, "SNOD", 4) != 0) throw IoError{"bad symbol table node signature"};
    const int nsym = (int)get(sh + 6, 2);
    const Bytes ent = read_bytes(f, child + 8, (size_t)nsym * 40);
    for (int k = 0; k < nsym; ++k)
      out.push_back({heap_name(f, seg, seg_size, get(&ent[40 * k], 8)), get(&ent[40 * k + 8], 8)});
  }
}

std::unique_ptr<Node> read_node(ns_h5* f, uint64_t addr, int depth, std::set<uint64_t>& path) {
  if (depth > kMaxDepth || path.count(addr)) throw IoError{"group cycle or nesting too deep"};
  auto n = std::make_unique<Node>();
  std::vector<Msg> msgs = read_messages(f, addr);
  const Msg* stab = nullptr;
  for (const Msg& m : msgs)
    if (m.type == MSG_STAB) stab = &m;
  if (stab) {
    if (stab->data.size() < 16) throw IoError{"short symbol table message"};
    const uint64_t bt = get(&stab->data[0], 8), heap = get(&stab->data[8], 8);
    uint8_t hh[32];
    read_at(f, heap, hh, 32);
    if (std::memcmp(hh, "HEAP", 4) != 0) throw IoError{"bad local heap signature"};
    const uint64_t seg_size = get(hh + 8, 8), seg = get(hh + 24, 8);
    std::vector<std::pair<std::string, uint64_t>> kids;
    read_btree(f, bt, seg, seg_size, 0, kids);
    path.insert(addr);
    for (auto& [name, child] : kids) n->kids[name] = read_node(f, child, depth + 1, path);
    path.erase(addr);
    n->group = true;
  }
  for (Msg& m : msgs)
    if (m.type != MSG_STAB && m.type != MSG_NIL && m.type != MSG_CONT) n->msgs.push_back(std::move(m));
  if (!n->group) {
    bool ds = false, dt = false, lay = false;
    for (const Msg& m : n->msgs) {
      ds |= m.type == MSG_DATASPACE;
      dt |= m.type == MSG_DATATYPE;
      lay |= m.type == MSG_LAYOUT;
    }
    if (!(ds && dt && lay)) throw IoError{"an object that is neither a symbol-table group nor a dataset"};
  }
  return n;
}

void read_file(ns_h5* f) {
  if (fseeko(f->fp, 0, SEEK_END) != 0) throw IoError{"seek failed"};
  const uint64_t size = (uint64_t)ftello(f->fp);
  uint8_t sb[96];
  bool found = false;
  for (uint64_t off = 0; off + 96 <= size; off = off ? off * 2 : 512) {
    if (fseeko(f->fp, (off_t)off, SEEK_SET) != 0 || std::fread(sb, 1, 96, f->fp) != 96) break;
    if (std::memcmp(sb, kSig, 8) == 0) {
      f->base = off;
      found = true;
      break;
    }
  }
  if (!found) throw IoError{"no HDF5 superblock"};
  if (sb[8] != 0) throw IoError{"superblock version " + std::to_string(sb[8]) + " is outside the subset"};
  if (sb[13] != 8 || sb[14] != 8) throw IoError{"offsets and lengths of 8 bytes only"};
  const uint64_t base_addr = get(sb + 24, 8);
  if (base_addr != f->base) throw IoError{"the base address is not the superblock's position"};
  // the stored end of file counts from the start of the file, user block included
  const uint64_t stored_eof = get(sb + 40, 8);
  if (stored_eof > size) throw IoError{"truncated file"};
  f->end = size - f->base;
  const uint64_t root = get(sb + 56 + 8, 8);
  std::set<uint64_t> path;
  std::unique_ptr<Node> r = read_node(f, root, 0, path);
  if (!r->group) throw IoError{"the root object is not a group"};
  f->root = std::move(*r);
}

}  // namespace

namespace {

// ---------------------------------------------------------------------------
// message decoding
// ---------------------------------------------------------------------------
// Dims of a version 1 or 2 dataspace (file order: slowest first); scalar = {}.
std::vector<uint64_t> decode_dataspace(const Bytes& d) {
  if (d.size() < 4) throw IoError{"short dataspace message"};
  const int ver = d[0], rank = d[1];
  size_t p;
  if (ver == 1) p = 8;
  else if (ver == 2) {
    if (d[3] == 2) return {};  // null dataspace: no elements (read as scalar of nothing)
    p = 4;
  } else throw IoError{"dataspace version " + std::to_string(ver) + " is outside the subset"};
  if (d.size() < p + 8 * (size_t)rank) throw IoError{"short dataspace message"};
  std::vector<uint64_t> dims(rank);
  for (int i = 0; i < rank; ++i) dims[i] = get(&d[p + 8 * i], 8);
  return dims;
}

// A numeric or string datatype: class 0 (integer), 1 (float), 3 (string).
struct Type {
  int cls = -1;
  size_t size = 0;
  bool big = false;
  bool is_signed = false;
};
Type decode_datatype(const Bytes& d) {
  if (d.size() < 8) throw IoError{"short datatype message"};
  Type t;
  t.cls = d[0] & 0x0F;
  const uint32_t bits = (uint32_t)get(&d[1], 3);
  t.size = (size_t)get(&d[4], 4);
  if (t.cls == 0) {
    t.big = bits & 1;
    t.is_signed = bits & 8;
    if (t.size != 1 && t.size != 2 && t.size != 4 && t.size != 8) throw IoError{"integer size outside the subset"};
  } else if (t.cls == 1) {
    t.big = bits & 1;
    if (bits & 0x40) throw IoError{"VAX floating point is outside the subset"};
    if (t.size != 4 && t.size != 8) throw IoError{"floating point size outside the subset"};
  } else if (t.cls != 3) {
    throw IoError{"datatype class " + std::to_string(t.cls) + " is outside the subset"};
  }
  return t;
}

// n elements of type t at src, as doubles.
void to_double(const Type& t, const uint8_t* src, uint64_t n, double* out) {
  for (uint64_t i = 0; i < n; ++i) {
    uint8_t e[8];
    const uint8_t* s = src + i * t.size;
    for (size_t k = 0; k < t.size; ++k) e[k] = t.big ? s[t.size - 1 - k] : s[k];
    const uint64_t raw = get(e, (int)t.size);
    if (t.cls == 1 && t.size == 8) {
      std::memcpy(&out[i], &raw, 8);
    } else if (t.cls == 1) {
      const uint32_t r32 = (uint32_t)raw;
      float x;
      std::memcpy(&x, &r32, 4);
      out[i] = x;
    } else if (t.cls == 0) {
      if (t.is_signed) {
        const int sh = 64 - 8 * (int)t.size;
        out[i] = (double)((int64_t)(raw << sh) >> sh);
      } else {
        out[i] = (double)raw;
      }
    } else {
      throw IoError{"a string is not numeric"};
    }
  }
}

const Msg* find_msg(const Node& n, uint16_t type) {
  for (const Msg& m : n.msgs)
    if (m.type == type) return &m;
  return nullptr;
}

// The raw bytes of a dataset (nbytes of them).
Bytes dataset_bytes(ns_h5* f, const Node& n, uint64_t nbytes) {
  const Msg* lay = find_msg(n, MSG_LAYOUT);
  const Bytes& d = lay->data;
  if (d.size() < 2) throw IoError{"short layout message"};
  const int ver = d[0];
  if (ver == 3) {
    const int cls = d[1];
    if (cls == 1) {
      if (d.size() < 18) throw IoError{"short layout message"};
      const uint64_t addr = get(&d[2], 8), size = get(&d[10], 8);
      if (addr == kUndef) return Bytes(nbytes, 0);  // never written: the default fill value
      if (size < nbytes) throw IoError{"contiguous storage smaller than the dataspace"};
      return read_bytes(f, addr, nbytes);
    }
    if (cls == 0) {
      if (d.size() < 4) throw IoError{"short layout message"};
      const uint64_t size = get(&d[2], 2);
      if (size < nbytes || d.size() < 4 + nbytes) throw IoError{"compact storage smaller than the dataspace"};
      return Bytes(d.begin() + 4, d.begin() + 4 + nbytes);
    }
    throw IoError{"chunked or virtual layouts are outside the subset"};
  }
  if (ver == 1 || ver == 2) {
    if (d.size() < 8) throw IoError{"short layout message"};
    const int rank = d[1], cls = d[2];
    if (cls == 1) {
      if (d.size() < 16) throw IoError{"short layout message"};
      const uint64_t addr = get(&d[8], 8);
      if (addr == kUndef) return Bytes(nbytes, 0);
      return read_bytes(f, addr, nbytes);
    }
    if (cls == 0) {
      const size_t p = 8 + 4 * (size_t)rank;
      if (d.size() < p + 4) throw IoError{"short layout message"};
      const uint64_t size = get(&d[p], 4);
      if (size < nbytes || d.size() < p + 4 + nbytes) throw IoError{"compact storage smaller than the dataspace"};
      return Bytes(d.begin() + p + 4, d.begin() + p + 4 + nbytes);
    }
    throw IoError{"chunked layouts are outside the subset"};
  }
  throw IoError{"layout version " + std::to_string(ver) + " is outside the subset"};
}

// A decoded attribute message (versions 1-3).
struct Attr {
  std::string name;
  Type type;
  std::vector<uint64_t> dims;
  Bytes value;
};
Attr decode_attr(const Bytes& d) {
  if (d.size() < 8) throw IoError{"short attribute message"};
  const int ver = d[0];
  if (ver < 1 || ver > 3) throw IoError{"attribute version outside the subset"};
  const size_t nl = (size_t)get(&d[2], 2), tl = (size_t)get(&d[4], 2), sl = (size_t)get(&d[6], 2);
  auto pad = [&](size_t n) { return ver == 1 ? (size_t)pad8(n) : n; };
  size_t p = ver == 3 ? 9 : 8;
  if (d.size() < p + pad(nl) + pad(tl) + pad(sl)) throw IoError{"short attribute message"};
  Attr a;
  a.name.assign(reinterpret_cast<const char*>(&d[p]), strnlen(reinterpret_cast<const char*>(&d[p]), nl));
  p += pad(nl);
  a.type = decode_datatype(Bytes(d.begin() + p, d.begin() + p + tl));
  p += pad(tl);
  a.dims = decode_dataspace(Bytes(d.begin() + p, d.begin() + p + sl));
  p += pad(sl);
  uint64_t n = 1;
  for (uint64_t x : a.dims) n *= x;
  const uint64_t nb = n * a.type.size;
  if (d.size() < p + nb) throw IoError{"attribute data past its message"};
  a.value.assign(d.begin() + p, d.begin() + p + nb);
  return a;
}

// The object at a slash-separated path ("" or "/" is the root).
Node* lookup(Node& root, const std::string& path) {
  Node* n = &root;
  size_t i = 0;
  while (i < path.size()) {
    if (path[i] == '/') {
      ++i;
      continue;
    }
    const size_t j = path.find('/', i);
    const std::string part = path.substr(i, j == std::string::npos ? std::string::npos : j - i);
    if (!n->group) return nullptr;
    auto it = n->kids.find(part);
    if (it == n->kids.end()) return nullptr;
    n = it->second.get();
    i = j == std::string::npos ? path.size() : j + 1;
  }
  return n;
}

// Parent group and last component of a path to be created.
Node* parent_of(Node& root, const std::string& path, std::string& leaf) {
  std::string p = path;
  while (!p.empty() && p.back() == '/') p.pop_back();
  const size_t s = p.rfind('/');
  leaf = s == std::string::npos ? p : p.substr(s + 1);
  Node* par = s == std::string::npos ? &root : lookup(root, p.substr(0, s));
  if (!par || !par->group) return nullptr;
  return par;
}

}  // namespace

namespace {

// ---------------------------------------------------------------------------
// encoding
// ---------------------------------------------------------------------------
// Version 1 dataspace of the given dims (file order); rank 0 is a scalar.
Bytes enc_dataspace(const std::vector<uint64_t>& dims) {
  Bytes b;
  put(b, 1, 1);
  put(b, dims.size(), 1);
  put(b, 0, 1);  // no maximum dims
  put(b, 0, 5);
  for (uint64_t d : dims) put(b, d, 8);
  return b;
}
// IEEE 754 binary64, little-endian: sign bit 63, exponent 52..62 (bias 1023),
// mantissa 0..51 with an implied leading one.
Bytes enc_double_type() {
  Bytes b = {0x11, 0x20, 0x3f, 0x00};
  put(b, 8, 4);
  put(b, 0, 2);     // bit offset
  put(b, 64, 2);    // precision
  put(b, 52, 1);    // exponent location
  put(b, 11, 1);    // exponent size
  put(b, 0, 1);     // mantissa location
  put(b, 52, 1);    // mantissa size
  put(b, 1023, 4);  // exponent bias
  return b;
}
// Signed 32-bit little-endian integer.
Bytes enc_int32_type() {
  Bytes b = {0x10, 0x08, 0x00, 0x00};
  put(b, 4, 4);
  put(b, 0, 2);
  put(b, 32, 2);
  return b;
}
// Null-terminated ASCII fixed string of n bytes.
Bytes enc_string_type(size_t n) {
  Bytes b = {0x13, 0x00, 0x00, 0x00};
  put(b, n, 4);
  return b;
}
Msg attr_msg(const std::string& name, const Bytes& type, const Bytes& space, const void* val, size_t nval) {
  Msg m{MSG_ATTR, 0, {}};
  Bytes& b = m.data;
  put(b, 1, 1);
  put(b, 0, 1);
  put(b, name.size() + 1, 2);
  put(b, type.size(), 2);
  put(b, space.size(), 2);
  put_bytes(b, name.c_str(), name.size() + 1);
  pad_to8(b);
  put_bytes(b, type.data(), type.size());
  pad_to8(b);
  put_bytes(b, space.data(), space.size());
  pad_to8(b);
  put_bytes(b, val, nval);
  return m;
}
// Replace the attribute of the same name, or add it.
void set_attr(Node& n, Msg m, const std::string& name) {
  for (Msg& x : n.msgs)
    if (x.type == MSG_ATTR && decode_attr(x.data).name == name) {
      x = std::move(m);
      return;
    }
  n.msgs.push_back(std::move(m));
}

// A version 1 object header holding msgs (each padded to 8 bytes).
Bytes object_header(const std::vector<const Msg*>& msgs) {
  uint64_t size = 0;
  for (const Msg* m : msgs) {
    if (pad8(m->data.size()) > 0xFFF8) throw IoError{"object header message too large"};
    size += 8 + pad8(m->data.size());
  }
  if (msgs.size() > 0xFFFF) throw IoError{"too many messages in one object header"};
  Bytes b;
  put(b, 1, 1);  // version
  put(b, 0, 1);
  put(b, msgs.size(), 2);
  put(b, 1, 4);  // reference count
  put(b, size, 4);
  put(b, 0, 4);  // the messages start 8-byte aligned
  for (const Msg* m : msgs) {
    put(b, m->type, 2);
    put(b, pad8(m->data.size()), 2);
    put(b, m->flags, 1);
    put(b, 0, 3);
    put_bytes(b, m->data.data(), m->data.size());
    pad_to8(b);
  }
  return b;
}

struct Placed {
  uint64_t ohdr = kUndef, btree = kUndef, heap = kUndef;
};

// Write node n and everything below it at the end of the file.
Placed write_node(ns_h5* f, Node& n) {
  Placed pl;
  std::vector<const Msg*> msgs;
  Msg stab{MSG_STAB, 1, {}};
  if (n.group) {
    std::vector<std::pair<const std::string*, Placed>> kids;
    for (auto& kv : n.kids) kids.push_back({&kv.first, write_node(f, *kv.second)});
    // local heap: the empty name at offset 0, the member names 8-aligned,
    // then one free block (next: none = 1, size 16)
    Bytes seg;
    put(seg, 0, 8);
    std::vector<uint64_t> off;
    for (auto& k : kids) {
      off.push_back(seg.size());
      put_bytes(seg, k.first->c_str(), k.first->size() + 1);
      pad_to8(seg);
    }
    const uint64_t free_off = seg.size();
    put(seg, 1, 8);
    put(seg, 16, 8);
    Bytes hh;
    put_bytes(hh, "HEAP", 4);
    put(hh, 0, 4);  // version 0, reserved
    put(hh, seg.size(), 8);
    put(hh, free_off, 8);
    pl.heap = f->end;
    put(hh, pl.heap + 32, 8);  // the data segment follows the header
    hh.insert(hh.end(), seg.begin(), seg.end());
    append(f, hh);
    // symbol table nodes: 2 * kLeafK entries each, sorted by name
    std::vector<uint64_t> child, last;  // node address, heap offset of its greatest name
    const size_t per = 2 * kLeafK;
    for (size_t lo = 0; lo < kids.size(); lo += per) {
      const size_t hi = std::min(kids.size(), lo + per);
      Bytes sn;
      put_bytes(sn, "SNOD", 4);
      put(sn, 1, 1);
      put(sn, 0, 1);
      put(sn, hi - lo, 2);
      for (size_t i = lo; i < hi; ++i) {
        const Placed& c = kids[i].second;
        const bool grp = c.btree != kUndef;
        put(sn, off[i], 8);
        put(sn, c.ohdr, 8);
        put(sn, grp ? 1 : 0, 4);  // cache type 1: the scratch pad holds the group's B-tree and heap
        put(sn, 0, 4);
        put(sn, grp ? c.btree : 0, 8);
        put(sn, grp ? c.heap : 0, 8);
      }
      sn.resize(8 + 40 * per, 0);
      child.push_back(append(f, sn));
      last.push_back(off[hi - 1]);
    }
    // B-tree levels (2 * kNodeK children a node, siblings linked); an empty
    // group has one empty level-0 node
    const uint64_t node_size = 24 + (2 * kNodeK + 1) * 8 + 2 * kNodeK * 8;
    int level = 0;
    do {
      const size_t per_node = 2 * kNodeK;
      const size_t nn = std::max<size_t>(1, (child.size() + per_node - 1) / per_node);
      const uint64_t first = f->end;
      std::vector<uint64_t> up, up_last;
      for (size_t c = 0; c < nn; ++c) {
        const size_t lo = c * per_node, hi = std::min(child.size(), lo + per_node);
        Bytes t;
        put_bytes(t, "TREE", 4);
        put(t, 0, 1);  // group node
        put(t, level, 1);
        put(t, hi - lo, 2);
        put(t, c ? first + (c - 1) * node_size : kUndef, 8);
        put(t, c + 1 < nn ? first + (c + 1) * node_size : kUndef, 8);
        put(t, lo == 0 ? 0 : last[lo - 1], 8);  // left key: the name before this node's first
        for (size_t i = lo; i < hi; ++i) {
          put(t, child[i], 8);
          put(t, last[i], 8);
        }
        t.resize(node_size, 0);
        up.push_back(append(f, t));
        up_last.push_back(hi > lo ? last[hi - 1] : 0);
      }
      child = up;
      last = up_last;
      ++level;
    } while (child.size() > 1);
    pl.btree = child[0];
    put(stab.data, pl.btree, 8);
    put(stab.data, pl.heap, 8);
    msgs.push_back(&stab);
  }
  for (const Msg& m : n.msgs) msgs.push_back(&m);
  pl.ohdr = append(f, object_header(msgs));
  return pl;
}

// Superblock version 0 at the base, pointing at the root group.
void write_superblock(ns_h5* f, const Placed& root) {
  Bytes b;
  put_bytes(b, kSig, 8);
  put(b, 0, 1);  // superblock version
  put(b, 0, 1);  // free-space storage version
  put(b, 0, 1);  // root group symbol table entry version
  put(b, 0, 1);
  put(b, 0, 1);  // shared header message format version
  put(b, 8, 1);  // size of offsets
  put(b, 8, 1);  // size of lengths
  put(b, 0, 1);
  put(b, kLeafK, 2);
  put(b, kNodeK, 2);
  put(b, 0, 4);  // file consistency flags
  put(b, f->base, 8);
  put(b, kUndef, 8);             // no free-space information
  put(b, f->base + f->end, 8);   // end of file, counted from the start of the file
  put(b, kUndef, 8);             // no driver information
  put(b, 0, 8);                  // root: link name offset
  put(b, root.ohdr, 8);
  put(b, 1, 4);
  put(b, 0, 4);
  put(b, root.btree, 8);
  put(b, root.heap, 8);
  if (fseeko(f->fp, (off_t)f->base, SEEK_SET) != 0 || std::fwrite(b.data(), 1, b.size(), f->fp) != b.size())
    throw IoError{"write failed"};
}

void flush(ns_h5* f) {
  const Placed root = write_node(f, f->root);
  write_superblock(f, root);
  if (std::fflush(f->fp) != 0) throw IoError{"write failed"};
  f->dirty = false;
}

bool host_little_endian() {
  const uint16_t one = 1;
  uint8_t b;
  std::memcpy(&b, &one, 1);
  return b == 1;
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
namespace {

thread_local std::string g_open_err;  // why the last ns_h5_create / ns_h5_open of this thread failed

template <class F>
int guarded(ns_h5* f, F&& body) {
  try {
    return body();
  } catch (const IoError& e) {
    if (f) f->err = e.what;
    return NS_ERR_IO;
  } catch (const std::bad_alloc&) {
    if (f) f->err = "out of host memory";
    return NS_ERR_NOMEM;
  }
}

int fail_h5(ns_h5* f, int code, const char* msg) {
  if (f) f->err = msg;
  return code;
}

std::vector<uint64_t> file_dims(int rank, const long long* dims) {
  std::vector<uint64_t> d(rank);
  for (int i = 0; i < rank; ++i) d[rank - 1 - i] = (uint64_t)dims[i];  // Fortran order -> file order
  return d;
}

}  // namespace

extern "C" {

int ns_h5_create(const char* path, int overwrite, ns_h5** out) {
  if (!path || !out) return NS_ERR_ARG;
  *out = nullptr;
  if (!overwrite) {
    if (std::FILE* e = std::fopen(path, "rb")) {
      std::fclose(e);
      g_open_err = "file exists";
      return NS_ERR_IO;
    }
  }
  auto* f = new ns_h5();
  f->fp = std::fopen(path, "w+b");
  if (!f->fp) {
    delete f;
    g_open_err = "cannot create the file";
    return NS_ERR_IO;
  }
  f->writable = true;
  f->root.group = true;
  f->end = 96;  // the superblock
  f->dirty = true;
  const int st = guarded(f, [&]() -> int {
    flush(f);
    return NS_OK;
  });
  if (st != NS_OK) {
    g_open_err = f->err;
    std::fclose(f->fp);
    delete f;
    return st;
  }
  *out = f;
  return NS_OK;
}

int ns_h5_open(const char* path, int writable, ns_h5** out) {
  if (!path || !out) return NS_ERR_ARG;
  *out = nullptr;
  auto* f = new ns_h5();
  f->fp = std::fopen(path, writable ? "r+b" : "rb");
  if (!f->fp) {
    delete f;
    g_open_err = "cannot open the file";
    return NS_ERR_IO;
  }
  f->writable = writable != 0;
  const int st = guarded(f, [&]() -> int {
    read_file(f);
    return NS_OK;
  });
  if (st != NS_OK) {
    g_open_err = f->err;
    std::fclose(f->fp);
    delete f;
    return st;
  }
  *out = f;
  return NS_OK;
}

const char* ns_h5_last_error(const ns_h5* f) { return f ? f->err.c_str() : g_open_err.c_str(); }

int ns_h5_flush(ns_h5* f) {
  if (!f) return NS_ERR_ARG;
  if (!f->writable || !f->dirty) return NS_OK;
  return guarded(f, [&]() -> int {
    flush(f);
    return NS_OK;
  });
}

int ns_h5_close(ns_h5* f) {
  if (!f) return NS_ERR_ARG;
  int st = ns_h5_flush(f);
  if (std::fclose(f->fp) != 0 && st == NS_OK) st = NS_ERR_IO;
  if (st != NS_OK) g_open_err = f->err.empty() ? "close failed" : f->err;
  delete f;
  return st;
}

int ns_h5_group(ns_h5* f, const char* path) {
  if (!f || !path) return NS_ERR_ARG;
  if (!f->writable) return fail_h5(f, NS_ERR_ARG, "file opened read-only");
  std::string leaf;
  Node* par = parent_of(f->root, path, leaf);
  if (!par || leaf.empty()) return fail_h5(f, NS_ERR_ARG, "the parent group does not exist");
  if (par->kids.count(leaf)) return fail_h5(f, NS_ERR_ARG, "an object of that name exists");
  auto g = std::make_unique<Node>();
  g->group = true;
  par->kids[leaf] = std::move(g);
  f->dirty = true;
  return NS_OK;
}

static int set_attr_common(ns_h5* f, const char* obj, const char* name, const Bytes& type, const Bytes& space,
                           const void* val, size_t nval) {
  if (!f || !name || !*name) return NS_ERR_ARG;
  if (!f->writable) return fail_h5(f, NS_ERR_ARG, "file opened read-only");
  Node* n = lookup(f->root, obj ? obj : "/");
  if (!n) return fail_h5(f, NS_ERR_ARG, "no such object");
  return guarded(f, [&]() -> int {
    set_attr(*n, attr_msg(name, type, space, val, nval), name);
    f->dirty = true;
    return NS_OK;
  });
}

int ns_h5_attr_int(ns_h5* f, const char* obj, const char* name, int value) {
  uint8_t v[4];
  for (int i = 0; i < 4; ++i) v[i] = (uint8_t)((uint32_t)value >> (8 * i));
  return set_attr_common(f, obj, name, enc_int32_type(), enc_dataspace({1}), v, 4);
}

int ns_h5_attr_double(ns_h5* f, const char* obj, const char* name, double value) {
  uint64_t r;
  std::memcpy(&r, &value, 8);
  uint8_t v[8];
  for (int i = 0; i < 8; ++i) v[i] = (uint8_t)(r >> (8 * i));
  return set_attr_common(f, obj, name, enc_double_type(), enc_dataspace({1}), v, 8);
}

int ns_h5_attr_string(ns_h5* f, const char* obj, const char* name, const char* value) {
  if (!value) return NS_ERR_ARG;
  const size_t n = std::strlen(value) + 1;
  return set_attr_common(f, obj, name, enc_string_type(n), enc_dataspace({}), value, n);
}

int ns_h5_write_double(ns_h5* f, const char* path, int rank, const long long* dims, const double* data) {
  if (!f || !path || rank < 1 || rank > 32 || !dims) return NS_ERR_ARG;
  if (!f->writable) return fail_h5(f, NS_ERR_ARG, "file opened read-only");
  uint64_t n = 1;
  for (int i = 0; i < rank; ++i) {
    if (dims[i] < 0) return fail_h5(f, NS_ERR_ARG, "negative dimension");
    n *= (uint64_t)dims[i];
  }
  if (n && !data) return NS_ERR_ARG;
  std::string leaf;
  Node* par = parent_of(f->root, path, leaf);
  if (!par || leaf.empty()) return fail_h5(f, NS_ERR_ARG, "the parent group does not exist");
  if (par->kids.count(leaf)) return fail_h5(f, NS_ERR_ARG, "an object of that name exists");
  return guarded(f, [&]() -> int {
    uint64_t addr = kUndef;
    if (n) {
      if (host_little_endian()) {
        addr = append(f, data, n * 8);
      } else {
        Bytes b;
        b.reserve(n * 8);
        for (uint64_t i = 0; i < n; ++i) {
          uint64_t r;
          std::memcpy(&r, &data[i], 8);
          put(b, r, 8);
        }
        addr = append(f, b);
      }
    }
    auto d = std::make_unique<Node>();
    d->msgs.push_back(Msg{MSG_FILL, 1, {1, 2, 2, 1, 0, 0, 0, 0}});  // allocation late, fill if set, default value
    d->msgs.push_back(Msg{MSG_DATATYPE, 1, enc_double_type()});
    d->msgs.push_back(Msg{MSG_DATASPACE, 0, enc_dataspace(file_dims(rank, dims))});
    Msg lay{MSG_LAYOUT, 0, {3, 1}};
    put(lay.data, addr, 8);
    put(lay.data, n * 8, 8);
    d->msgs.push_back(std::move(lay));
    par->kids[leaf] = std::move(d);
    f->dirty = true;
    return NS_OK;
  });
}

int ns_h5_dims(ns_h5* f, const char* path, int* rank, long long* dims) {
  if (!f || !path || !rank || !dims) return NS_ERR_ARG;
  Node* n = lookup(f->root, path);
  if (!n || n->group) return fail_h5(f, NS_ERR_ARG, "no such dataset");
  return guarded(f, [&]() -> int {
    const std::vector<uint64_t> d = decode_dataspace(find_msg(*n, MSG_DATASPACE)->data);
    if (d.size() > 32) throw IoError{"rank above 32"};
    *rank = (int)d.size();
    for (size_t i = 0; i < d.size(); ++i) dims[i] = (long long)d[d.size() - 1 - i];  // Fortran order
    return NS_OK;
  });
}

int ns_h5_read_double(ns_h5* f, const char* path, int rank, const long long* dims, double* out) {
  if (!f || !path || !dims || !out || rank < 0 || rank > 32) return NS_ERR_ARG;
  Node* n = lookup(f->root, path);
  if (!n || n->group) return fail_h5(f, NS_ERR_ARG, "no such dataset");
  return guarded(f, [&]() -> int {
    const std::vector<uint64_t> d = decode_dataspace(find_msg(*n, MSG_DATASPACE)->data);
    if (d != file_dims(rank, dims)) return fail_h5(f, NS_ERR_SHAPE, "the dataset's dims differ from the buffer's");
    const Type t = decode_datatype(find_msg(*n, MSG_DATATYPE)->data);
    if (t.cls == 3) return fail_h5(f, NS_ERR_ARG, "a string dataset");
    uint64_t cnt = 1;
    for (uint64_t x : d) cnt *= x;
    if (t.cls == 1 && t.size == 8 && !t.big && host_little_endian()) {
      const Msg* lay = find_msg(*n, MSG_LAYOUT);
      // contiguous doubles straight into the caller's buffer
      if (lay->data.size() >= 18 && lay->data[0] == 3 && lay->data[1] == 1 && get(&lay->data[2], 8) != kUndef) {
        if (get(&lay->data[10], 8) < cnt * 8) throw IoError{"contiguous storage smaller than the dataspace"};
        if (cnt) read_at(f, get(&lay->data[2], 8), out, cnt * 8);
        return NS_OK;
      }
    }
    const Bytes raw = dataset_bytes(f, *n, cnt * t.size);
    to_double(t, raw.data(), cnt, out);
    return NS_OK;
  });
}

static int get_attr(ns_h5* f, const char* obj, const char* name, Attr& a) {
  if (!f || !name) return NS_ERR_ARG;
  Node* n = lookup(f->root, obj ? obj : "/");
  if (!n) return fail_h5(f, NS_ERR_ARG, "no such object");
  return guarded(f, [&]() -> int {
    for (const Msg& m : n->msgs)
      if (m.type == MSG_ATTR) {
        Attr x = decode_attr(m.data);
        if (x.name == name) {
          a = std::move(x);
          return NS_OK;
        }
      }
    return fail_h5(f, NS_ERR_ARG, "no such attribute");
  });
}

int ns_h5_get_attr_int(ns_h5* f, const char* obj, const char* name, long long* value) {
  if (!value) return NS_ERR_ARG;
  Attr a;
  int st = get_attr(f, obj, name, a);
  if (st) return st;
  if (a.type.cls != 0 || a.value.size() < a.type.size) return fail_h5(f, NS_ERR_ARG, "not an integer attribute");
  double v;
  to_double(a.type, a.value.data(), 1, &v);
  *value = (long long)v;
  return NS_OK;
}

int ns_h5_get_attr_double(ns_h5* f, const char* obj, const char* name, double* value) {
  if (!value) return NS_ERR_ARG;
  Attr a;
  int st = get_attr(f, obj, name, a);
  if (st) return st;
  if (a.type.cls == 3 || a.value.size() < a.type.size) return fail_h5(f, NS_ERR_ARG, "not a numeric attribute");
  to_double(a.type, a.value.data(), 1, value);
  return NS_OK;
}

int ns_h5_get_attr_string(ns_h5* f, const char* obj, const char* name, char* buf, int buflen) {
  if (!buf || buflen < 1) return NS_ERR_ARG;
  Attr a;
  int st = get_attr(f, obj, name, a);
  if (st) return st;
  if (a.type.cls != 3) return fail_h5(f, NS_ERR_ARG, "not a string attribute");
  const size_t len = strnlen(reinterpret_cast<const char*>(a.value.data()), a.value.size());
  if (len + 1 > (size_t)buflen) return fail_h5(f, NS_ERR_ARG, "buffer too short");
  std::memcpy(buf, a.value.data(), len);
  buf[len] = 0;
  return NS_OK;
}

int ns_h5_members(ns_h5* f, const char* group, char* buf, long long buflen, long long* needed) {
  if (!f || !group) return NS_ERR_ARG;
  Node* n = lookup(f->root, group);
  if (!n || !n->group) return fail_h5(f, NS_ERR_ARG, "no such group");
  std::string s;
  for (auto& kv : n->kids) s += kv.first + (kv.second->group ? "/\n" : "\n");
  if (needed) *needed = (long long)s.size() + 1;
  if (!buf) return NS_OK;
  if ((long long)s.size() + 1 > buflen) return fail_h5(f, NS_ERR_ARG, "buffer too short");
  std::memcpy(buf, s.c_str(), s.size() + 1);
  return NS_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Session state as a reference snapshot (big_periodic_3D.f90:630-651) and the
// restart from one (:309-324)
// ---------------------------------------------------------------------------
namespace {

const char* const kStateNames[7] = {"u", "v", "w", "p", "rhs_x_previous", "rhs_y_previous", "rhs_z_previous"};

// Fortran extents of state field q (u, v, w, p, then the three histories).
void state_dims(const ns_config& c, int q, long long d[3]) {
  const int f = q < 4 ? q : q - 4;
  d[0] = c.nx + (f == 0 ? 1 : 2);
  d[1] = c.ny + (f == 1 ? 1 : 2);
  d[2] = c.nz + (f == 2 ? 1 : 2);
}

const char* scheme_name(int s) { return s == NS_EULER ? "Euler" : (s == NS_AB2 ? "AB2" : "AB2-CN"); }

}  // namespace

extern "C" {

int ns_h5_write_state(ns_handle* h, const char* path, double time, int time_step, int overwrite) {
  if (!h || !path) return NS_ERR_ARG;
  const ns_config& c = h->cfg;
  ns_h5* f = nullptr;
  int st = ns_h5_create(path, overwrite, &f);
  if (st) return ns::api_fail(h, st, std::string("ns_h5_write_state: ") + ns_h5_last_error(nullptr));
  auto bail = [&](int code) {
    const std::string why = std::string("ns_h5_write_state: ") + ns_h5_last_error(f);
    ns_h5_close(f);
    return ns::api_fail(h, code, why);
  };
  // the root attributes of :637-642, in that order; ny and nz only when the box is not cubic
  if ((st = ns_h5_attr_int(f, "/", "nx", c.nx))) return bail(st);
  if (c.ny != c.nx || c.nz != c.nx) {
    if ((st = ns_h5_attr_int(f, "/", "ny", c.ny))) return bail(st);
    if ((st = ns_h5_attr_int(f, "/", "nz", c.nz))) return bail(st);
  }
  if ((st = ns_h5_attr_double(f, "/", "dt", c.dt))) return bail(st);
  if ((st = ns_h5_attr_double(f, "/", "nu", c.nu))) return bail(st);
  if ((st = ns_h5_attr_string(f, "/", "time_scheme", scheme_name(c.scheme)))) return bail(st);
  if ((st = ns_h5_attr_int(f, "/", "time_step", time_step))) return bail(st);
  if ((st = ns_h5_attr_double(f, "/", "time", time))) return bail(st);
  // one field at a time through one host buffer
  std::vector<double> buf;
  try {
    buf.resize((size_t)(c.nx + 2) * (c.ny + 2) * (c.nz + 2));
  } catch (const std::bad_alloc&) {
    ns_h5_close(f);
    return ns::api_fail(h, NS_ERR_NOMEM, "ns_h5_write_state: out of host memory");
  }
  for (int q = 0; q < 7; ++q) {
    double* dst[7] = {};
    dst[q] = buf.data();
    if ((st = ns_get_state(h, dst[0], dst[1], dst[2], dst[3], dst[4], dst[5], dst[6]))) {
      ns_h5_close(f);
      return st;
    }
    long long d[3];
    state_dims(c, q, d);
    if ((st = ns_h5_write_double(f, kStateNames[q], 3, d, buf.data()))) return bail(st);
  }
  if ((st = ns_h5_close(f))) return ns::api_fail(h, st, std::string("ns_h5_write_state: ") + ns_h5_last_error(nullptr));
  return NS_OK;
}

int ns_h5_read_state(ns_handle* h, const char* path, double* time, int* time_step) {
  if (!h || !path) return NS_ERR_ARG;
  const ns_config& c = h->cfg;
  ns_h5* f = nullptr;
  int st = ns_h5_open(path, 0, &f);
  if (st) return ns::api_fail(h, st, std::string("ns_h5_read_state: ") + ns_h5_last_error(nullptr));
  auto bail = [&](int code) {
    const std::string why = std::string("ns_h5_read_state: ") + ns_h5_last_error(f);
    ns_h5_close(f);
    return ns::api_fail(h, code, why);
  };
  // u, v, w, p always; the history when all three are present (a snapshot
  // of :644-650), else the next step is the Euler start (the init file of :296-301)
  bool hist = true;
  for (int q = 4; q < 7; ++q) {
    int r;
    long long d[32];
    hist = hist && ns_h5_dims(f, kStateNames[q], &r, d) == NS_OK;
  }
  std::vector<std::vector<double>> fields(hist ? 7 : 4);
  for (size_t q = 0; q < fields.size(); ++q) {
    long long d[3];
    state_dims(c, (int)q, d);
    try {
      fields[q].resize((size_t)(d[0] * d[1] * d[2]));
    } catch (const std::bad_alloc&) {
      ns_h5_close(f);
      return ns::api_fail(h, NS_ERR_NOMEM, "ns_h5_read_state: out of host memory");
    }
    if ((st = ns_h5_read_double(f, kStateNames[q], 3, d, fields[q].data()))) return bail(st);
  }
  if (time) {
    *time = 0;
    ns_h5_get_attr_double(f, "/", "time", time);
  }
  if (time_step) {
    long long ts = 0;
    ns_h5_get_attr_int(f, "/", "time_step", &ts);
    *time_step = (int)ts;
  }
  ns_h5_close(f);
  return ns_set_state(h, fields[0].data(), fields[1].data(), fields[2].data(), fields[3].data(),
                      hist ? fields[4].data() : nullptr, hist ? fields[5].data() : nullptr,
                      hist ? fields[6].data() : nullptr);
}

}  // extern "C"
