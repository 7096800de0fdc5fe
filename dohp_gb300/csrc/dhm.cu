// DHM checkpoint / visualization files (src/viewer/dhm.c, src/fs/impls/cont/contviewdhm.c): function spaces and vectors
// in HDF5 with the reference's group layout
//   /dohp/type   committed datatypes (Units_type, Time_type, BoundingBox_type, FS_type, Vec_type)
//   /dohp/mesh   /<mesh name>/000: the mesh (here the block mesh itself: vertex coordinates, hex connectivity,
//                generator extents; the reference stores a MOAB file name there)
//   /dohp/fs     /<fs name>: one FS record (compound FS_type: names of the per-entity tags, mesh path, time, state,
//                subdomain count, bounding box, block size); the tags it names (element degrees, boundary status)
//                are datasets in the mesh group
//   /dohp/step   /NNN: one group per time step with attribute "time" (Time_type {value, units}) and one dataset per
//                vector, [closure nodes][bs] FP64 with attribute "meta" (Vec_type {fs, time, units, internal_state})
// Simplifications against the reference, each because the library it relies on is absent: strings are fixed-length
// (no variable-length strings, which need HDF5's global heap), references are path strings (object and region
// references), and the mesh is stored in the file instead of a MOAB file beside it.
//
// The file is written from the public HDF5 file format specification (version 2 superblock, version 2 object headers
// with compact link storage, contiguous datasets, version 3 attribute messages, Jenkins lookup3 checksums), by a writer
// that lays out the whole tree when the viewer is destroyed; the reader parses that subset of the format.
#include <stddef.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "internal.h"

using namespace dgb;

namespace dgb {

// Bob Jenkins' lookup3 hashlittle (public domain, 2006): the checksum of HDF5 metadata blocks
uint32_t lookup3(const uint8_t *k, size_t length, uint32_t initval) {
  auto rot = [](uint32_t x, int r) { return (x << r) | (x >> (32 - r)); };
  uint32_t a, b, c;
  a = b = c = 0xdeadbeefu + (uint32_t)length + initval;
  auto word = [&](size_t i) { return (uint32_t)k[i] | ((uint32_t)k[i + 1] << 8) | ((uint32_t)k[i + 2] << 16) | ((uint32_t)k[i + 3] << 24); };
  while (length > 12) {
    a += word(0), b += word(4), c += word(8);
    a -= c; a ^= rot(c, 4);  c += b;
    b -= a; b ^= rot(a, 6);  a += c;
    c -= b; c ^= rot(b, 8);  b += a;
    a -= c; a ^= rot(c, 16); c += b;
    b -= a; b ^= rot(a, 19); a += c;
    c -= b; c ^= rot(b, 4);  b += a;
    length -= 12, k += 12;
  }
  switch (length) {
    case 12: c += (uint32_t)k[11] << 24; /* fall through */
    case 11: c += (uint32_t)k[10] << 16; /* fall through */
    case 10: c += (uint32_t)k[9] << 8;   /* fall through */
    case 9:  c += k[8];                  /* fall through */
    case 8:  b += (uint32_t)k[7] << 24;  /* fall through */
    case 7:  b += (uint32_t)k[6] << 16;  /* fall through */
    case 6:  b += (uint32_t)k[5] << 8;   /* fall through */
    case 5:  b += k[4];                  /* fall through */
    case 4:  a += (uint32_t)k[3] << 24;  /* fall through */
    case 3:  a += (uint32_t)k[2] << 16;  /* fall through */
    case 2:  a += (uint32_t)k[1] << 8;   /* fall through */
    case 1:  a += k[0]; break;
    case 0: return c;
  }
  c ^= b; c -= rot(b, 14);
  a ^= c; a -= rot(c, 11);
  b ^= a; b -= rot(a, 25);
  c ^= b; c -= rot(b, 16);
  a ^= c; a -= rot(c, 4);
  b ^= a; b -= rot(a, 14);
  c ^= b; c -= rot(b, 24);
  return c;
}

}  // namespace dgb

namespace {

constexpr uint64_t UNDEF = ~0ull;

struct Bytes {
  std::vector<uint8_t> v;
  void u8(uint32_t x) { v.push_back((uint8_t)x); }
  void u16(uint32_t x) { u8(x & 0xff), u8((x >> 8) & 0xff); }
  void u32(uint32_t x) { u16(x & 0xffff), u16(x >> 16); }
  void u64(uint64_t x) { u32((uint32_t)x), u32((uint32_t)(x >> 32)); }
  void raw(const void *p, size_t n) { v.insert(v.end(), (const uint8_t *)p, (const uint8_t *)p + n); }
  void str0(const std::string &s) { raw(s.data(), s.size()), u8(0); }
  void put_u64(size_t at, uint64_t x) {
    for (int i = 0; i < 8; i++) v[at + i] = (uint8_t)(x >> (8 * i));
  }
};

// ------------------------------------------------------------------------------------------------- datatypes
struct Type {
  std::vector<uint8_t> enc;  // the datatype message body
  uint32_t size = 0;         // bytes per element
};

Type t_f64() {
  Bytes b;
  b.u8((1 << 4) | 1);          // version 1, class 1 (floating point)
  b.u8(0x20), b.u8(63), b.u8(0);  // little endian, implied mantissa MSB; sign at bit 63
  b.u32(8);
  b.u16(0), b.u16(64);         // bit offset, precision
  b.u8(52), b.u8(11), b.u8(0), b.u8(52);  // exponent location and size, mantissa location and size
  b.u32(1023);                 // exponent bias
  return {b.v, 8};
}

Type t_int(int bytes) {
  Bytes b;
  b.u8((1 << 4) | 0);  // version 1, class 0 (fixed point)
  b.u8(0x08), b.u8(0), b.u8(0);  // little endian, signed
  b.u32((uint32_t)bytes);
  b.u16(0), b.u16((uint32_t)(8 * bytes));
  return {b.v, (uint32_t)bytes};
}

Type t_str(int len) {
  Bytes b;
  b.u8((1 << 4) | 3);  // version 1, class 3 (string)
  b.u8(0x00), b.u8(0), b.u8(0);  // null terminated, ASCII
  b.u32((uint32_t)len);
  return {b.v, (uint32_t)len};
}

Type t_array(const Type &base, std::vector<uint32_t> dims) {
  Bytes b;
  b.u8((3 << 4) | 10);  // version 3, class 10 (array)
  b.u8(0), b.u8(0), b.u8(0);
  uint32_t n = 1;
  for (uint32_t d : dims) n *= d;
  b.u32(n * base.size);
  b.u8((uint32_t)dims.size());
  for (uint32_t d : dims) b.u32(d);
  b.raw(base.enc.data(), base.enc.size());
  return {b.v, n * base.size};
}

struct Member {
  std::string name;
  uint32_t offset;
  Type type;
};

Type t_compound(const std::vector<Member> &m, uint32_t size) {
  Bytes b;
  b.u8((3 << 4) | 6);  // version 3, class 6 (compound)
  b.u16((uint32_t)m.size()), b.u8(0);
  b.u32(size);
  const int ob = size < 256 ? 1 : size < 65536 ? 2 : 4;  // bytes of a member offset (enough for the size)
  for (const Member &x : m) {
    b.str0(x.name);
    for (int i = 0; i < ob; i++) b.u8((x.offset >> (8 * i)) & 0xff);
    b.raw(x.type.enc.data(), x.type.enc.size());
  }
  return {b.v, size};
}

// ------------------------------------------------------------------------------------------------- the tree
struct Attr {
  std::string name;
  Type type;
  std::vector<uint64_t> dims;  // empty: scalar
  std::vector<uint8_t> data;
};

struct Node {
  enum Kind { GROUP, DATASET, NAMED_TYPE } kind = GROUP;
  std::vector<std::pair<std::string, std::shared_ptr<Node>>> links;  // groups: children in insertion order
  Type type;                                                          // datasets and named types
  std::vector<uint64_t> dims;
  std::vector<uint8_t> data;
  std::vector<Attr> attrs;
  // layout
  uint64_t addr = 0, data_addr = UNDEF;
  std::vector<uint8_t> header;
};

std::vector<uint8_t> dataspace_msg(const std::vector<uint64_t> &dims) {
  Bytes b;
  b.u8(2), b.u8((uint32_t)dims.size()), b.u8(0), b.u8(dims.empty() ? 0 : 1);  // version 2, rank, no max dims, scalar / simple
  for (uint64_t d : dims) b.u64(d);
  return b.v;
}

std::vector<uint8_t> attr_msg(const Attr &a) {
  Bytes b;
  const std::vector<uint8_t> ds = dataspace_msg(a.dims);
  b.u8(3), b.u8(0);  // version 3, flags
  b.u16((uint32_t)a.name.size() + 1), b.u16((uint32_t)a.type.enc.size()), b.u16((uint32_t)ds.size());
  b.u8(0);  // ASCII name
  b.str0(a.name);
  b.raw(a.type.enc.data(), a.type.enc.size());
  b.raw(ds.data(), ds.size());
  b.raw(a.data.data(), a.data.size());
  return b.v;
}

// one version 2 object header; addresses of children and data must be assigned (their values only; sizes are fixed)
std::vector<uint8_t> object_header(const Node &n) {
  Bytes m;  // messages
  auto msg = [&](uint32_t type, const std::vector<uint8_t> &body, uint32_t flags = 0) {
    m.u8(type), m.u16((uint32_t)body.size()), m.u8(flags);
    m.raw(body.data(), body.size());
  };
  if (n.kind == Node::GROUP) {
    Bytes li;  // link info: version 0, no creation order, no dense storage
    li.u8(0), li.u8(0), li.u64(UNDEF), li.u64(UNDEF);
    msg(0x02, li.v);
    Bytes gi;  // group info: version 0, defaults
    gi.u8(0), gi.u8(0);
    msg(0x0A, gi.v);
    for (const auto &l : n.links) {
      Bytes lk;  // link: version 1, hard link, 1-byte name length
      lk.u8(1), lk.u8(0), lk.u8((uint32_t)l.first.size());
      lk.raw(l.first.data(), l.first.size());
      lk.u64(l.second->addr);
      msg(0x06, lk.v);
    }
  } else if (n.kind == Node::NAMED_TYPE) {
    msg(0x03, n.type.enc, 0x01);  // constant datatype message
  } else {
    msg(0x01, dataspace_msg(n.dims));
    msg(0x03, n.type.enc, 0x01);
    Bytes fv;  // fill value: version 3, allocation early, never written, undefined
    fv.u8(3), fv.u8(0x01 | (2 << 2) | 0x10);
    msg(0x05, fv.v, 0x01);
    Bytes ly;  // data layout: version 3, contiguous
    ly.u8(3), ly.u8(1), ly.u64(n.data_addr), ly.u64(n.data.size());
    msg(0x08, ly.v);
  }
  for (const Attr &a : n.attrs) msg(0x0C, attr_msg(a));
  Bytes h;
  h.raw("OHDR", 4);
  h.u8(2), h.u8(0x02);  // version 2; chunk size field of 4 bytes
  h.u32((uint32_t)m.v.size());
  h.raw(m.v.data(), m.v.size());
  h.u32(lookup3(h.v.data(), h.v.size(), 0));
  return h.v;
}

void collect(const std::shared_ptr<Node> &n, std::vector<Node *> &out) {
  out.push_back(n.get());
  for (const auto &l : n->links) collect(l.second, out);
}

// lay out and write the tree: superblock, object headers (pre-order), then dataset data (8-byte aligned)
dErr write_file(const std::string &path, const std::shared_ptr<Node> &root) {
  std::vector<Node *> nodes;
  collect(root, nodes);
  for (Node *n : nodes) n->header = object_header(*n);  // sizes do not depend on the address values
  uint64_t at = 48;
  for (Node *n : nodes) n->addr = at, at += n->header.size();
  for (Node *n : nodes)
    if (n->kind == Node::DATASET && !n->data.empty()) {
      at = (at + 7) & ~7ull;
      n->data_addr = at, at += n->data.size();
    }
  for (Node *n : nodes) n->header = object_header(*n);
  Bytes sb;
  sb.raw("\x89HDF\r\n\x1a\n", 8);
  sb.u8(2), sb.u8(8), sb.u8(8), sb.u8(0);  // version 2, 8-byte offsets and lengths, consistency flags
  sb.u64(0), sb.u64(UNDEF), sb.u64(at), sb.u64(root->addr);
  sb.u32(lookup3(sb.v.data(), sb.v.size(), 0));
  std::vector<uint8_t> file(at, 0);
  std::copy(sb.v.begin(), sb.v.end(), file.begin());
  for (Node *n : nodes) {
    std::copy(n->header.begin(), n->header.end(), file.begin() + n->addr);
    if (n->data_addr != UNDEF) std::copy(n->data.begin(), n->data.end(), file.begin() + n->data_addr);
  }
  FILE *f = fopen(path.c_str(), "wb");
  if (!f) return set_error("DHM: cannot open %s for writing", path.c_str());
  const size_t w = fwrite(file.data(), 1, file.size(), f);
  fclose(f);
  if (w != file.size()) return set_error("DHM: short write to %s", path.c_str());
  return 0;
}

// ------------------------------------------------------------------------------------------------- reading
struct Reader {
  std::vector<uint8_t> f;
  uint64_t u(uint64_t at, int n) const {
    uint64_t x = 0;
    for (int i = 0; i < n; i++) x |= (uint64_t)f.at(at + i) << (8 * i);
    return x;
  }
};

// decode a datatype message body: class and element size (the parts the reader needs)
void type_info(const uint8_t *p, int *cls, uint32_t *size) {
  *cls = p[0] & 0x0f;
  *size = (uint32_t)p[4] | ((uint32_t)p[5] << 8) | ((uint32_t)p[6] << 16) | ((uint32_t)p[7] << 24);
}

dErr parse_object(Reader &R, uint64_t addr, std::shared_ptr<Node> &out, int depth) {
  if (depth > 32) return set_error("DHM: objects nested too deep");
  if (addr + 10 > R.f.size() || memcmp(&R.f[addr], "OHDR", 4) != 0) return set_error("DHM: no object header at %llu", (unsigned long long)addr);
  const int flags = R.f[addr + 5];
  if (R.f[addr + 4] != 2) return set_error("DHM: object header version %d", R.f[addr + 4]);
  if (flags & 0x30) return set_error("DHM: object header with times or attribute phase values");
  const int csz = 1 << (flags & 3);
  const uint64_t chunk = R.u(addr + 6, csz), m0 = addr + 6 + csz, end = m0 + chunk;
  if (end + 4 > R.f.size()) return set_error("DHM: object header beyond the end of the file");
  if (lookup3(&R.f[addr], end - addr, 0) != (uint32_t)R.u(end, 4)) return set_error("DHM: object header checksum mismatch");
  auto n = std::make_shared<Node>();
  n->kind = Node::GROUP;
  bool has_layout = false, has_type = false, has_space = false;
  uint64_t dsize = 0;
  for (uint64_t p = m0; p + 4 <= end;) {
    const int type = R.f[p];
    const uint64_t size = R.u(p + 1, 2), body = p + 4;
    if (body + size > end) return set_error("DHM: message beyond its object header");
    const uint8_t *b = &R.f[body];
    if (type == 0x06) {  // link
      const int lf = b[1];
      if (lf & 0x1c) return set_error("DHM: unsupported link flags");
      const int lsz = 1 << (lf & 3);
      uint64_t nl = 0;
      for (int i = 0; i < lsz; i++) nl |= (uint64_t)b[2 + i] << (8 * i);
      std::string name((const char *)b + 2 + lsz, nl);
      std::shared_ptr<Node> child;
      DCHK(parse_object(R, R.u(body + 2 + lsz + nl, 8), child, depth + 1));
      n->links.push_back({name, child});
    } else if (type == 0x01) {  // dataspace (version 2)
      if (b[0] != 2) return set_error("DHM: dataspace version %d", b[0]);
      n->dims.clear();
      for (int i = 0; i < b[1]; i++) n->dims.push_back(R.u(body + 4 + 8 * i, 8));
      has_space = true;
    } else if (type == 0x03) {
      n->type.enc.assign(b, b + size);
      int cls;
      type_info(b, &cls, &n->type.size);
      has_type = true;
    } else if (type == 0x08) {  // layout (version 3, contiguous)
      if (b[0] != 3 || b[1] != 1) return set_error("DHM: unsupported data layout");
      n->data_addr = R.u(body + 2, 8);
      dsize = R.u(body + 10, 8);
      has_layout = true;
    } else if (type == 0x0C) {  // attribute (version 3)
      if (b[0] != 3) return set_error("DHM: attribute message version %d", b[0]);
      const uint64_t nsz = R.u(body + 2, 2), tsz = R.u(body + 4, 2), ssz = R.u(body + 6, 2);
      Attr a;
      a.name.assign((const char *)b + 9, nsz ? nsz - 1 : 0);
      a.type.enc.assign(b + 9 + nsz, b + 9 + nsz + tsz);
      int cls;
      type_info(b + 9 + nsz, &cls, &a.type.size);
      const uint8_t *s = b + 9 + nsz + tsz;
      for (int i = 0; i < s[1]; i++) a.dims.push_back(R.u(body + 9 + nsz + tsz + 4 + 8 * i, 8));
      uint64_t cnt = 1;
      for (uint64_t d : a.dims) cnt *= d;
      const uint64_t dat = body + 9 + nsz + tsz + ssz;
      if (dat + cnt * a.type.size > body + size) return set_error("DHM: attribute data beyond its message");
      a.data.assign(&R.f[dat], &R.f[dat] + cnt * a.type.size);
      n->attrs.push_back(a);
    }
    p = body + size;
  }
  if (has_layout) {
    n->kind = Node::DATASET;
    if (!has_type || !has_space) return set_error("DHM: dataset without datatype or dataspace");
    if (dsize && (n->data_addr == UNDEF || n->data_addr + dsize > R.f.size())) return set_error("DHM: dataset data beyond the file");
    if (dsize) n->data.assign(&R.f[n->data_addr], &R.f[n->data_addr] + dsize);
  } else if (has_type && !has_space) {
    n->kind = Node::NAMED_TYPE;
  }
  out = n;
  return 0;
}

dErr read_file(const std::string &path, std::shared_ptr<Node> &root) {
  FILE *fp = fopen(path.c_str(), "rb");
  if (!fp) return set_error("DHM: cannot open %s", path.c_str());
  Reader R;
  fseek(fp, 0, SEEK_END);
  const long len = ftell(fp);
  fseek(fp, 0, SEEK_SET);
  R.f.resize(len > 0 ? (size_t)len : 0);
  const size_t got = R.f.empty() ? 0 : fread(R.f.data(), 1, R.f.size(), fp);
  fclose(fp);
  if (got != R.f.size() || R.f.size() < 48 || memcmp(R.f.data(), "\x89HDF\r\n\x1a\n", 8) != 0) return set_error("DHM: %s is not an HDF5 file", path.c_str());
  if (R.f[8] != 2 || R.f[9] != 8 || R.f[10] != 8) return set_error("DHM: superblock version %d (version 2 with 8-byte addresses expected)", R.f[8]);
  if (lookup3(R.f.data(), 44, 0) != (uint32_t)R.u(44, 4)) return set_error("DHM: superblock checksum mismatch");
  return parse_object(R, R.u(36, 8), root, 0);
}

std::shared_ptr<Node> child(const std::shared_ptr<Node> &g, const std::string &name) {
  if (!g) return nullptr;
  for (auto &l : g->links)
    if (l.first == name) return l.second;
  return nullptr;
}

std::shared_ptr<Node> lookup(const std::shared_ptr<Node> &root, const std::string &path) {
  std::shared_ptr<Node> n = root;
  size_t i = 0;
  while (n && i < path.size()) {
    while (i < path.size() && path[i] == '/') i++;
    const size_t j = path.find('/', i);
    const std::string part = path.substr(i, j == std::string::npos ? std::string::npos : j - i);
    if (!part.empty()) n = child(n, part);
    i = j == std::string::npos ? path.size() : j;
  }
  return n;
}

std::shared_ptr<Node> ensure_group(const std::shared_ptr<Node> &g, const std::string &name) {
  if (auto c = child(g, name)) return c;
  auto c = std::make_shared<Node>();
  g->links.push_back({name, c});
  return c;
}

template <typename T>
std::vector<uint8_t> bytes_of(const T *p, size_t n) {
  return std::vector<uint8_t>((const uint8_t *)p, (const uint8_t *)p + n * sizeof(T));
}

std::shared_ptr<Node> dataset(const Type &t, std::vector<uint64_t> dims, std::vector<uint8_t> data) {
  auto d = std::make_shared<Node>();
  d->kind = Node::DATASET;
  d->type = t, d->dims = std::move(dims), d->data = std::move(data);
  return d;
}

// ------------------------------------------------------------------------------------------------- DHM types
constexpr int kStr = 64;  // fixed string length of the records

struct UnitsRec {
  char dimensions[kStr];
  double scale;
};
struct TimeRec {
  double value;
  UnitsRec units;
};
struct FSRec {
  char degree[kStr], global_offset[kStr], partition[kStr], ordered_subdomain[kStr], bstatus[kStr], mesh[kStr];
  double time;
  int32_t internal_state, number_of_subdomains;
  double boundingbox[3][2];
  int32_t block_size;
};
struct VecRec {
  char fs[kStr];
  double time;
  UnitsRec units;
  int32_t internal_state;
};

Type units_type() { return t_compound({{"dimensions", offsetof(UnitsRec, dimensions), t_str(kStr)}, {"scale", offsetof(UnitsRec, scale), t_f64()}}, sizeof(UnitsRec)); }
Type time_type() { return t_compound({{"value", offsetof(TimeRec, value), t_f64()}, {"units", offsetof(TimeRec, units), units_type()}}, sizeof(TimeRec)); }
Type bbox_type() { return t_array(t_f64(), {3, 2}); }
Type fs_type() {
  return t_compound({{"degree", offsetof(FSRec, degree), t_str(kStr)},
                     {"global_offset", offsetof(FSRec, global_offset), t_str(kStr)},
                     {"partition", offsetof(FSRec, partition), t_str(kStr)},
                     {"ordered_subdomain", offsetof(FSRec, ordered_subdomain), t_str(kStr)},
                     {"bstatus", offsetof(FSRec, bstatus), t_str(kStr)},
                     {"mesh", offsetof(FSRec, mesh), t_str(kStr)},
                     {"time", offsetof(FSRec, time), t_f64()},
                     {"internal_state", offsetof(FSRec, internal_state), t_int(4)},
                     {"number_of_subdomains", offsetof(FSRec, number_of_subdomains), t_int(4)},
                     {"boundingbox", offsetof(FSRec, boundingbox), bbox_type()},
                     {"block_size", offsetof(FSRec, block_size), t_int(4)}},
                    sizeof(FSRec));
}
Type vec_type() {
  return t_compound({{"fs", offsetof(VecRec, fs), t_str(kStr)},
                     {"time", offsetof(VecRec, time), t_f64()},
                     {"units", offsetof(VecRec, units), units_type()},
                     {"internal_state", offsetof(VecRec, internal_state), t_int(4)}},
                    sizeof(VecRec));
}

void copy_str(char (&dst)[kStr], const std::string &s) {
  memset(dst, 0, kStr);
  memcpy(dst, s.data(), std::min<size_t>(s.size(), kStr - 1));
}

}  // namespace

struct _p_dViewer {
  std::string path;
  int mode = 0;  // 0 write, 1 read
  std::shared_ptr<Node> root, dohp;
  double time = 0, timescale = 1;
  std::string timeunits = "s";
  int stepnumber = -1, totalsteps = 0;
  std::map<const void *, std::string> fsname;  // name given to each dFS written
  std::map<const void *, std::string> meshname;  // group name of each dMesh written: mesh0, mesh1, ...
  int state = 0;                               // increments per object written (the reference's internal_state)
};

namespace {

std::string step_name(int k) {
  char b[16];
  snprintf(b, sizeof b, "%03d", k);
  return b;
}

// the current step group, made on first use in write mode with its "time" attribute (dViewerDHMGetStep, dhm.c:374-410)
dErr current_step(dViewer v, std::shared_ptr<Node> &step) {
  auto steps = child(v->dohp, "step");
  if (v->stepnumber < 0) v->stepnumber = 0, v->totalsteps = std::max(v->totalsteps, 1);
  step = child(steps, step_name(v->stepnumber));
  if (step) return 0;
  if (v->mode != 0) return set_error("DHM: step %d is not in the file", v->stepnumber);
  step = ensure_group(steps, step_name(v->stepnumber));
  TimeRec t{};
  t.value = v->time;
  copy_str(t.units.dimensions, v->timeunits);
  t.units.scale = v->timescale;
  step->attrs.push_back({"time", time_type(), {}, bytes_of(&t, 1)});
  return 0;
}

}  // namespace

extern "C" {

dErr dViewerDHMOpen(const char *path, dFileMode mode, dViewer *viewer) {
  if (!path || !viewer) return set_error("null argument");
  if (mode != dFILE_MODE_WRITE && mode != dFILE_MODE_READ) return set_error("DHM: mode must be dFILE_MODE_WRITE or dFILE_MODE_READ");
  auto *v = new _p_dViewer();
  v->path = path;
  v->mode = mode == dFILE_MODE_WRITE ? 0 : 1;
  if (v->mode == 0) {  // dViewerDHMSetUp (dhm.c:259-273): the dohp group and its four children
    v->root = std::make_shared<Node>();
    v->dohp = ensure_group(v->root, "dohp");
    for (const char *g : {"mesh", "fs", "step", "type"}) ensure_group(v->dohp, g);
    auto types = child(v->dohp, "type");
    for (auto &kv : std::vector<std::pair<std::string, Type>>{{"Units_type", units_type()}, {"Time_type", time_type()},
                                                              {"BoundingBox_type", bbox_type()}, {"FS_type", fs_type()},
                                                              {"Vec_type", vec_type()}}) {
      auto t = std::make_shared<Node>();
      t->kind = Node::NAMED_TYPE;
      t->type = kv.second;
      types->links.push_back({kv.first, t});
    }
  } else {
    dErr e = read_file(v->path, v->root);
    if (!e) {
      v->dohp = child(v->root, "dohp");
      if (!v->dohp || !child(v->dohp, "step") || !child(v->dohp, "fs") || !child(v->dohp, "mesh")) e = set_error("DHM: %s has no dohp layout", path);
    }
    if (e) {
      delete v;
      return e;
    }
    v->totalsteps = (int)child(v->dohp, "step")->links.size();
  }
  *viewer = v;
  return 0;
}

dErr dViewerDestroy(dViewer *viewer) {
  if (!viewer || !*viewer) return 0;
  dViewer v = *viewer;
  dErr e = v->mode == 0 ? write_file(v->path, v->root) : 0;
  delete v;
  *viewer = nullptr;
  return e;
}

dErr dViewerDHMSetTime(dViewer v, dReal time) {
  if (!v) return set_error("null viewer");
  if (v->mode != 0) return set_error("DHM: dViewerDHMSetTime on a viewer opened for reading (use dViewerDHMSetTimeStep)");
  if (!v->totalsteps || time != v->time) v->stepnumber++, v->totalsteps++;  // dViewerDHMSetTime_DHM (dhm.c:339-349)
  v->time = time;
  return 0;
}

dErr dViewerDHMSetTimeUnits(dViewer v, const char *units, dReal scale) {
  if (!v || !units) return set_error("null argument");
  v->timeunits = units;
  v->timescale = scale;
  return 0;
}

dErr dViewerDHMGetSteps(dViewer v, dInt *nsteps, dReal *times) {
  if (!v || !nsteps) return set_error("null argument");
  auto steps = child(v->dohp, "step");
  std::vector<std::pair<std::string, double>> st;
  for (auto &l : steps->links) {
    double t = 0;
    for (auto &a : l.second->attrs)
      if (a.name == "time" && a.data.size() >= sizeof(double)) memcpy(&t, a.data.data(), sizeof t);
    st.push_back({l.first, t});
  }
  std::sort(st.begin(), st.end());
  *nsteps = (dInt)st.size();
  if (times)
    for (size_t i = 0; i < st.size(); i++) times[i] = st[i].second;
  return 0;
}

dErr dViewerDHMSetTimeStep(dViewer v, dInt step) {
  if (!v) return set_error("null viewer");
  if (step < 0 || step >= v->totalsteps) return set_error("Step %d out of range [0 .. %d]", step, v->totalsteps);
  v->stepnumber = step;
  if (v->mode == 1) {
    std::shared_ptr<Node> s;
    DCHK(current_step(v, s));
    for (auto &a : s->attrs)
      if (a.name == "time" && a.data.size() >= sizeof(TimeRec)) {
        TimeRec t;
        memcpy(&t, a.data.data(), sizeof t);
        v->time = t.value, v->timescale = t.units.scale;
        v->timeunits.assign(t.units.dimensions, strnlen(t.units.dimensions, kStr));
      }
  }
  return 0;
}

dErr dViewerDHMGetTime(dViewer v, dReal *time) {
  if (!v || !time) return set_error("null argument");
  *time = v->time;
  return 0;
}

// dFSView_Cont_DHM (contviewdhm.c:58-116): the mesh (once per mesh) and the FS record under /dohp/fs/<name>
dErr dFSViewDHM(dFS fs, const char *name, dViewer v) {
  if (!fs || !name || !v) return set_error("null argument");
  if (v->mode != 0) return set_error("DHM: viewer opened for reading");
  if (!fs->built) return set_error("dFS space not built");
  if (!*name || strlen(name) >= kStr - 16 || strchr(name, '/')) return set_error("DHM: FS name must be 1..%d characters without '/'", kStr - 17);
  _p_dMesh *m = fs->mesh;
  auto mit = v->meshname.find(m);  // one mesh group per dMesh
  if (mit == v->meshname.end()) mit = v->meshname.insert({m, "mesh" + std::to_string(v->meshname.size())}).first;
  const std::string mname = mit->second, mpath = "/dohp/mesh/" + mname + "/000";
  auto meshroot = child(v->dohp, "mesh");
  auto mg = ensure_group(ensure_group(meshroot, mname), "000");
  if (mg->links.empty()) {  // the mesh itself (the reference writes a MOAB file and its name here)
    std::vector<int64_t> hex(m->hconn.begin(), m->hconn.end());
    mg->links.push_back({"vertices", dataset(t_f64(), {(uint64_t)m->nv, 3}, bytes_of(m->vx.data(), m->vx.size()))});
    mg->links.push_back({"hexes", dataset(t_int(8), {(uint64_t)m->nr, 8}, bytes_of(hex.data(), hex.size()))});
    if (m->structured) {  // a block: its extents give the entity order back
      const int32_t np[3] = {m->nx, m->ny, m->nz};
      mg->links.push_back({"npoints", dataset(t_int(4), {3}, bytes_of(np, 3))});
    } else {  // a mesh from connectivity: its edges and faces in their order
      std::vector<int64_t> ed(m->econn.begin(), m->econn.end()), fa(m->fconn.begin(), m->fconn.end());
      mg->links.push_back({"edges", dataset(t_int(8), {(uint64_t)m->ne, 2}, bytes_of(ed.data(), ed.size()))});
      mg->links.push_back({"faces", dataset(t_int(8), {(uint64_t)m->nf, 4}, bytes_of(fa.data(), fa.size()))});
    }
  }
  // per-FS tags (the reference's degree and boundary-status tags of the MOAB mesh)
  const std::string deg_name = std::string(name) + "_degree", bst_name = std::string(name) + "_bstatus";
  if (!child(mg, deg_name)) {
    const std::vector<int32_t> deg(fs->edeg.begin(), fs->edeg.end());
    mg->links.push_back({deg_name, dataset(t_int(4), {(uint64_t)fs->nelem, 3}, bytes_of(deg.data(), deg.size()))});
    const int32_t bst[2] = {fs->dirichlet_mask, fs->weak_mask};
    mg->links.push_back({bst_name, dataset(t_int(4), {2}, bytes_of(bst, 2))});
  }
  FSRec r{};
  copy_str(r.degree, deg_name);
  copy_str(r.global_offset, "");
  copy_str(r.partition, "");
  copy_str(r.ordered_subdomain, "");
  copy_str(r.bstatus, bst_name);
  copy_str(r.mesh, mpath);
  r.time = v->time;
  r.internal_state = v->state++;
  r.number_of_subdomains = 1;
  for (int d = 0; d < 3; d++) r.boundingbox[d][0] = 1e300, r.boundingbox[d][1] = -1e300;
  for (int64_t i = 0; i < m->nv; i++)
    for (int d = 0; d < 3; d++) {
      r.boundingbox[d][0] = std::min(r.boundingbox[d][0], m->vx[3 * i + d]);
      r.boundingbox[d][1] = std::max(r.boundingbox[d][1], m->vx[3 * i + d]);
    }
  r.block_size = fs->bs;
  auto fsroot = child(v->dohp, "fs");
  auto old = child(fsroot, name);
  auto rec = dataset(fs_type(), {1}, bytes_of(&r, 1));
  if (old) *old = *rec;
  else fsroot->links.push_back({name, rec});
  v->fsname[fs] = name;
  return 0;
}

// VecView_Dohp_FSCont_DHM (contviewdhm.c:133-209): the closure vector [nc][bs] (global values followed by the Dirichlet
// values) as dataset <vname> of the current step with its "meta" record; on_device: closure is a device pointer
dErr dVecViewDHM(dFS fs, const char *vname, const dScalar *closure, int on_device, dViewer v) {
  if (!fs || !vname || !closure || !v) return set_error("null argument");
  if (v->mode != 0) return set_error("DHM: viewer opened for reading");
  if (!*vname || strlen(vname) >= kStr || strchr(vname, '/')) return set_error("DHM: vector name must be 1..%d characters without '/'", kStr - 1);
  auto it = v->fsname.find(fs);
  if (it == v->fsname.end()) return set_error("DHM: write the vector's dFS with dFSViewDHM first");
  std::shared_ptr<Node> step;
  DCHK(current_step(v, step));
  const int64_t n = fs->nc * fs->bs;
  std::vector<double> h(std::max<int64_t>(n, 1));
  if (on_device) CUCHK(cudaMemcpy(h.data(), closure, n * sizeof(double), cudaMemcpyDeviceToHost));
  else std::copy(closure, closure + n, h.begin());
  auto d = dataset(t_f64(), {(uint64_t)fs->nc, (uint64_t)fs->bs}, bytes_of(h.data(), n));
  VecRec r{};
  copy_str(r.fs, "/dohp/fs/" + it->second);
  r.time = v->time;
  copy_str(r.units.dimensions, "");
  r.units.scale = 1.0;
  r.internal_state = v->state++;
  d->attrs.push_back({"meta", vec_type(), {1}, bytes_of(&r, 1)});
  for (auto &l : step->links)
    if (l.first == vname) return set_error("DHM: vector %s already written in this step", vname);
  step->links.push_back({vname, d});
  return 0;
}

// VecDohpLoadIntoVector (contviewdhm.c:350-401): the closure vector <vname> of the current step, scaled by the record's
// units scale, into closure (nc * bs values; device pointer when on_device)
dErr dVecLoadDHM(dViewer v, const char *vname, dFS fs, dScalar *closure, int on_device) {
  if (!fs || !vname || !closure || !v) return set_error("null argument");
  std::shared_ptr<Node> step;
  DCHK(current_step(v, step));
  auto d = child(step, vname);
  if (!d || d->kind != Node::DATASET) return set_error("DHM: no vector %s in step %d", vname, v->stepnumber);
  if (d->dims.size() != 2 || d->dims[0] != (uint64_t)fs->nc || d->dims[1] != (uint64_t)fs->bs || d->type.size != 8)
    return set_error("DHM: vector %s does not match the space (closure %lld x %d)", vname, (long long)fs->nc, fs->bs);
  double scale = 1.0;
  for (auto &a : d->attrs)
    if (a.name == "meta" && a.data.size() >= sizeof(VecRec)) {
      VecRec r;
      memcpy(&r, a.data.data(), sizeof r);
      scale = r.units.scale;
    }
  const int64_t n = fs->nc * fs->bs;
  std::vector<double> h(std::max<int64_t>(n, 1));
  memcpy(h.data(), d->data.data(), n * sizeof(double));
  if (scale != 1.0)
    for (double &x : h) x *= scale;
  if (on_device) CUCHK(cudaMemcpy(closure, h.data(), n * sizeof(double), cudaMemcpyHostToDevice));
  else std::copy(h.begin(), h.begin() + n, closure);
  return 0;
}

// dFSLoadIntoFS_Cont_DHM (contviewdhm.c:228-348): the mesh and the space recorded as /dohp/fs/<name>; the result is
// built (dFSBuildSpace), the caller sets a stream and calls dFSSetUp
dErr dFSLoadDHM(dViewer v, const char *name, dJacobi jac, dMesh *mesh, dFS *fs) {
  if (!v || !name || !mesh || !fs) return set_error("null argument");
  auto rec = child(child(v->dohp, "fs"), name);
  if (!rec || rec->data.size() < sizeof(FSRec)) return set_error("DHM: could not find FS by name \"%s\"", name);
  FSRec r;
  memcpy(&r, rec->data.data(), sizeof r);
  auto mg = lookup(v->root, std::string(r.mesh, strnlen(r.mesh, kStr)));
  auto vx = child(mg, "vertices"), np = child(mg, "npoints"), hx = child(mg, "hexes");
  auto eds = child(mg, "edges"), fas = child(mg, "faces");
  auto deg = child(mg, std::string(r.degree, strnlen(r.degree, kStr))), bst = child(mg, std::string(r.bstatus, strnlen(r.bstatus, kStr)));
  if (!vx || !hx || !(np || (eds && fas)) || !deg || !bst) return set_error("DHM: incomplete mesh record for FS \"%s\"", name);
  int32_t masks[2];
  memcpy(masks, bst->data.data(), sizeof masks);
  if (np) {
    int32_t npts[3];
    memcpy(npts, np->data.data(), sizeof npts);
    const dReal box[6] = {0, 1, 0, 1, 0, 1};
    DCHK(dMeshCreateBlock(npts, box, 0.0, 0, mesh));
    _p_dMesh *m = *mesh;
    if (vx->data.size() != m->vx.size() * sizeof(double)) {
      dMeshDestroy(mesh);
      return set_error("DHM: vertex count of the file does not match its block extents");
    }
    memcpy(m->vx.data(), vx->data.data(), vx->data.size());
  } else {  // a mesh from connectivity: entities in the order written
    auto ints = [](const std::shared_ptr<Node> &d, std::vector<dInt> &out) {
      const int64_t *p = (const int64_t *)d->data.data();
      out.resize(d->data.size() / sizeof(int64_t));
      for (size_t i = 0; i < out.size(); i++) out[i] = (dInt)p[i];
    };
    std::vector<dInt> e2, f4, h8;
    ints(eds, e2), ints(fas, f4), ints(hx, h8);
    DCHK(dMeshCreateFromConnectivity((dInt)(vx->data.size() / (3 * sizeof(double))), (const double *)vx->data.data(),
                                     (dInt)(e2.size() / 2), e2.data(), (dInt)(f4.size() / 4), f4.data(), (dInt)(h8.size() / 8),
                                     h8.data(), mesh));
  }
  _p_dMesh *m = *mesh;
  dErr e = dFSCreate(m, jac, fs);
  const int32_t *dg = (const int32_t *)deg->data.data();
  const int64_t ne = (int64_t)deg->dims[0];
  std::vector<dInt> ed(ne);
  bool uniform = true;
  for (int64_t i = 0; i < ne; i++) ed[i] = dg[3 * i], uniform = uniform && dg[3 * i] == dg[0] && dg[3 * i + 1] == dg[0] && dg[3 * i + 2] == dg[0];
  if (!e) e = dFSSetDegree(*fs, ne ? dg[0] : 1, uniform ? nullptr : ed.data());
  if (!e) e = dFSSetBlockSize(*fs, r.block_size);
  const int sets[3] = {100, 200, 300};
  for (int i = 0; i < 3 && !e; i++) {
    const int st = ((masks[0] >> i) & 1 ? dFSBSTATUS_DIRICHLET : 0) | ((masks[1] >> i) & 1 ? dFSBSTATUS_WEAK : 0);
    if (st) e = dFSRegisterBoundary(*fs, sets[i], (dFSBStatus)st);
  }
  if (!e) e = dFSBuildSpace(*fs);
  if (e) {
    dFSDestroy(fs);
    dMeshDestroy(mesh);
  }
  return e;
}

// the checksum of HDF5 metadata (exported for the format tests)
uint32_t dHDF5Checksum(const void *data, size_t len, uint32_t initval) { return lookup3((const uint8_t *)data, len, initval); }

}  // extern "C"
