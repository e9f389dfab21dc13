// h5io.cu -- the reference's diagnostic and restart files, written and read without an HDF5
// library (none exists on these machines).
//
// The reference writes its field dumps and beam restart files through libhdf5 with default
// (earliest-format) settings (hdf5io_class.f03:264-335 attributes, 338-795 fields,
// 1584-1819 particles).  This file produces that subset of the HDF5 file format directly, as
// the published HDF5 File Format Specification describes it:
//   superblock version 0 (8-byte offsets and lengths), version 1 object headers, groups as
//   symbol tables (a local heap of names, one version 1 B-tree node, symbol table nodes),
//   datasets with a version 1 dataspace, an IEEE little-endian double or 32-bit integer
//   datatype, a version 2 fill-value message and version 3 contiguous layout, and version 1
//   attributes (doubles, 32-bit integers, fixed-length strings).
// The reader understands the same subset, plus what libhdf5 adds to such files (superblock
// version 1, continuation and NIL messages, version 2/3 attributes and dataspaces, compact
// layout, multi-level group B-trees), so that restart files written by the reference can be
// read back.  All integers in the format are little-endian; the host code below assembles
// them byte by byte and so does not depend on the host's byte order.
#include <sys/stat.h>
#include <sys/types.h>

#include <algorithm>
#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "qpad_internal.cuh"

namespace h5 {

static constexpr uint64_t kUndef = ~0ull;
static constexpr int kLeafK = 4, kInternalK = 16;   // symbol table / B-tree node ranks

// ---- what a file holds ------------------------------------------------------------------
struct Attr {
  std::string name;
  int kind = 0;                      // 0 double, 1 int32, 2 string
  std::vector<double> f;
  std::vector<int32_t> i;
  std::string s;
};

struct Obj {
  std::string name;
  bool group = false;
  std::vector<Obj> kids;             // group members
  std::vector<Attr> attrs;
  std::vector<uint64_t> dims;        // dataset
  int dtype = 0;                     // 0 double, 1 int32
  const void* data = nullptr;
  uint64_t nbytes = 0;
};

// ---- byte assembly ------------------------------------------------------------------------
struct Buf {
  std::vector<uint8_t> b;
  size_t size() const { return b.size(); }
  void u8(unsigned v) { b.push_back((uint8_t)v); }
  void u16(unsigned v) { u8(v & 0xff); u8((v >> 8) & 0xff); }
  void u32(uint32_t v) { for (int k = 0; k < 4; ++k) u8((v >> (8 * k)) & 0xff); }
  void u64(uint64_t v) { for (int k = 0; k < 8; ++k) u8((unsigned)((v >> (8 * k)) & 0xff)); }
  void bytes(const void* p, size_t n) { const uint8_t* q = (const uint8_t*)p; b.insert(b.end(), q, q + n); }
  void zeros(size_t n) { b.insert(b.end(), n, 0); }
  void pad8() { while (b.size() % 8) u8(0); }
  void put64(size_t at, uint64_t v) { for (int k = 0; k < 8; ++k) b[at + k] = (uint8_t)((v >> (8 * k)) & 0xff); }
  void put32(size_t at, uint32_t v) { for (int k = 0; k < 4; ++k) b[at + k] = (uint8_t)((v >> (8 * k)) & 0xff); }
};

static size_t up8(size_t n) { return (n + 7) & ~(size_t)7; }

// datatype message bodies
static void dt_f64(Buf& o) {
  o.u8(0x10 | 1);                    // version 1, class floating point
  o.u8(0x20);                        // little endian, no padding bits, implied mantissa msb
  o.u8(63);                          // sign bit position
  o.u8(0);
  o.u32(8);
  o.u16(0); o.u16(64);               // bit offset, precision
  o.u8(52); o.u8(11); o.u8(0); o.u8(52);   // exponent location / size, mantissa location / size
  o.u32(1023);                       // exponent bias
}
static void dt_i32(Buf& o) {
  o.u8(0x10 | 0);                    // version 1, class fixed point
  o.u8(0x08);                        // little endian, signed
  o.u8(0); o.u8(0);
  o.u32(4);
  o.u16(0); o.u16(32);
}
static void dt_str(Buf& o, uint32_t len) {
  o.u8(0x10 | 3);                    // version 1, class string
  o.u8(0x02);                        // space padded (the reference's Fortran strings), ASCII
  o.u8(0); o.u8(0);
  o.u32(len ? len : 1);
}
static void space_v1(Buf& o, const std::vector<uint64_t>& dims) {
  o.u8(1); o.u8((unsigned)dims.size()); o.u8(0); o.u8(0); o.u32(0);
  for (uint64_t d : dims) o.u64(d);
}

// one v1 object header message
static void msg(Buf& o, unsigned type, const Buf& body) {
  o.u16(type);
  o.u16((unsigned)up8(body.size()));
  o.u8(0); o.u8(0); o.u8(0); o.u8(0);
  o.bytes(body.b.data(), body.size());
  o.pad8();
}

static Buf attr_msg(const Attr& a) {
  Buf dt, sp, data;
  if (a.kind == 0) {
    dt_f64(dt);
    space_v1(sp, {(uint64_t)a.f.size()});
    for (double v : a.f) { uint64_t u; memcpy(&u, &v, 8); data.u64(u); }
  } else if (a.kind == 1) {
    dt_i32(dt);
    space_v1(sp, {(uint64_t)a.i.size()});
    for (int32_t v : a.i) data.u32((uint32_t)v);
  } else {
    dt_str(dt, (uint32_t)a.s.size());
    space_v1(sp, {1});
    data.bytes(a.s.data(), a.s.size());
    if (a.s.empty()) data.u8(' ');
  }
  Buf m;
  m.u8(1); m.u8(0);
  m.u16((unsigned)a.name.size() + 1);
  m.u16((unsigned)dt.size());
  m.u16((unsigned)sp.size());
  m.bytes(a.name.c_str(), a.name.size() + 1); m.pad8();
  m.bytes(dt.b.data(), dt.size()); m.pad8();
  m.bytes(sp.b.data(), sp.size()); m.pad8();
  m.bytes(data.b.data(), data.size());
  return m;
}

// writes the object header of `o` (and for a group its heap, B-tree and symbol nodes, and
// all members) at the end of `f`; returns the object header's address
static uint64_t emit(Buf& f, const Obj& o);

static uint64_t emit_header(Buf& f, const std::vector<std::pair<unsigned, Buf>>& msgs) {
  f.pad8();
  const uint64_t at = f.size();
  Buf body;
  for (auto& m : msgs) msg(body, m.first, m.second);
  f.u8(1); f.u8(0);
  f.u16((unsigned)msgs.size());
  f.u32(1);
  f.u32((uint32_t)body.size());
  f.u32(0);                          // pads the 12-byte prefix to 16
  f.bytes(body.b.data(), body.size());
  return at;
}

static uint64_t emit(Buf& f, const Obj& o) {
  std::vector<std::pair<unsigned, Buf>> msgs;
  if (!o.group) {
    Buf sp, dt, fill, lay;
    space_v1(sp, o.dims);
    if (o.dtype == 0) dt_f64(dt); else dt_i32(dt);
    fill.u8(2); fill.u8(2); fill.u8(2); fill.u8(0);     // fill value: v2, late, if set, undefined
    lay.u8(3); lay.u8(1);                               // layout v3, contiguous
    const size_t addr_pos = 2;
    lay.u64(0); lay.u64(o.nbytes);
    msgs.push_back({0x0001, sp});
    msgs.push_back({0x0003, dt});
    msgs.push_back({0x0005, fill});
    msgs.push_back({0x0008, lay});
    for (auto& a : o.attrs) msgs.push_back({0x000C, attr_msg(a)});
    const uint64_t hdr = emit_header(f, msgs);
    // the raw data right after the header; patch the layout's address
    f.pad8();
    const uint64_t data_at = f.size();
    if (o.nbytes) f.bytes(o.data, o.nbytes);
    // layout message position: prefix 16 + dataspace, datatype and fill messages
    size_t pos = hdr + 16;
    for (int k = 0; k < 3; ++k) pos += 8 + up8(msgs[k].second.size());
    f.put64(pos + 8 + addr_pos, o.nbytes ? data_at : kUndef);
    return hdr;
  }
  // group: members sorted by name (the B-tree order); names into the local heap
  std::vector<const Obj*> kids;
  for (auto& k : o.kids) kids.push_back(&k);
  std::sort(kids.begin(), kids.end(), [](const Obj* a, const Obj* b) { return a->name < b->name; });
  Buf heap;
  heap.zeros(8);                     // offset 0: the empty name
  std::vector<uint64_t> name_off;
  for (auto* k : kids) {
    name_off.push_back(heap.size());
    heap.bytes(k->name.c_str(), k->name.size() + 1);
    heap.pad8();
  }
  // (an empty group has a B-tree node with no entries and no symbol table node, as libhdf5 makes it)
  const size_t nsnod = (kids.size() + 2 * kLeafK - 1) / (2 * kLeafK);
  // members first, so their header addresses are known
  std::vector<uint64_t> kid_hdr, kid_bt(kids.size(), 0), kid_hp(kids.size(), 0);
  // (a member group's B-tree and heap addresses go into its symbol table entry)
  for (size_t k = 0; k < kids.size(); ++k) {
    kid_hdr.push_back(emit(f, *kids[k]));
    if (kids[k]->group) {
      // read the member's symbol table message back from its header: B-tree, heap
      const size_t p = kid_hdr[k] + 16 + 8;
      uint64_t bt = 0, hp = 0;
      for (int q = 0; q < 8; ++q) bt |= (uint64_t)f.b[p + q] << (8 * q);
      for (int q = 0; q < 8; ++q) hp |= (uint64_t)f.b[p + 8 + q] << (8 * q);
      kid_bt[k] = bt;
      kid_hp[k] = hp;
    }
  }
  // local heap
  f.pad8();
  const uint64_t heap_at = f.size();
  f.bytes("HEAP", 4); f.u8(0); f.zeros(3);
  f.u64(heap.size());
  f.u64(1);                          // no free block (the library's end-of-free-list mark)
  f.u64(heap_at + 32);
  f.bytes(heap.b.data(), heap.size());
  // symbol table nodes
  std::vector<uint64_t> snod_at;
  for (size_t s = 0; s < nsnod; ++s) {
    f.pad8();
    snod_at.push_back(f.size());
    const size_t lo = s * 2 * kLeafK, hi = std::min(kids.size(), lo + 2 * kLeafK);
    f.bytes("SNOD", 4); f.u8(1); f.u8(0); f.u16((unsigned)(hi - lo));
    for (size_t k = lo; k < lo + 2 * kLeafK; ++k) {
      if (k < hi) {
        f.u64(name_off[k]); f.u64(kid_hdr[k]);
        f.u32(kids[k]->group ? 1 : 0); f.u32(0);
        f.u64(kid_bt[k]); f.u64(kid_hp[k]);
      } else {
        f.zeros(40);
      }
    }
  }
  // one B-tree node (leaf level) over the symbol table nodes
  f.pad8();
  const uint64_t bt_at = f.size();
  f.bytes("TREE", 4); f.u8(0); f.u8(0); f.u16((unsigned)nsnod);
  f.u64(kUndef); f.u64(kUndef);
  f.u64(0);                          // key 0: the empty name
  for (size_t s = 0; s < 2 * kInternalK; ++s) {
    if (s < nsnod) {
      const size_t last = std::min(kids.size(), (s + 1) * 2 * kLeafK);
      f.u64(snod_at[s]);
      f.u64(last ? name_off[last - 1] : 0);
    } else {
      f.u64(0); f.u64(0);
    }
  }
  // the group's object header: its symbol table message, then attributes
  Buf stab;
  stab.u64(bt_at); stab.u64(heap_at);
  msgs.push_back({0x0011, stab});
  for (auto& a : o.attrs) msgs.push_back({0x000C, attr_msg(a)});
  return emit_header(f, msgs);
}

static int mkdirs(const std::string& dir) {
  std::string cur;
  for (size_t i = 0; i < dir.size(); ++i) {
    cur += dir[i];
    if ((dir[i] == '/' && i > 0) || i + 1 == dir.size())
      if (mkdir(cur.c_str(), 0755) != 0 && errno != EEXIST) return -1;
  }
  return 0;
}

// Writes a file whose root group is `root` (its kids and attributes).
static int write_file(const std::string& path, const Obj& root, std::string& err) {
  Buf f;
  f.zeros(96);                       // superblock, filled in below
  const uint64_t root_hdr = emit(f, root);
  uint64_t bt = 0, hp = 0;
  for (int q = 0; q < 8; ++q) bt |= (uint64_t)f.b[root_hdr + 24 + q] << (8 * q);
  for (int q = 0; q < 8; ++q) hp |= (uint64_t)f.b[root_hdr + 32 + q] << (8 * q);
  Buf sb;
  const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
  sb.bytes(sig, 8);
  sb.u8(0); sb.u8(0); sb.u8(0); sb.u8(0); sb.u8(0);
  sb.u8(8); sb.u8(8); sb.u8(0);
  sb.u16(kLeafK); sb.u16(kInternalK);
  sb.u32(0);
  sb.u64(0); sb.u64(kUndef); sb.u64(f.size()); sb.u64(kUndef);
  sb.u64(0); sb.u64(root_hdr); sb.u32(1); sb.u32(0); sb.u64(bt); sb.u64(hp);
  memcpy(f.b.data(), sb.b.data(), 96);
  const size_t slash = path.rfind('/');
  if (slash != std::string::npos && slash > 0 && mkdirs(path.substr(0, slash + 1))) {
    err = "cannot create the directory of " + path;
    return QPAD_E_ARG;
  }
  FILE* fp = fopen(path.c_str(), "wb");
  if (!fp) { err = "cannot open " + path + " for writing"; return QPAD_E_ARG; }
  const size_t n = fwrite(f.b.data(), 1, f.size(), fp);
  const int c = fclose(fp);
  if (n != f.size() || c != 0) { err = "short write to " + path; return QPAD_E_ARG; }
  return 0;
}

// ---- reader -------------------------------------------------------------------------------
struct Reader {
  std::vector<uint8_t> b;
  std::string err;
  bool ok(uint64_t at, uint64_t n) const { return at <= b.size() && n <= b.size() - at; }
  uint64_t le(uint64_t at, int n) const {
    uint64_t v = 0;
    for (int k = 0; k < n; ++k) v |= (uint64_t)b[at + k] << (8 * k);
    return v;
  }
};

struct ObjInfo {
  std::map<std::string, uint64_t> kids;     // group members: name -> object header
  bool is_group = false;
  uint64_t btree = 0, heap = 0;
  std::vector<uint64_t> dims;
  int dclass = -1, dsize = 0, dsigned = 0;  // datatype
  int layout = -1;                          // 0 compact, 1 contiguous
  uint64_t data_at = 0, data_n = 0;
  std::map<std::string, std::vector<uint8_t>> attr_raw;   // name -> raw bytes
  std::map<std::string, std::pair<int, int>> attr_type;   // name -> (class, size)
  std::map<std::string, uint64_t> attr_count;
};

static bool parse_dt(const Reader& R, uint64_t at, uint64_t n, int& cls, int& size, int& sgn) {
  if (!R.ok(at, 8) || n < 8) return false;
  cls = R.b[at] & 0x0f;
  sgn = (R.b[at + 1] >> 3) & 1;
  size = (int)R.le(at + 4, 4);
  return true;
}

static bool parse_space(const Reader& R, uint64_t at, uint64_t n, std::vector<uint64_t>& dims) {
  if (!R.ok(at, 8) || n < 2) return false;
  const int ver = R.b[at], rank = R.b[at + 1], flags = R.b[at + 2];
  uint64_t p = ver == 1 ? at + 8 : at + 4;
  dims.clear();
  if (!R.ok(p, 8ull * rank)) return false;
  for (int k = 0; k < rank; ++k) dims.push_back(R.le(p + 8ull * k, 8));
  (void)flags;
  if (rank == 0) dims.push_back(1);  // a scalar holds one element
  return true;
}

static bool parse_header(Reader& R, uint64_t at, ObjInfo& o) {
  if (!R.ok(at, 16) || R.b[at] != 1) { R.err = "unsupported object header (only version 1)"; return false; }
  const unsigned nmsg = (unsigned)R.le(at + 2, 2);
  std::vector<std::pair<uint64_t, uint64_t>> blocks = {{at + 16, R.le(at + 8, 4)}};
  unsigned seen = 0;
  for (size_t bi = 0; bi < blocks.size() && seen < nmsg; ++bi) {
    uint64_t p = blocks[bi].first;
    const uint64_t end = p + blocks[bi].second;
    while (p + 8 <= end && seen < nmsg) {
      if (!R.ok(p, 8)) { R.err = "truncated object header"; return false; }
      const unsigned type = (unsigned)R.le(p, 2), size = (unsigned)R.le(p + 2, 2);
      const uint64_t d = p + 8;
      if (!R.ok(d, size)) { R.err = "truncated header message"; return false; }
      ++seen;
      switch (type) {
        case 0x0001: parse_space(R, d, size, o.dims); break;
        case 0x0003: parse_dt(R, d, size, o.dclass, o.dsize, o.dsigned); break;
        case 0x0008: {
          const int ver = R.b[d];
          if (ver != 3) { R.err = "unsupported data layout message version"; return false; }
          o.layout = R.b[d + 1];
          if (o.layout == 1) { o.data_at = R.le(d + 2, 8); o.data_n = R.le(d + 10, 8); }
          else if (o.layout == 0) { o.data_n = R.le(d + 2, 2); o.data_at = d + 4; }
          else { R.err = "chunked datasets are not read"; return false; }
          break;
        }
        case 0x0010: blocks.push_back({R.le(d, 8), R.le(d + 8, 8)}); break;   // continuation
        case 0x0011: o.is_group = true; o.btree = R.le(d, 8); o.heap = R.le(d + 8, 8); break;
        case 0x000C: {
          const int ver = R.b[d];
          const unsigned nl = (unsigned)R.le(d + 2, 2), dl = (unsigned)R.le(d + 4, 2), sl = (unsigned)R.le(d + 6, 2);
          uint64_t q = d + (ver == 3 ? 9 : 8);
          auto adv = [&](uint64_t n) { return ver == 1 ? up8(n) : n; };
          std::string name((const char*)&R.b[q], nl ? nl - 1 : 0);
          name = std::string(name.c_str());
          q += adv(nl);
          int cls, sz, sg;
          parse_dt(R, q, dl, cls, sz, sg);
          q += adv(dl);
          std::vector<uint64_t> ad;
          parse_space(R, q, sl, ad);
          q += adv(sl);
          uint64_t cnt = 1;
          for (uint64_t x : ad) cnt *= x;
          const uint64_t nb = cnt * (uint64_t)sz;
          if (!R.ok(q, nb)) { R.err = "truncated attribute"; return false; }
          o.attr_raw[name].assign(R.b.begin() + q, R.b.begin() + q + nb);
          o.attr_type[name] = {cls, sz};
          o.attr_count[name] = cnt;
          break;
        }
        default: break;                // NIL, fill value, times, ... not needed
      }
      p = d + size;
    }
  }
  return true;
}

static bool heap_name(const Reader& R, uint64_t heap, uint64_t off, std::string& name) {
  if (!R.ok(heap, 32) || memcmp(&R.b[heap], "HEAP", 4)) return false;
  const uint64_t seg = R.le(heap + 24, 8), segn = R.le(heap + 8, 8);
  if (off >= segn || !R.ok(seg, segn)) return false;
  name.clear();
  for (uint64_t p = seg + off; p < seg + segn && R.b[p]; ++p) name += (char)R.b[p];
  return true;
}

static bool walk_btree(Reader& R, uint64_t node, uint64_t heap, std::map<std::string, uint64_t>& out, int depth = 0) {
  if (depth > 16 || !R.ok(node, 24) || memcmp(&R.b[node], "TREE", 4)) { R.err = "bad group B-tree"; return false; }
  const int level = R.b[node + 5];
  const unsigned used = (unsigned)R.le(node + 6, 2);
  for (unsigned c = 0; c < used; ++c) {
    const uint64_t child = R.le(node + 24 + 8 + 16ull * c, 8);
    if (level > 0) {
      if (!walk_btree(R, child, heap, out, depth + 1)) return false;
      continue;
    }
    if (!R.ok(child, 8) || memcmp(&R.b[child], "SNOD", 4)) { R.err = "bad symbol table node"; return false; }
    const unsigned ns = (unsigned)R.le(child + 6, 2);
    for (unsigned e = 0; e < ns; ++e) {
      const uint64_t ent = child + 8 + 40ull * e;
      if (!R.ok(ent, 40)) { R.err = "truncated symbol table node"; return false; }
      std::string name;
      if (!heap_name(R, heap, R.le(ent, 8), name)) { R.err = "bad local heap"; return false; }
      out[name] = R.le(ent + 8, 8);
    }
  }
  return true;
}

static bool open_file(Reader& R, const std::string& path, uint64_t& root) {
  FILE* fp = fopen(path.c_str(), "rb");
  if (!fp) { R.err = "cannot open " + path; return false; }
  fseek(fp, 0, SEEK_END);
  const long n = ftell(fp);
  fseek(fp, 0, SEEK_SET);
  R.b.resize(n > 0 ? (size_t)n : 0);
  const size_t got = n > 0 ? fread(R.b.data(), 1, (size_t)n, fp) : 0;
  fclose(fp);
  const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
  if (got != R.b.size() || R.b.size() < 96 || memcmp(R.b.data(), sig, 8)) { R.err = path + ": not an HDF5 file"; return false; }
  const int ver = R.b[8];
  if (ver > 1 || R.b[13] != 8 || R.b[14] != 8) { R.err = path + ": unsupported superblock"; return false; }
  const uint64_t entry = ver == 0 ? 56 : 60;   // version 1 adds the indexed-storage K and padding
  root = R.le(entry + 8, 8);
  return true;
}

// Resolves "a/b/c" from the root; returns the object's header info.
static bool lookup(Reader& R, uint64_t root, const std::string& path, ObjInfo& o) {
  uint64_t at = root;
  size_t pos = 0;
  while (true) {
    o = ObjInfo();
    if (!parse_header(R, at, o)) return false;
    if (pos >= path.size()) return true;
    const size_t slash = path.find('/', pos);
    const std::string part = path.substr(pos, slash == std::string::npos ? std::string::npos : slash - pos);
    pos = slash == std::string::npos ? path.size() : slash + 1;
    if (part.empty()) continue;
    if (!o.is_group) { R.err = "not a group on the way to " + path; return false; }
    std::map<std::string, uint64_t> kids;
    if (!walk_btree(R, o.btree, o.heap, kids)) return false;
    auto it = kids.find(part);
    if (it == kids.end()) { R.err = "no member " + part + " in " + path; return false; }
    at = it->second;
  }
}

}  // namespace h5

// =========================================================================================
// C ABI
// =========================================================================================
namespace {
thread_local std::string g_h5err;

std::string field_dir_part(int part) {
  if (part == 0) return "Re0";
  return (part % 2 ? "Re" : "Im") + std::to_string((part + 1) / 2);
}

std::string fortran_str(const char* s, size_t len) {   // character(len=100) as the reference writes it
  std::string v = s ? s : "";
  if (v.size() < len) v.append(len - v.size(), ' ');
  return v;
}

void file_attrs(h5::Obj& root, const char* name, const char* ty, double time, int iter, double dt,
                const char* timeunit) {
  h5::Attr a;
  a.name = "NAME"; a.kind = 2; a.s = fortran_str(name, 100); root.attrs.push_back(a);
  a = h5::Attr(); a.name = "TYPE"; a.kind = 2; a.s = fortran_str(ty, 100); root.attrs.push_back(a);
  a = h5::Attr(); a.name = "TIME"; a.kind = 0; a.f = {time}; root.attrs.push_back(a);
  a = h5::Attr(); a.name = "ITER"; a.kind = 1; a.i = {iter}; root.attrs.push_back(a);
  a = h5::Attr(); a.name = "DT"; a.kind = 0; a.f = {dt}; root.attrs.push_back(a);
  a = h5::Attr(); a.name = "TIME UNIT"; a.kind = 2; a.s = fortran_str(timeunit, 100); root.attrs.push_back(a);
}

void dset_attrs(h5::Obj& d, const char* units, const char* label) {
  h5::Attr a;
  a.name = "UNITS"; a.kind = 2; a.s = fortran_str(units, 100); d.attrs.push_back(a);
  a = h5::Attr(); a.name = "LONG_NAME"; a.kind = 2; a.s = fortran_str(label, 100); d.attrs.push_back(a);
}

std::string step_file(const char* dir, const char* dataname, int iter) {
  char num[16];
  snprintf(num, sizeof(num), "%08d", iter);
  std::string d = dir ? dir : ".";
  if (!d.empty() && d.back() != '/') d += '/';
  return d + dataname + "_" + num + ".h5";
}
}  // namespace

extern "C" const char* qpad_h5_last_error(void) { return g_h5err.c_str(); }

extern "C" int qpad_h5_write_grid(const char* path, const char* dataname, const double* data, int nz, int nr,
                                  const qpad_h5_grid_info* info) {
  if (!path || !dataname || !info || nz < 0 || nr < 0 || (!data && (int64_t)nz * nr > 0)) {
    g_h5err = "h5 grid: bad arguments";
    return QPAD_E_ARG;
  }
  h5::Obj root;
  root.group = true;
  const bool grid = !info->type || std::string(info->type) == "grid";
  file_attrs(root, dataname, grid ? "grid" : info->type, info->time, info->iter, info->dt, info->timeunit);
  std::vector<std::vector<double>> ax(2);          // (outlives the objects that point into it)
  if (grid) {
  h5::Obj axis;
  axis.name = "AXIS";
  axis.group = true;
  for (int k = 0; k < 2; ++k) {
    ax[k] = {info->axis_min[k], info->axis_max[k]};
    h5::Obj a;
    a.name = std::string("AXIS") + (char)('1' + k);
    a.dims = {2};
    a.data = ax[k].data();
    a.nbytes = 16;
    h5::Attr t;
    t.name = "TYPE"; t.kind = 2; t.s = "linear"; a.attrs.push_back(t);
    t = h5::Attr(); t.name = "UNITS"; t.kind = 2; t.s = info->axis_units[k] ? info->axis_units[k] : ""; a.attrs.push_back(t);
    t = h5::Attr(); t.name = "NAME"; t.kind = 2; t.s = info->axis_name[k] ? info->axis_name[k] : ""; a.attrs.push_back(t);
    t = h5::Attr(); t.name = "LONG_NAME"; t.kind = 2; t.s = info->axis_label[k] ? info->axis_label[k] : ""; a.attrs.push_back(t);
    axis.kids.push_back(a);
  }
  root.kids.push_back(axis);
  }
  h5::Obj d;
  d.name = dataname;
  d.dims = {(uint64_t)nz, (uint64_t)nr};
  d.data = data;
  d.nbytes = (uint64_t)nz * nr * 8;
  dset_attrs(d, info->units, info->label);
  root.kids.push_back(d);
  return h5::write_file(path, root, g_h5err);
}

extern "C" int qpad_h5_write_particles(const char* path, const char* dataname, const double* x, const double* p,
                                       const double* q, int64_t n, int iter, double time, double dt) {
  if (!path || !dataname || n < 0 || n > INT32_MAX || (n > 0 && (!x || !p || !q))) {
    g_h5err = "h5 particles: bad arguments";
    return QPAD_E_ARG;
  }
  h5::Obj root;
  root.group = true;
  file_attrs(root, dataname, "restart", time, iter, dt, "a.u.");
  h5::Attr tp;
  tp.name = "tp"; tp.kind = 1; tp.i = {(int32_t)n};
  root.attrs.push_back(tp);
  if (n > 0) {                       // the reference writes no datasets for an empty beam
    const char* names[3] = {"x", "p", "q"};
    const double* arr[3] = {x, p, q};
    for (int k = 0; k < 3; ++k) {
      h5::Obj d;
      d.name = names[k];
      d.dims = k < 2 ? std::vector<uint64_t>{(uint64_t)n, 3} : std::vector<uint64_t>{(uint64_t)n};
      d.data = arr[k];
      d.nbytes = (uint64_t)n * (k < 2 ? 3 : 1) * 8;
      dset_attrs(d, "a.u.", "Data");
      root.kids.push_back(d);
    }
  }
  return h5::write_file(path, root, g_h5err);
}

extern "C" int qpad_h5_read_dataset(const char* path, const char* name, double* out, int64_t cap, int64_t* count,
                                    int32_t* rank, int64_t* dims) {
  h5::Reader R;
  uint64_t root;
  if (!path || !name || !h5::open_file(R, path, root)) { g_h5err = R.err.empty() ? "h5 read: bad arguments" : R.err; return QPAD_E_ARG; }
  h5::ObjInfo o;
  if (!h5::lookup(R, root, name, o)) { g_h5err = R.err; return QPAD_E_ARG; }
  if (o.is_group || o.layout < 0) { g_h5err = std::string(name) + " is not a dataset"; return QPAD_E_ARG; }
  uint64_t n = 1;
  for (uint64_t d : o.dims) n *= d;
  if (rank) *rank = (int32_t)o.dims.size();
  if (dims) for (size_t k = 0; k < o.dims.size() && k < 8; ++k) dims[k] = (int64_t)o.dims[k];
  if (count) *count = (int64_t)n;
  if (!out) return 0;
  if ((int64_t)n > cap) { g_h5err = "h5 read: buffer too small"; return QPAD_E_CAPACITY; }
  const int esz = o.dsize;
  if (!((o.dclass == 1 && (esz == 8 || esz == 4)) || (o.dclass == 0 && (esz == 4 || esz == 8)))) {
    g_h5err = "h5 read: only float and integer datasets";
    return QPAD_E_ARG;
  }
  if (n && (o.data_at == h5::kUndef || !R.ok(o.data_at, n * (uint64_t)esz))) { g_h5err = "h5 read: data outside the file"; return QPAD_E_ARG; }
  for (uint64_t k = 0; k < n; ++k) {
    const uint64_t at = o.data_at + k * (uint64_t)esz;
    if (o.dclass == 1 && esz == 8) { uint64_t u = R.le(at, 8); memcpy(&out[k], &u, 8); }
    else if (o.dclass == 1) { uint32_t u = (uint32_t)R.le(at, 4); float f; memcpy(&f, &u, 4); out[k] = f; }
    else if (esz == 4) { const uint32_t u = (uint32_t)R.le(at, 4); out[k] = o.dsigned ? (double)(int32_t)u : (double)u; }
    else { const uint64_t u = R.le(at, 8); out[k] = o.dsigned ? (double)(int64_t)u : (double)u; }
  }
  return 0;
}

extern "C" int qpad_h5_read_attr(const char* path, const char* object, const char* attr, double* value, char* text,
                                 int64_t text_cap) {
  h5::Reader R;
  uint64_t root;
  if (!path || !attr || !h5::open_file(R, path, root)) { g_h5err = R.err.empty() ? "h5 attr: bad arguments" : R.err; return QPAD_E_ARG; }
  h5::ObjInfo o;
  if (!h5::lookup(R, root, object ? object : "", o)) { g_h5err = R.err; return QPAD_E_ARG; }
  auto it = o.attr_raw.find(attr);
  if (it == o.attr_raw.end()) { g_h5err = std::string("no attribute ") + attr; return QPAD_E_ARG; }
  const auto ty = o.attr_type[attr];
  const std::vector<uint8_t>& raw = it->second;
  if (ty.first == 3) {
    if (text && text_cap > 0) {
      const size_t n = std::min((size_t)text_cap - 1, raw.size());
      memcpy(text, raw.data(), n);
      text[n] = 0;
    }
    return 0;
  }
  if (!value || raw.size() < (size_t)ty.second) { g_h5err = "h5 attr: no value"; return QPAD_E_ARG; }
  uint64_t u = 0;
  for (int k = 0; k < ty.second; ++k) u |= (uint64_t)raw[k] << (8 * k);
  if (ty.first == 1 && ty.second == 8) memcpy(value, &u, 8);
  else if (ty.first == 1 && ty.second == 4) { uint32_t v = (uint32_t)u; float f; memcpy(&f, &v, 4); *value = f; }
  else if (ty.first == 0 && ty.second == 4) *value = (double)(int32_t)(uint32_t)u;
  else if (ty.first == 0 && ty.second == 8) *value = (double)(int64_t)u;
  else { g_h5err = "h5 attr: unsupported type"; return QPAD_E_ARG; }
  return 0;
}

// ---- the reference's file sets on top ------------------------------------------------------
extern "C" int qpad_diag_write_field(qpad_ctx* ctx, int field, int comp, const char* dir, const char* dataname,
                                     const char* units, const char* label, int iter, double time, double dt) {
  if (!ctx || !dir || !dataname || field < 0 || field >= QPAD_NFIELDS || comp < 0 || comp >= qpad::field_ncomp(field))
    return ctx ? qpad::set_err(ctx, QPAD_E_ARG, "diag field: bad arguments") : QPAD_E_ARG;
  const int nr = ctx->g.nr, nz = ctx->g.nz, P = ctx->g.P, nc = qpad::field_ncomp(field), ld = ctx->g.ld;
  std::vector<double> store((size_t)nz * P * nc * ld);
  if (int r = qpad_store_read(ctx, field, 1, nz, store.data())) return r;    // (refuses fields without a store)
  qpad_h5_grid_info info = {};
  info.time = time; info.iter = iter; info.dt = dt; info.timeunit = "1 / \\omega_p";
  info.units = units ? units : "a.u."; info.label = label ? label : dataname;
  info.axis_min[0] = 0.0; info.axis_max[0] = nr * ctx->g.dr;
  info.axis_min[1] = 0.0; info.axis_max[1] = nz * ctx->g.dxi;
  for (int k = 0; k < 2; ++k) {
    info.axis_name[k] = k == 0 ? "r" : "\\xi";
    info.axis_label[k] = k == 0 ? "r" : "\\xi";
    info.axis_units[k] = "c / \\omega_p";
  }
  std::vector<double> slab((size_t)nz * nr);
  for (int p = 0; p < P; ++p) {
    for (int s = 0; s < nz; ++s)
      for (int i = 0; i < nr; ++i) slab[(size_t)s * nr + i] = store[(((size_t)s * P + p) * nc + comp) * ld + i + 1];
    std::string d = dir;
    if (!d.empty() && d.back() != '/') d += '/';
    const std::string path = step_file((d + field_dir_part(p) + "/").c_str(), dataname, iter);
    if (int r = qpad_h5_write_grid(path.c_str(), dataname, slab.data(), nz, nr, &info))
      return qpad::set_err(ctx, r, g_h5err);
  }
  return 0;
}

extern "C" int qpad_beam_write_rst(qpad_beam* bm, const char* path, const char* dataname, int iter, double time,
                                   double dt) {
  if (!bm || !path || !dataname) return QPAD_E_ARG;
  int64_t n = 0;
  if (int r = qpad_beam_count(bm, &n)) return r;
  std::vector<double> x((size_t)3 * (n ? n : 1)), p((size_t)3 * (n ? n : 1)), q((size_t)(n ? n : 1));
  int64_t got = 0;
  if (int r = qpad_beam_download(bm, x.data(), p.data(), q.data(), &got)) return r;
  return qpad_h5_write_particles(path, dataname, x.data(), p.data(), q.data(), got, iter, time, dt);
}

extern "C" int qpad_rst_read(const char* path, double* x, double* p, double* q, int64_t cap, int64_t* n) {
  double tp = 0.0;
  if (int r = qpad_h5_read_attr(path, "", "tp", &tp, nullptr, 0)) return r;
  const int64_t np = (int64_t)tp;
  if (n) *n = np;
  if (!x && !p && !q) return 0;
  if (np > cap) { g_h5err = "restart read: buffer too small"; return QPAD_E_CAPACITY; }
  if (np == 0) return 0;
  int64_t cnt = 0;
  if (int r = qpad_h5_read_dataset(path, "x", x, 3 * cap, &cnt, nullptr, nullptr)) return r;
  if (int r = qpad_h5_read_dataset(path, "p", p, 3 * cap, &cnt, nullptr, nullptr)) return r;
  if (int r = qpad_h5_read_dataset(path, "q", q, cap, &cnt, nullptr, nullptr)) return r;
  return 0;
}
