// HDF5 subset reader and writer; the format choices are listed in h5file.h.
//
// Structure sizes below assume 8-byte offsets and lengths when writing (the
// libhdf5 default); the reader takes the sizes from the superblock.
#include "h5file.h"

#include <algorithm>
#include <cstring>
#include <set>

#include "htr_rhs.h"

namespace htr {
namespace h5 {

namespace {

// ---------------------------------------------------------------- encoding

struct Buf {
  std::vector<uint8_t> b;
  void u8(uint64_t v) { b.push_back(static_cast<uint8_t>(v)); }
  void uint(uint64_t v, int bytes) {
    for (int k = 0; k < bytes; k++) b.push_back(static_cast<uint8_t>(v >> (8 * k)));
  }
  void u16(uint64_t v) { uint(v, 2); }
  void u32(uint64_t v) { uint(v, 4); }
  void u64(uint64_t v) { uint(v, 8); }
  void zeros(size_t n) { b.insert(b.end(), n, 0); }
  void bytes(const void *p, size_t n) {
    const uint8_t *q = static_cast<const uint8_t *>(p);
    b.insert(b.end(), q, q + n);
  }
  void pad8() { zeros((8 - b.size() % 8) % 8); }
  // NUL-terminated name padded with NULs to a multiple of 8 bytes
  void name8(const std::string &s) {
    bytes(s.data(), s.size());
    zeros(8 - s.size() % 8);
  }
  size_t size() const { return b.size(); }
};

uint64_t align8(uint64_t v) { return (v + 7) & ~uint64_t(7); }

// a * b, or kOverflow when the product does not fit in 64 bits (a file can
// declare dimensions whose product wraps; every size derived from them is
// checked against the bytes actually present, which kOverflow never passes)
constexpr uint64_t kOverflow = ~uint64_t(0);
uint64_t mul_checked(uint64_t a, uint64_t b) {
  if (a == kOverflow || b == kOverflow) return kOverflow;
  if (a != 0 && b > kOverflow / a) return kOverflow;
  return a * b;
}

uint64_t product(const std::vector<uint64_t> &dims) {
  uint64_t n = 1;
  for (uint64_t d : dims) n = mul_checked(n, d);
  return n;
}

// element `index` of `size` bytes lies inside `bytes` bytes of data
bool element_inside(uint64_t index, uint64_t size, uint64_t bytes) {
  const uint64_t end = mul_checked(index + 1 == 0 ? kOverflow : index + 1, size);
  return end != kOverflow && end <= bytes;
}

bool has_array_member(const Type &t) {
  for (const auto &m : t.members)
    if (m.type->cls == Type::kArray) return true;
  return false;
}

// Datatype message body.  Versions: 1 for atomic types and compounds of
// atomic members, 2 for arrays and compounds holding arrays (libhdf5's
// choice for the earliest format).
void encode_type(Buf &o, const Type &t) {
  switch (t.cls) {
    case Type::kFixed:
      o.u8(0x10);
      o.u8((t.big_endian ? 0x01 : 0) | (t.is_signed ? 0x08 : 0));
      o.u8(0);
      o.u8(0);
      o.u32(t.size);
      o.u16(0);           // bit offset
      o.u16(t.size * 8);  // precision
      break;
    case Type::kFloat:  // IEEE binary64, little-endian, implied leading mantissa bit
      o.u8(0x11);
      o.u8(0x20);
      o.u8(63);  // sign bit position
      o.u8(0);
      o.u32(8);
      o.u16(0);
      o.u16(64);
      o.u8(52);  // exponent position and size
      o.u8(11);
      o.u8(0);  // mantissa position and size
      o.u8(52);
      o.u32(1023);
      break;
    case Type::kString:
      o.u8(0x13);
      o.u8(t.pad & 0x0f);  // ASCII
      o.u8(0);
      o.u8(0);
      o.u32(t.size);
      break;
    case Type::kCompound: {
      const int version = has_array_member(t) ? 2 : 1;
      const size_t n = t.members.size();
      o.u8((version << 4) | 6);
      o.u8(n & 0xff);
      o.u8((n >> 8) & 0xff);
      o.u8(0);
      o.u32(t.size);
      for (const auto &m : t.members) {
        o.name8(m.name);
        o.u32(m.offset);
        if (version == 1) {
          o.u8(0);     // dimensionality
          o.zeros(3);  // reserved
          o.u32(0);    // dimension permutation
          o.u32(0);    // reserved
          o.zeros(16); // dimension sizes
        }
        encode_type(o, *m.type);
      }
      break;
    }
    case Type::kArray:
      o.u8(0x2a);
      o.u8(0);
      o.u8(0);
      o.u8(0);
      o.u32(t.size);
      o.u8(t.dims.size());
      o.zeros(3);
      for (uint32_t d : t.dims) o.u32(d);
      for (size_t i = 0; i < t.dims.size(); i++) o.u32(i);  // permutation (unused by readers)
      encode_type(o, *t.base);
      break;
    default:
      break;
  }
}

// Dataspace message, version 1 (rank 0 = scalar).
void encode_space(Buf &o, const std::vector<uint64_t> &dims, bool max_dims) {
  o.u8(1);
  o.u8(dims.size());
  o.u8(max_dims ? 1 : 0);
  o.u8(0);
  o.u32(0);
  for (uint64_t d : dims) o.u64(d);
  if (max_dims)
    for (uint64_t d : dims) o.u64(d);
}

struct Msg {
  uint16_t type;
  uint8_t flags;
  std::vector<uint8_t> data;  // padded to a multiple of 8
};

Msg attribute_message(const std::string &name, const Value &v) {
  Buf dt, ds;
  encode_type(dt, v.type);
  encode_space(ds, v.dims, false);
  Buf o;
  o.u8(1);
  o.u8(0);
  o.u16(name.size() + 1);
  o.u16(dt.size());
  o.u16(ds.size());
  o.name8(name);
  o.bytes(dt.b.data(), dt.size());
  o.pad8();
  o.bytes(ds.b.data(), ds.size());
  o.pad8();
  o.bytes(v.data.data(), v.data.size());
  o.pad8();
  return {0x000c, 0, o.b};
}

// Version-1 object header: 16-byte prefix, then the messages.
std::vector<uint8_t> object_header(const std::vector<Msg> &msgs) {
  size_t body = 0;
  for (const auto &m : msgs) body += 8 + m.data.size();
  Buf o;
  o.u8(1);
  o.u8(0);
  o.u16(msgs.size());
  o.u32(1);  // reference count
  o.u32(body);
  o.u32(0);  // alignment of the first message to 8 bytes
  for (const auto &m : msgs) {
    o.u16(m.type);
    o.u16(m.data.size());
    o.u8(m.flags);
    o.zeros(3);
    o.bytes(m.data.data(), m.data.size());
  }
  return o.b;
}

constexpr int kLeafK = 4;       // symbol table node capacity 2K = 8 entries
constexpr int kInternalK = 16;  // B-tree node capacity 2K = 32 children
constexpr uint64_t kSuperblockSize = 96;
constexpr uint64_t kHeapHeaderSize = 32;
constexpr uint64_t kBtreeNodeSize = 24 + (2 * kInternalK + 1) * 8 + 2 * kInternalK * 8;
constexpr uint64_t kSnodSize = 8 + 2 * kLeafK * 40;

// ---------------------------------------------------------------- decoding

struct Cur {
  const uint8_t *p;
  size_t n;
  size_t i = 0;
  bool bad = false;
  Cur(const uint8_t *p_, size_t n_) : p(p_), n(n_) {}
  explicit Cur(const std::vector<uint8_t> &v) : p(v.data()), n(v.size()) {}
  bool need(size_t k) {
    if (bad || k > n || i > n - k) {
      bad = true;
      return false;
    }
    return true;
  }
  uint64_t uint(int bytes) {
    if (!need(bytes)) return 0;
    uint64_t v = 0;
    for (int k = 0; k < bytes; k++) v |= uint64_t(p[i + k]) << (8 * k);
    i += bytes;
    return v;
  }
  uint64_t addr(int bytes) {
    uint64_t v = uint(bytes);
    if (bytes < 8 && v == (uint64_t(1) << (8 * bytes)) - 1) return kUndef;
    return v;
  }
  uint8_t u8() { return static_cast<uint8_t>(uint(1)); }
  uint16_t u16() { return static_cast<uint16_t>(uint(2)); }
  uint32_t u32() { return static_cast<uint32_t>(uint(4)); }
  void skip(size_t k) {
    if (need(k)) i += k;
  }
  std::string cstr() {
    size_t j = i;
    while (j < n && p[j] != 0) j++;
    if (j >= n) {
      bad = true;
      return {};
    }
    std::string s(reinterpret_cast<const char *>(p + i), j - i);
    i = j + 1;
    return s;
  }
  size_t left() const { return bad ? 0 : n - i; }
};

// number of bytes that hold the member offsets of a version-3 compound
int offset_bytes(uint32_t size) {
  if (size < (1u << 8)) return 1;
  if (size < (1u << 16)) return 2;
  if (size < (1u << 24)) return 3;
  return 4;
}

// Decodes one datatype at the cursor; false if it could not be decoded far
// enough to know where it ends.
bool decode_type(Cur &c, Type &t, int depth = 0) {
  if (depth > 16) return false;
  const uint8_t b0 = c.u8();
  const int version = b0 >> 4;
  const int cls = b0 & 0x0f;
  const uint8_t bf0 = c.u8(), bf1 = c.u8();
  c.u8();
  t = Type();
  t.raw_class = cls;
  t.size = c.u32();
  if (c.bad) return false;
  switch (cls) {
    case 0: {  // fixed-point
      t.big_endian = bf0 & 0x01;
      t.is_signed = bf0 & 0x08;
      const uint16_t off = c.u16(), prec = c.u16();
      t.cls = (off == 0 && prec == t.size * 8) ? Type::kFixed : Type::kOther;
      break;
    }
    case 1: {  // floating point
      t.big_endian = (bf0 & 0x01) != 0;
      const bool vax = (bf0 & 0x40) != 0;
      const int norm = (bf0 >> 4) & 0x03;
      const uint8_t sign = bf1;
      const uint16_t off = c.u16(), prec = c.u16();
      const uint8_t eloc = c.u8(), esize = c.u8(), mloc = c.u8(), msize = c.u8();
      const uint32_t bias = c.u32();
      t.cls = Type::kFloat;
      t.ieee64 = !vax && t.size == 8 && off == 0 && prec == 64 && eloc == 52 && esize == 11 &&
                 mloc == 0 && msize == 52 && bias == 1023 && sign == 63 && norm == 2;
      break;
    }
    case 2:  // time
      c.skip(2);
      break;
    case 3:  // string
      t.cls = Type::kString;
      t.pad = bf0 & 0x0f;
      break;
    case 4:  // bit field
      c.skip(4);
      break;
    case 5: {  // opaque: ASCII tag, NUL-padded to a multiple of 8
      c.skip(bf0);
      break;
    }
    case 6: {  // compound
      const unsigned n = bf0 | (unsigned(bf1) << 8);
      bool all_known = true;
      for (unsigned k = 0; k < n; k++) {
        Type::Member m;
        const size_t start = c.i;
        m.name = c.cstr();
        if (version < 3) {
          const size_t used = c.i - start;  // name with its NUL
          c.skip((8 - used % 8) % 8);
          m.offset = c.u32();
          if (version == 1) {
            const uint8_t ndims = c.u8();
            c.skip(3 + 4 + 4 + 16);
            if (ndims != 0) all_known = false;  // old-style array member
          }
        } else {
          m.offset = static_cast<uint32_t>(c.uint(offset_bytes(t.size)));
        }
        m.type = std::make_shared<Type>();
        if (!decode_type(c, *m.type, depth + 1)) return false;
        if (m.type->cls == Type::kOther) all_known = false;
        t.members.push_back(std::move(m));
      }
      t.cls = all_known ? Type::kCompound : Type::kOther;
      break;
    }
    case 7:  // reference
      break;
    case 8: {  // enumeration: base type, names, values
      const unsigned n = bf0 | (unsigned(bf1) << 8);
      Type base;
      if (!decode_type(c, base, depth + 1)) return false;
      for (unsigned k = 0; k < n; k++) {
        const size_t start = c.i;
        c.cstr();
        if (version < 3) c.skip((8 - (c.i - start) % 8) % 8);
      }
      c.skip(size_t(n) * base.size);
      break;
    }
    case 9: {  // variable length
      Type base;
      if (!decode_type(c, base, depth + 1)) return false;
      break;
    }
    case 10: {  // array
      if (version < 2) return false;
      const uint8_t rank = c.u8();
      if (version == 2) c.skip(3);
      for (int k = 0; k < rank; k++) t.dims.push_back(c.u32());
      if (version == 2) c.skip(4 * size_t(rank));
      t.base = std::make_shared<Type>();
      if (!decode_type(c, *t.base, depth + 1)) return false;
      t.cls = t.base->cls == Type::kOther ? Type::kOther : Type::kArray;
      break;
    }
    default:
      return false;
  }
  return !c.bad;
}

// Bob Jenkins' lookup3 `hashlittle` (public domain, 2006), byte-wise form:
// the checksum HDF5 stores after metadata blocks of its newer format
// versions (superblock 2/3, version-2 object headers), with initial value 0.
uint32_t lookup3(const uint8_t *k, size_t length, uint32_t initval) {
  auto rot = [](uint32_t x, int s) { return (x << s) | (x >> (32 - s)); };
  auto word = [](const uint8_t *q) {
    return uint32_t(q[0]) | uint32_t(q[1]) << 8 | uint32_t(q[2]) << 16 | uint32_t(q[3]) << 24;
  };
  uint32_t a, b, c;
  a = b = c = 0xdeadbeefu + static_cast<uint32_t>(length) + initval;
  while (length > 12) {
    a += word(k);
    b += word(k + 4);
    c += word(k + 8);
    a -= c; a ^= rot(c, 4);  c += b;
    b -= a; b ^= rot(a, 6);  a += c;
    c -= b; c ^= rot(b, 8);  b += a;
    a -= c; a ^= rot(c, 16); c += b;
    b -= a; b ^= rot(a, 19); a += c;
    c -= b; c ^= rot(b, 4);  b += a;
    length -= 12;
    k += 12;
  }
  switch (length) {  // the last 1..12 bytes
    case 12: c += uint32_t(k[11]) << 24; [[fallthrough]];
    case 11: c += uint32_t(k[10]) << 16; [[fallthrough]];
    case 10: c += uint32_t(k[9]) << 8;   [[fallthrough]];
    case 9:  c += k[8];                  [[fallthrough]];
    case 8:  b += uint32_t(k[7]) << 24;  [[fallthrough]];
    case 7:  b += uint32_t(k[6]) << 16;  [[fallthrough]];
    case 6:  b += uint32_t(k[5]) << 8;   [[fallthrough]];
    case 5:  b += k[4];                  [[fallthrough]];
    case 4:  a += uint32_t(k[3]) << 24;  [[fallthrough]];
    case 3:  a += uint32_t(k[2]) << 16;  [[fallthrough]];
    case 2:  a += uint32_t(k[1]) << 8;   [[fallthrough]];
    case 1:  a += k[0]; break;
    case 0:  return c;
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

struct Space {
  std::vector<uint64_t> dims;
  bool null = false;
};

bool decode_space(Cur &c, int sl, Space &s, Status &st) {
  const uint8_t version = c.u8();
  const uint8_t rank = c.u8();
  const uint8_t flags = c.u8();
  if (version == 1) {
    c.skip(5);
  } else if (version == 2) {
    const uint8_t type = c.u8();
    s.null = (type == 2);
  } else {
    st = {HTR_ERR_UNSUPPORTED, "dataspace message version " + std::to_string(version)};
    return false;
  }
  for (int k = 0; k < rank; k++) s.dims.push_back(c.uint(sl));
  if (flags & 0x01) c.skip(size_t(rank) * sl);
  if (c.bad) {
    st = {HTR_ERR_FORMAT, "truncated dataspace message"};
    return false;
  }
  return true;
}

}  // namespace

// ---------------------------------------------------------------- Type

Type Type::f64() {
  Type t;
  t.cls = kFloat;
  t.raw_class = 1;
  t.size = 8;
  t.ieee64 = true;
  return t;
}

Type Type::integer(uint32_t bytes, bool is_signed) {
  Type t;
  t.cls = kFixed;
  t.raw_class = 0;
  t.size = bytes;
  t.is_signed = is_signed;
  return t;
}

Type Type::string(uint32_t bytes) {
  Type t;
  t.cls = kString;
  t.raw_class = 3;
  t.size = bytes;
  return t;
}

Type Type::array(const Type &base, std::vector<uint32_t> dims) {
  Type t;
  t.cls = kArray;
  t.raw_class = 10;
  t.base = std::make_shared<Type>(base);
  uint64_t n = 1;
  for (uint32_t d : dims) n *= d;
  t.dims = std::move(dims);
  t.size = static_cast<uint32_t>(n * base.size);
  return t;
}

Type Type::compound(uint32_t size, std::vector<Member> members) {
  Type t;
  t.cls = kCompound;
  t.raw_class = 6;
  t.size = size;
  t.members = std::move(members);
  return t;
}

bool Type::is_f64_elements(uint64_t *count) const {
  if (cls == kFloat && ieee64 && !big_endian) {
    *count = 1;
    return true;
  }
  if (cls == kArray && base && base->cls == kFloat && base->ieee64 && !base->big_endian) {
    uint64_t n = 1;
    for (uint32_t d : dims) n = mul_checked(n, d);
    if (n == kOverflow) return false;
    *count = n;
    return true;
  }
  return false;
}

const Type::Member *Type::member(const std::string &name) const {
  for (const auto &m : members)
    if (m.name == name) return &m;
  return nullptr;
}

uint64_t Value::elements() const { return product(dims); }
uint64_t Dataset::elements() const { return product(dims); }

// ---------------------------------------------------------------- Writer

void Writer::attribute(const std::string &name, Value v) { attrs_.emplace_back(name, std::move(v)); }

void Writer::dataset(const std::string &name, const Type &type, std::vector<uint64_t> dims,
                     std::function<bool(FILE *)> emit, bool max_dims) {
  sets_.push_back({name, type, std::move(dims), max_dims, std::move(emit)});
}

Status Writer::write(const std::string &path) const {
  for (const auto &s : sets_)
    if (s.name.empty() || s.name.find('/') != std::string::npos)
      return {HTR_ERR_ARGUMENT, "dataset name '" + s.name + "' must be a plain name"};
  for (const auto &a : attrs_) {
    const Value &v = a.second;
    if (v.data.size() != mul_checked(v.elements(), v.type.size))
      return {HTR_ERR_ARGUMENT, "attribute '" + a.first + "' holds the wrong number of bytes"};
  }

  // link names in the order the symbol table keeps them
  std::vector<size_t> order(sets_.size());
  for (size_t i = 0; i < order.size(); i++) order[i] = i;
  std::sort(order.begin(), order.end(),
            [&](size_t a, size_t b) { return std::strcmp(sets_[a].name.c_str(), sets_[b].name.c_str()) < 0; });
  for (size_t i = 1; i < order.size(); i++)
    if (sets_[order[i]].name == sets_[order[i - 1]].name)
      return {HTR_ERR_ARGUMENT, "duplicate dataset name '" + sets_[order[i]].name + "'"};
  const size_t nsnod = (sets_.size() + 2 * kLeafK - 1) / (2 * kLeafK);
  if (nsnod > 2 * kInternalK) return {HTR_ERR_ARGUMENT, "too many datasets for one group node"};

  // local heap: "" at offset 0, then the names, then one free block
  Buf names;
  names.zeros(8);
  std::vector<uint64_t> name_off(sets_.size());
  for (size_t k : order) {
    name_off[k] = names.size();
    names.name8(sets_[k].name);
  }
  const uint64_t free_at = names.size();
  names.u64(1);   // next free block: none (the on-disk end-of-list value)
  names.u64(16);  // size of this free block

  const uint64_t heap_at = kSuperblockSize;
  const uint64_t heap_data_at = heap_at + kHeapHeaderSize;
  const uint64_t btree_at = align8(heap_data_at + names.size());
  const uint64_t snod_at = btree_at + kBtreeNodeSize;

  // dataset object headers (sizes do not depend on the addresses)
  std::vector<uint64_t> data_bytes(sets_.size());
  std::vector<std::vector<Msg>> set_msgs(sets_.size());
  for (size_t k = 0; k < sets_.size(); k++) {
    const auto &s = sets_[k];
    data_bytes[k] = mul_checked(product(s.dims), s.type.size);
    if (data_bytes[k] == kOverflow) return {HTR_ERR_ARGUMENT, "dataset '" + s.name + "' is too large"};
    Buf fill, dt, ds, layout;
    // fill value message version 1: late allocation, fill written if set,
    // default (zero) fill value, as libhdf5 writes it for a default dataset
    fill.u8(1);
    fill.u8(2);
    fill.u8(2);
    fill.u8(1);
    fill.u32(0);
    encode_type(dt, s.type);
    dt.pad8();
    encode_space(ds, s.dims, s.max_dims);
    ds.pad8();
    layout.u8(3);
    layout.u8(1);  // contiguous
    layout.u64(kUndef);
    layout.u64(data_bytes[k]);
    layout.pad8();
    set_msgs[k] = {{0x0005, 1, fill.b}, {0x0003, 1, dt.b}, {0x0001, 0, ds.b}, {0x0008, 1, layout.b}};
  }
  std::vector<Msg> root_msgs;
  {
    Buf stab;
    stab.u64(btree_at);
    stab.u64(heap_at);
    root_msgs.push_back({0x0011, 1, stab.b});
    for (const auto &a : attrs_) {
      Msg m = attribute_message(a.first, a.second);
      if (m.data.size() > 0xffff) return {HTR_ERR_ARGUMENT, "attribute '" + a.first + "' is too large"};
      root_msgs.push_back(std::move(m));
    }
  }
  const uint64_t root_at = snod_at + nsnod * kSnodSize;
  uint64_t at = root_at + object_header(root_msgs).size();
  std::vector<uint64_t> oh_at(sets_.size());
  for (size_t k = 0; k < sets_.size(); k++) {
    oh_at[k] = at;
    at += 16 + 8 * set_msgs[k].size() + [&] {
      size_t n = 0;
      for (const auto &m : set_msgs[k]) n += m.data.size();
      return n;
    }();
  }
  // contiguous data, each block on a 16-byte boundary
  std::vector<uint64_t> data_at(sets_.size());
  for (size_t k = 0; k < sets_.size(); k++) {
    at = (at + 15) & ~uint64_t(15);
    data_at[k] = data_bytes[k] ? at : kUndef;
    at += data_bytes[k];
    // the layout message's address sits at offset 2 of its body
    std::vector<uint8_t> &lay = set_msgs[k][3].data;
    for (int b = 0; b < 8; b++) lay[2 + b] = static_cast<uint8_t>(data_at[k] >> (8 * b));
  }
  const uint64_t eof = at;

  Buf meta;
  // superblock version 0
  const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
  meta.bytes(sig, 8);
  meta.u8(0);  // superblock version
  meta.u8(0);  // free-space storage version
  meta.u8(0);  // root symbol table entry version
  meta.u8(0);
  meta.u8(0);  // shared header message format version
  meta.u8(8);  // size of offsets
  meta.u8(8);  // size of lengths
  meta.u8(0);
  meta.u16(kLeafK);
  meta.u16(kInternalK);
  meta.u32(0);  // file consistency flags
  meta.u64(0);  // base address
  meta.u64(kUndef);
  meta.u64(eof);
  meta.u64(kUndef);
  meta.u64(0);  // root entry: link name offset
  meta.u64(root_at);
  meta.u32(1);  // cache type: B-tree and heap addresses cached
  meta.u32(0);
  meta.u64(btree_at);
  meta.u64(heap_at);
  // local heap
  meta.bytes("HEAP", 4);
  meta.u8(0);
  meta.zeros(3);
  meta.u64(names.size());
  meta.u64(free_at);
  meta.u64(heap_data_at);
  meta.bytes(names.b.data(), names.size());
  meta.zeros(btree_at - meta.size());
  // B-tree node (group, leaf level) over the symbol table nodes
  {
    const size_t start = meta.size();
    meta.bytes("TREE", 4);
    meta.u8(0);
    meta.u8(0);
    meta.u16(nsnod);
    meta.u64(kUndef);
    meta.u64(kUndef);
    meta.u64(0);  // key 0: the empty name
    for (size_t s = 0; s < nsnod; s++) {
      meta.u64(snod_at + s * kSnodSize);
      const size_t last = std::min(sets_.size(), (s + 1) * 2 * kLeafK) - 1;
      meta.u64(name_off[order[last]]);
    }
    meta.zeros(start + kBtreeNodeSize - meta.size());
  }
  // symbol table nodes
  for (size_t s = 0; s < nsnod; s++) {
    const size_t start = meta.size();
    const size_t first = s * 2 * kLeafK;
    const size_t count = std::min(sets_.size() - first, size_t(2 * kLeafK));
    meta.bytes("SNOD", 4);
    meta.u8(1);
    meta.u8(0);
    meta.u16(count);
    for (size_t e = 0; e < count; e++) {
      const size_t k = order[first + e];
      meta.u64(name_off[k]);
      meta.u64(oh_at[k]);
      meta.u32(0);
      meta.u32(0);
      meta.zeros(16);
    }
    meta.zeros(start + kSnodSize - meta.size());
  }
  {
    auto oh = object_header(root_msgs);
    meta.bytes(oh.data(), oh.size());
  }
  for (size_t k = 0; k < sets_.size(); k++) {
    auto oh = object_header(set_msgs[k]);
    meta.bytes(oh.data(), oh.size());
  }

  const std::string tmp = path + ".partial";
  FILE *f = std::fopen(tmp.c_str(), "wb");
  if (f == nullptr) return {HTR_ERR_IO, "cannot create " + tmp};
  bool ok = std::fwrite(meta.b.data(), 1, meta.size(), f) == meta.size();
  uint64_t pos = meta.size();
  static const uint8_t kZeros[16] = {};
  for (size_t k = 0; ok && k < sets_.size(); k++) {
    if (data_bytes[k] == 0) continue;
    ok = std::fwrite(kZeros, 1, data_at[k] - pos, f) == data_at[k] - pos;
    ok = ok && sets_[k].emit(f);
    pos = data_at[k] + data_bytes[k];
    ok = ok && static_cast<uint64_t>(ftello(f)) == pos;
  }
  ok = ok && pos == eof;
  if (std::fclose(f) != 0) ok = false;
  if (!ok) {
    std::remove(tmp.c_str());
    return {HTR_ERR_IO, "writing " + path + " failed"};
  }
  if (std::rename(tmp.c_str(), path.c_str()) != 0) {
    std::remove(tmp.c_str());
    return {HTR_ERR_IO, "cannot rename " + tmp + " to " + path};
  }
  return {};
}

// ---------------------------------------------------------------- Reader

struct Parser {
  Reader &r;
  Status st;
  int so = 8;  // size of offsets
  int sl = 8;  // size of lengths
  std::set<uint64_t> visited;
  size_t nodes = 0;  // B-tree nodes read (bounds the work on a corrupt file)

  explicit Parser(Reader &r_) : r(r_) {}

  bool fail(int code, const std::string &msg) {
    if (st.ok()) st = {code, msg};
    return false;
  }
  bool read_abs(uint64_t at, void *dst, size_t n) {
    if (at > r.size_ || n > r.size_ - at) return fail(HTR_ERR_FORMAT, "truncated file (structure beyond its end)");
    if (fseeko(r.f_, static_cast<off_t>(at), SEEK_SET) != 0 || std::fread(dst, 1, n, r.f_) != n)
      return fail(HTR_ERR_IO, "read error");
    return true;
  }
  bool block(uint64_t rel, size_t n, std::vector<uint8_t> &out) {
    if (rel == kUndef) return fail(HTR_ERR_FORMAT, "undefined address");
    if (rel > r.size_ || r.base_ > r.size_ - rel || n > r.size_ - r.base_ - rel)
      return fail(HTR_ERR_FORMAT, "truncated file (structure beyond its end)");
    out.resize(n);
    return read_abs(r.base_ + rel, out.data(), n);
  }

  bool superblock() {
    const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    uint64_t at = 0;
    for (;;) {
      if (at + 8 > r.size_) return fail(HTR_ERR_FORMAT, "not an HDF5 file (no signature)");
      uint8_t s[8];
      if (!read_abs(at, s, 8)) return false;
      if (std::memcmp(s, sig, 8) == 0) break;
      at = at ? at * 2 : 512;
    }
    std::vector<uint8_t> h(12);
    if (!read_abs(at, h.data(), 12)) return false;
    const int version = h[8];
    if (version > 3) return fail(HTR_ERR_UNSUPPORTED, "superblock version " + std::to_string(version));
    if (version < 2) {
      std::vector<uint8_t> v(24);
      if (!read_abs(at, v.data(), 24)) return false;
      so = v[13];
      sl = v[14];
    } else {
      so = h[9];
      sl = h[10];
    }
    if ((so != 2 && so != 4 && so != 8) || (sl != 2 && sl != 4 && sl != 8))
      return fail(HTR_ERR_FORMAT, "bad sizes of offsets/lengths");
    uint64_t eof = kUndef, root = kUndef;
    if (version >= 2) {
      // versions 2 and 3: addresses, root object header, lookup3 checksum
      const size_t n = 12 + 4 * size_t(so) + 4;
      std::vector<uint8_t> b(n);
      if (!read_abs(at, b.data(), n)) return false;
      Cur c(b.data() + 12, n - 12);
      r.base_ = c.addr(so);
      c.addr(so);  // superblock extension (file-space settings; not needed to read)
      eof = c.addr(so);
      root = c.addr(so);
      const uint32_t sum = c.u32();
      if (c.bad || sum != lookup3(b.data(), n - 4, 0)) return fail(HTR_ERR_FORMAT, "superblock checksum mismatch");
    } else {
      const size_t rest = (version == 1 ? 4 : 0) + 4 * so + (2 * so + 8 + 16);
      std::vector<uint8_t> b(rest);
      if (!read_abs(at + 24, b.data(), rest)) return false;
      Cur c(b);
      if (version == 1) c.skip(4);
      r.base_ = c.addr(so);
      c.addr(so);  // free-space info
      eof = c.addr(so);
      c.addr(so);  // driver info
      c.addr(so);  // root link name offset
      root = c.addr(so);
      if (c.bad) return fail(HTR_ERR_FORMAT, "bad root group entry");
    }
    if (root == kUndef) return fail(HTR_ERR_FORMAT, "no root group");
    if (eof != kUndef && eof > r.size_)
      return fail(HTR_ERR_FORMAT, "truncated file (" + std::to_string(r.size_) + " of " + std::to_string(eof) + " bytes)");
    return group(root, "", true);
  }

  // Messages of one object header block.  Version 1: 8-byte message
  // headers, bodies padded to 8.  Version 2: type (1), size (2), flags (1)
  // and a creation order (2) when the header tracks it; a gap smaller than
  // a message header may end the block.
  bool messages(const uint8_t *p, size_t n, int version, bool crt_order, std::vector<Msg> &msgs,
                std::vector<std::pair<uint64_t, uint64_t>> &chunks) {
    Cur c(p, n);
    const size_t hdr = version == 1 ? 8 : (crt_order ? 6 : 4);
    while (c.left() >= hdr) {
      uint16_t type, size;
      uint8_t flags;
      if (version == 1) {
        type = c.u16();
        size = c.u16();
        flags = c.u8();
        c.skip(3);
      } else {
        type = c.u8();
        size = c.u16();
        flags = c.u8();
        if (crt_order) c.skip(2);
      }
      if (!c.need(size)) return fail(HTR_ERR_FORMAT, "object header message beyond its block");
      Msg m{type, flags, std::vector<uint8_t>(c.p + c.i, c.p + c.i + size)};
      c.skip(size);
      if (type == 0x0010) {
        Cur k(m.data);
        const uint64_t addr = k.addr(so), len = k.uint(sl);
        if (k.bad || addr == kUndef) return fail(HTR_ERR_FORMAT, "bad continuation message");
        chunks.emplace_back(addr, len);
      }
      msgs.push_back(std::move(m));
      if (msgs.size() > 65536) return fail(HTR_ERR_FORMAT, "too many header messages");
    }
    return true;
  }

  // all messages of an object header (version 1, or version 2 "OHDR" with
  // "OCHK" continuation blocks and lookup3 checksums), continuations followed
  bool object(uint64_t rel, std::vector<Msg> &msgs) {
    std::vector<uint8_t> pre;
    if (!block(rel, 6, pre)) return false;
    std::vector<std::pair<uint64_t, uint64_t>> chunks;
    int version = 1;
    bool crt_order = false;
    if (std::memcmp(pre.data(), "OHDR", 4) == 0) {
      version = 2;
      if (pre[4] != 2) return fail(HTR_ERR_FORMAT, "bad object header version " + std::to_string(pre[4]));
      const uint8_t flags = pre[5];
      crt_order = (flags & 0x04) != 0;
      const size_t fixed = 6 + ((flags & 0x20) ? 16 : 0) + ((flags & 0x10) ? 4 : 0);
      const int szb = 1 << (flags & 0x03);
      std::vector<uint8_t> h;
      if (!block(rel, fixed + szb, h)) return false;
      Cur c(h.data() + fixed, szb);
      const uint64_t chunk0 = c.uint(szb);
      if (chunk0 > r.size_) return fail(HTR_ERR_FORMAT, "object header beyond the end of the file");
      const size_t total = fixed + szb + chunk0 + 4;
      std::vector<uint8_t> all;
      if (!block(rel, total, all)) return false;
      uint32_t sum = 0;
      for (int k = 0; k < 4; k++) sum |= uint32_t(all[total - 4 + k]) << (8 * k);
      if (sum != lookup3(all.data(), total - 4, 0)) return fail(HTR_ERR_FORMAT, "object header checksum mismatch");
      if (!messages(all.data() + fixed + szb, chunk0, 2, crt_order, msgs, chunks)) return false;
    } else {
      if (!block(rel, 16, pre)) return false;
      if (pre[0] != 1) return fail(HTR_ERR_FORMAT, "bad object header version " + std::to_string(pre[0]));
      Cur p(pre);
      p.skip(8);
      const uint32_t hsize = p.u32();
      chunks.emplace_back(rel + 16, hsize);
    }
    for (size_t ci = 0; ci < chunks.size(); ci++) {
      if (ci > 256) return fail(HTR_ERR_FORMAT, "too many object header continuation blocks");
      std::vector<uint8_t> body;
      if (!block(chunks[ci].first, chunks[ci].second, body)) return false;
      if (version == 1) {
        if (!messages(body.data(), body.size(), 1, false, msgs, chunks)) return false;
        continue;
      }
      if (body.size() < 8 || std::memcmp(body.data(), "OCHK", 4) != 0)
        return fail(HTR_ERR_FORMAT, "bad object header continuation block");
      uint32_t sum = 0;
      for (int k = 0; k < 4; k++) sum |= uint32_t(body[body.size() - 4 + k]) << (8 * k);
      if (sum != lookup3(body.data(), body.size() - 4, 0))
        return fail(HTR_ERR_FORMAT, "object header continuation checksum mismatch");
      if (!messages(body.data() + 4, body.size() - 8, 2, crt_order, msgs, chunks)) return false;
    }
    return true;
  }

  bool attribute(const Msg &m, std::string &name, Value &v) {
    Cur c(m.data);
    const uint8_t version = c.u8();
    const uint8_t flags = c.u8();
    const uint16_t nlen = c.u16(), dlen = c.u16(), slen = c.u16();
    if (version < 1 || version > 3) return fail(HTR_ERR_UNSUPPORTED, "attribute message version " + std::to_string(version));
    if (version >= 2 && (flags & 0x03)) return fail(HTR_ERR_UNSUPPORTED, "attribute with a shared datatype or dataspace");
    if (version == 3) c.u8();  // name character set
    auto padded = [&](size_t n) { return version == 1 ? align8(n) : n; };
    if (!c.need(padded(nlen))) return fail(HTR_ERR_FORMAT, "truncated attribute message");
    name.assign(reinterpret_cast<const char *>(c.p + c.i), nlen ? nlen - 1 : 0);
    name = name.c_str();
    c.skip(padded(nlen));
    if (!c.need(padded(dlen))) return fail(HTR_ERR_FORMAT, "truncated attribute message");
    {
      Cur t(c.p + c.i, dlen);
      if (!decode_type(t, v.type)) v.type = Type();
    }
    c.skip(padded(dlen));
    if (!c.need(padded(slen))) return fail(HTR_ERR_FORMAT, "truncated attribute message");
    Space s;
    {
      Cur t(c.p + c.i, slen);
      if (!decode_space(t, sl, s, st)) return false;
    }
    c.skip(padded(slen));
    v.dims = s.dims;
    const uint64_t bytes = s.null ? 0 : mul_checked(v.elements(), v.type.size);
    if (bytes == kOverflow) return fail(HTR_ERR_FORMAT, "attribute '" + name + "': size overflows");
    if (!c.need(bytes)) return fail(HTR_ERR_FORMAT, "attribute '" + name + "': data beyond its message");
    v.data.assign(c.p + c.i, c.p + c.i + bytes);
    return true;
  }

  bool local_heap(uint64_t rel, std::vector<uint8_t> &data) {
    std::vector<uint8_t> h;
    if (!block(rel, 8 + 2 * sl + so, h)) return false;
    if (std::memcmp(h.data(), "HEAP", 4) != 0) return fail(HTR_ERR_FORMAT, "bad local heap signature");
    Cur c(h);
    c.skip(8);
    const uint64_t size = c.uint(sl);
    c.uint(sl);
    const uint64_t at = c.addr(so);
    if (size > (uint64_t(1) << 32)) return fail(HTR_ERR_FORMAT, "implausible local heap size");
    return block(at, size, data);
  }

  static std::string heap_name(const std::vector<uint8_t> &heap, uint64_t off, bool &ok) {
    if (off >= heap.size()) {
      ok = false;
      return {};
    }
    size_t j = off;
    while (j < heap.size() && heap[j] != 0) j++;
    if (j == heap.size()) ok = false;
    return std::string(reinterpret_cast<const char *>(heap.data() + off), j - off);
  }

  bool btree(uint64_t rel, const std::vector<uint8_t> &heap,
             std::vector<std::pair<std::string, uint64_t>> &links, int depth, int expect_level = -1) {
    if (depth > 32 || ++nodes > 100000) return fail(HTR_ERR_FORMAT, "group B-tree too deep or too large");
    std::vector<uint8_t> h;
    if (!block(rel, 8 + 2 * so, h)) return false;
    if (std::memcmp(h.data(), "TREE", 4) != 0) return fail(HTR_ERR_FORMAT, "bad B-tree signature");
    if (h[4] != 0) return fail(HTR_ERR_FORMAT, "group B-tree node of type " + std::to_string(h[4]));
    const int level = h[5];
    if (expect_level >= 0 && level != expect_level) return fail(HTR_ERR_FORMAT, "B-tree levels out of order");
    const unsigned used = h[6] | (unsigned(h[7]) << 8);
    std::vector<uint8_t> kc;
    if (!block(rel + 8 + 2 * so, used * size_t(so + sl) + sl, kc)) return false;
    Cur c(kc);
    c.uint(sl);
    for (unsigned k = 0; k < used; k++) {
      const uint64_t child = c.addr(so);
      c.uint(sl);
      if (c.bad || child == kUndef) return fail(HTR_ERR_FORMAT, "bad B-tree child");
      if (level > 0) {
        if (!btree(child, heap, links, depth + 1, level - 1)) return false;
        continue;
      }
      std::vector<uint8_t> sh;
      if (!block(child, 8, sh)) return false;
      if (std::memcmp(sh.data(), "SNOD", 4) != 0) return fail(HTR_ERR_FORMAT, "bad symbol table node signature");
      const unsigned n = sh[6] | (unsigned(sh[7]) << 8);
      const size_t esize = 2 * size_t(so) + 24;
      std::vector<uint8_t> es;
      if (!block(child + 8, n * esize, es)) return false;
      Cur e(es);
      for (unsigned j = 0; j < n; j++) {
        const uint64_t name_off = e.uint(so);
        const uint64_t oh = e.addr(so);
        const uint32_t cache = e.u32();
        e.skip(4 + 16);
        bool ok = true;
        std::string name = heap_name(heap, name_off, ok);
        if (!ok) return fail(HTR_ERR_FORMAT, "bad link name offset");
        if (cache == 2 || oh == kUndef) continue;  // soft link
        links.emplace_back(name, oh);
        if (links.size() > 100000) return fail(HTR_ERR_FORMAT, "too many links");
      }
    }
    return !c.bad || fail(HTR_ERR_FORMAT, "truncated B-tree node");
  }

  // reads a checksummed block of `n` bytes (the last 4 are its lookup3
  // checksum) that starts with `sig`
  bool checked(uint64_t rel, size_t n, const char *sig, std::vector<uint8_t> &out) {
    if (!block(rel, n, out)) return false;
    if (std::memcmp(out.data(), sig, 4) != 0) return fail(HTR_ERR_FORMAT, std::string("bad ") + sig + " signature");
    uint32_t sum = 0;
    for (int k = 0; k < 4; k++) sum |= uint32_t(out[n - 4 + k]) << (8 * k);
    if (sum != lookup3(out.data(), n - 4, 0)) return fail(HTR_ERR_FORMAT, std::string(sig) + " checksum mismatch");
    return true;
  }

  // Objects of dense storage: messages kept as objects of a fractal heap,
  // found through a version-2 B-tree of name records — type 5 for links
  // (name hash, heap ID), type 8 for attributes (heap ID, message flags,
  // creation order, name hash).  Handled: an unfiltered heap that is one
  // root direct block and a B-tree that is one root leaf — the shape of up
  // to about fifteen short links or a few attributes, more than any restart
  // file has; a larger heap or tree is reported as unsupported.
  bool dense_objects(uint64_t fheap, uint64_t bt2, int want, std::vector<std::vector<uint8_t>> &objects) {
    const char *what = want == 5 ? "link" : "attribute";
    const size_t hsize = 4 + 1 + 2 + 2 + 1 + 4 + 12 * size_t(sl) + 3 * size_t(so) + 2 + 2 + 2 + 2 + 4;
    std::vector<uint8_t> h;
    if (!checked(fheap, hsize, "FRHP", h)) return false;
    Cur c(h.data() + 4, hsize - 4);
    if (c.u8() != 0) return fail(HTR_ERR_UNSUPPORTED, "fractal heap version");
    const uint16_t id_len = c.u16(), filt_len = c.u16();
    c.u8();   // flags
    c.u32();  // maximum size of managed objects
    c.uint(sl);
    c.addr(so);  // huge objects
    c.uint(sl);
    c.addr(so);  // free-space manager
    for (int k = 0; k < 8; k++) c.uint(sl);  // managed space, iterator, object counts and sizes
    const uint16_t width = c.u16();
    const uint64_t start_block = c.uint(sl), max_direct = c.uint(sl);
    const uint16_t max_bits = c.u16();
    c.u16();  // starting rows of the root indirect block
    const uint64_t root = c.addr(so);
    const uint16_t rows = c.u16();
    if (c.bad) return fail(HTR_ERR_FORMAT, "truncated fractal heap header");
    if (filt_len != 0) return fail(HTR_ERR_UNSUPPORTED, "filtered fractal heap");
    const int off_size = (max_bits + 7) / 8;
    const int len_size = int(id_len) - 1 - off_size;
    if (width == 0 || start_block == 0 || max_direct < start_block || off_size < 1 || off_size > 8 || len_size < 1 ||
        len_size > 8)
      return fail(HTR_ERR_FORMAT, "bad fractal heap parameters");
    if (rows != 0) return fail(HTR_ERR_UNSUPPORTED, "fractal heap grown past its root direct block");
    // the name index: header, then its root leaf
    const size_t bsize = 4 + 1 + 1 + 4 + 2 + 2 + 1 + 1 + size_t(so) + 2 + size_t(sl) + 4;
    std::vector<uint8_t> bh;
    if (!checked(bt2, bsize, "BTHD", bh)) return false;
    Cur b(bh.data() + 4, bsize - 4);
    b.u8();
    const uint8_t type = b.u8();
    b.u32();  // node size
    const uint16_t rec = b.u16(), depth = b.u16();
    b.u8();
    b.u8();
    const uint64_t leaf = b.addr(so);
    const uint16_t nrec = b.u16();
    if (type != want || rec != id_len + (want == 5 ? 4 : 9))
      return fail(HTR_ERR_FORMAT, std::string(what) + " name index of another record type");
    if (depth != 0) return fail(HTR_ERR_UNSUPPORTED, std::string(what) + " name index deeper than one leaf");
    if (nrec == 0) return true;
    std::vector<uint8_t> lf;
    if (!checked(leaf, 6 + size_t(nrec) * rec + 4, "BTLF", lf)) return false;
    for (unsigned r = 0; r < nrec; r++) {
      Cur e(lf.data() + 6 + size_t(r) * rec, rec);
      if (want == 5) e.u32();  // name hash first in a link record
      const uint8_t idb = e.u8();
      if (((idb >> 4) & 0x03) != 0)
        return fail(HTR_ERR_UNSUPPORTED, std::string(what) + " stored as a huge or tiny heap object");
      const uint64_t off = e.uint(off_size), len = e.uint(len_size);
      // an object's offset counts from the start of the root direct block
      if (len == 0 || off >= start_block || len > start_block - off) return fail(HTR_ERR_FORMAT, "bad heap ID");
      objects.emplace_back();
      if (!block(root + off, len, objects.back())) return false;
    }
    return true;
  }

  bool dense_links(uint64_t fheap, uint64_t bt2, std::vector<std::pair<std::string, uint64_t>> &links) {
    std::vector<std::vector<uint8_t>> objs;
    if (!dense_objects(fheap, bt2, 5, objs)) return false;
    for (auto &o : objs)
      if (!link_message(Msg{0x0006, 0, std::move(o)}, links)) return false;
    return true;
  }

  // attributes named by an attribute info message (dense storage), if any
  bool dense_attributes(const Msg &info, std::vector<std::pair<std::string, Value>> &out) {
    Cur c(info.data);
    if (c.u8() != 0) return fail(HTR_ERR_UNSUPPORTED, "attribute info message version");
    const uint8_t flags = c.u8();
    if (flags & 0x01) c.skip(2);
    const uint64_t fheap = c.addr(so), names = c.addr(so);
    if (c.bad) return fail(HTR_ERR_FORMAT, "bad attribute info message");
    if (fheap == kUndef) return true;
    std::vector<std::vector<uint8_t>> objs;
    if (!dense_objects(fheap, names, 8, objs)) return false;
    for (auto &o : objs) {
      std::string name;
      Value v;
      if (!attribute(Msg{0x000c, 0, std::move(o)}, name, v)) return false;
      out.emplace_back(name, std::move(v));
    }
    return true;
  }

  bool link_message(const Msg &m, std::vector<std::pair<std::string, uint64_t>> &links) {
    Cur c(m.data);
    if (c.u8() != 1) return fail(HTR_ERR_UNSUPPORTED, "link message version");
    const uint8_t flags = c.u8();
    int type = 0;
    if (flags & 0x08) type = c.u8();
    if (flags & 0x04) c.skip(8);
    if (flags & 0x10) c.u8();
    const uint64_t len = c.uint(1 << (flags & 0x03));
    if (!c.need(len)) return fail(HTR_ERR_FORMAT, "truncated link message");
    std::string name(reinterpret_cast<const char *>(c.p + c.i), len);
    c.skip(len);
    if (type != 0) return true;  // soft or external link
    const uint64_t oh = c.addr(so);
    if (c.bad) return fail(HTR_ERR_FORMAT, "truncated link message");
    links.emplace_back(name, oh);
    return true;
  }

  bool group(uint64_t rel, const std::string &prefix, bool root) {
    if (!visited.insert(rel).second) return true;
    if (visited.size() > 100000) return fail(HTR_ERR_FORMAT, "too many objects");
    std::vector<Msg> msgs;
    if (!object(rel, msgs)) return false;
    std::vector<std::pair<std::string, uint64_t>> links;
    for (const auto &m : msgs) {
      if (m.type == 0x0011) {
        Cur c(m.data);
        const uint64_t bt = c.addr(so), hp = c.addr(so);
        if (c.bad) return fail(HTR_ERR_FORMAT, "bad symbol table message");
        std::vector<uint8_t> heap;
        if (!local_heap(hp, heap) || !btree(bt, heap, links, 0)) return false;
      } else if (m.type == 0x0006) {
        if (!link_message(m, links)) return false;
      } else if (m.type == 0x0002) {
        Cur c(m.data);
        c.u8();
        const uint8_t flags = c.u8();
        if (flags & 0x01) c.skip(8);
        const uint64_t fheap = c.addr(so);
        const uint64_t names = c.addr(so);
        if (c.bad) return fail(HTR_ERR_FORMAT, "bad link info message");
        if (fheap != kUndef && !dense_links(fheap, names, links)) return false;
      } else if (m.type == 0x0015 && root) {
        if (!dense_attributes(m, r.attrs_)) return false;
      } else if (m.type == 0x000c && root) {
        std::string name;
        Value v;
        if (!attribute(m, name, v)) return false;
        r.attrs_.emplace_back(name, std::move(v));
      }
    }
    for (const auto &l : links) {
      const std::string path = prefix.empty() ? l.first : prefix + "/" + l.first;
      std::vector<Msg> om;
      if (!object(l.second, om)) return false;
      bool is_group = false, is_set = false;
      for (const auto &m : om) {
        is_group = is_group || m.type == 0x0011 || m.type == 0x0006 || m.type == 0x0002;
        is_set = is_set || m.type == 0x0008;
      }
      if (is_set) {
        if (!visited.insert(l.second).second) continue;
        if (!dataset(om, path)) return false;
      } else if (is_group) {
        if (!group(l.second, path, false)) return false;
      }
    }
    return true;
  }

  bool dataset(const std::vector<Msg> &msgs, const std::string &name) {
    Dataset d;
    d.name = name;
    bool have_type = false, have_space = false;
    Space s;
    for (const auto &m : msgs) {
      if ((m.flags & 0x02) && (m.type == 0x0001 || m.type == 0x0003))
        return fail(HTR_ERR_UNSUPPORTED, "dataset '" + name + "': shared datatype or dataspace");
      Cur c(m.data);
      switch (m.type) {
        case 0x0001:
          if (!decode_space(c, sl, s, st)) return false;
          have_space = true;
          break;
        case 0x0003:
          if (!decode_type(c, d.type)) d.type = Type();
          have_type = true;
          break;
        case 0x000b:
          d.filtered = true;
          break;
        case 0x0008: {
          const uint8_t version = c.u8();
          if (version == 1 || version == 2) {
            const uint8_t rank = c.u8();
            d.layout = c.u8();
            c.skip(5);
            if (d.layout != 0) d.address = c.addr(so);
            c.skip(4 * size_t(rank));
            if (d.layout == 0) {
              const uint32_t n = c.u32();
              if (!c.need(n)) return fail(HTR_ERR_FORMAT, "truncated compact data");
              d.compact.assign(c.p + c.i, c.p + c.i + n);
            }
          } else if (version == 3 || version == 4) {
            d.layout = c.u8();
            if (d.layout == 0) {
              const uint16_t n = c.u16();
              if (!c.need(n)) return fail(HTR_ERR_FORMAT, "truncated compact data");
              d.compact.assign(c.p + c.i, c.p + c.i + n);
            } else if (d.layout == 1) {
              d.address = c.addr(so);
              c.uint(sl);
            }
          } else {
            return fail(HTR_ERR_UNSUPPORTED, "data layout message version " + std::to_string(version));
          }
          if (c.bad) return fail(HTR_ERR_FORMAT, "truncated data layout message");
          break;
        }
        case 0x000c: {
          std::string an;
          Value v;
          if (!attribute(m, an, v)) return false;
          d.attrs.emplace_back(an, std::move(v));
          break;
        }
        case 0x0015:
          if (!dense_attributes(m, d.attrs)) return false;
          break;
        default:
          break;
      }
    }
    if (!have_type || !have_space) return fail(HTR_ERR_FORMAT, "dataset '" + name + "' lacks a datatype or dataspace");
    d.dims = s.dims;
    if (s.null) d.dims = {0};
    r.sets_.push_back(std::move(d));
    return true;
  }
};

Reader::~Reader() {
  if (f_) std::fclose(f_);
}

Status Reader::open(const std::string &path) {
  if (f_) {
    std::fclose(f_);
    f_ = nullptr;
  }
  sets_.clear();
  attrs_.clear();
  f_ = std::fopen(path.c_str(), "rb");
  if (f_ == nullptr) return {HTR_ERR_IO, "cannot open " + path};
  if (fseeko(f_, 0, SEEK_END) != 0) return {HTR_ERR_IO, "cannot seek in " + path};
  size_ = static_cast<uint64_t>(ftello(f_));
  Parser p(*this);
  if (!p.superblock()) {
    p.st.msg = path + ": " + p.st.msg;
    return p.st;
  }
  return {};
}

const Dataset *Reader::find(const std::string &name) const {
  for (const auto &d : sets_)
    if (d.name == name) return &d;
  return nullptr;
}

const Value *Reader::attribute(const std::string &name) const {
  for (const auto &a : attrs_)
    if (a.first == name) return &a.second;
  return nullptr;
}

Status Reader::read(const Dataset &d, uint64_t offset, uint64_t bytes, void *dst) const {
  const uint64_t total = mul_checked(d.elements(), d.type.size);
  if (total == kOverflow) return {HTR_ERR_FORMAT, "dataset '" + d.name + "': size overflows"};
  if (offset > total || bytes > total - offset)
    return {HTR_ERR_ARGUMENT, "read beyond dataset '" + d.name + "'"};
  if (d.filtered) return {HTR_ERR_UNSUPPORTED, "dataset '" + d.name + "' is filtered (compressed)"};
  if (d.layout == 0) {
    if (d.compact.size() < total) return {HTR_ERR_FORMAT, "dataset '" + d.name + "': short compact data"};
    std::memcpy(dst, d.compact.data() + offset, bytes);
    return {};
  }
  if (d.layout != 1)
    return {HTR_ERR_UNSUPPORTED, "dataset '" + d.name + "' uses " +
                                     (d.layout == 2 ? "chunked" : d.layout == 3 ? "virtual" : "unknown") + " storage"};
  if (d.address == kUndef) {
    std::memset(dst, 0, bytes);
    return {};
  }
  const uint64_t at = base_ + d.address + offset;
  if (at > size_ || bytes > size_ - at) return {HTR_ERR_FORMAT, "dataset '" + d.name + "': data beyond the end of the file"};
  if (fseeko(f_, static_cast<off_t>(at), SEEK_SET) != 0 || std::fread(dst, 1, bytes, f_) != bytes)
    return {HTR_ERR_IO, "read error in dataset '" + d.name + "'"};
  return {};
}

bool Reader::as_int64(const Value &v, uint64_t index, int64_t *out) {
  if (v.type.cls != Type::kFixed || v.type.big_endian || v.type.size > 8 || index >= v.elements()) return false;
  if (!element_inside(index, v.type.size, v.data.size())) return false;
  const uint8_t *p = v.data.data() + index * v.type.size;
  uint64_t u = 0;
  for (uint32_t k = 0; k < v.type.size; k++) u |= uint64_t(p[k]) << (8 * k);
  if (v.type.is_signed && v.type.size < 8 && (u >> (8 * v.type.size - 1)) & 1) u |= ~uint64_t(0) << (8 * v.type.size);
  *out = static_cast<int64_t>(u);
  return true;
}

bool Reader::as_double(const Value &v, uint64_t index, double *out) {
  if (v.type.cls != Type::kFloat || !v.type.ieee64 || v.type.big_endian || index >= v.elements()) return false;
  if (!element_inside(index, 8, v.data.size())) return false;
  std::memcpy(out, v.data.data() + index * 8, 8);
  return true;
}

bool Reader::as_string(const Value &v, uint64_t index, std::string *out) {
  if (v.type.cls != Type::kString || index >= v.elements()) return false;
  if (!element_inside(index, v.type.size, v.data.size())) return false;
  const char *p = reinterpret_cast<const char *>(v.data.data() + index * v.type.size);
  size_t n = 0;
  while (n < v.type.size && p[n] != 0) n++;
  out->assign(p, n);
  if (v.type.pad == 2)
    while (!out->empty() && out->back() == ' ') out->pop_back();
  return true;
}

bool Reader::as_point3(const Value &v, uint64_t index, const char *member, int64_t out[3]) {
  if (v.type.cls != Type::kCompound || index >= v.elements()) return false;
  if (!element_inside(index, v.type.size, v.data.size())) return false;
  const Type *t = &v.type;
  uint64_t at = index * v.type.size;
  if (member != nullptr) {
    const Type::Member *m = t->member(member);
    if (m == nullptr) return false;
    at += m->offset;
    t = m->type.get();
    if (t->cls != Type::kCompound) return false;
  }
  const char *names[3] = {"x", "y", "z"};
  for (int k = 0; k < 3; k++) {
    const Type::Member *m = t->member(names[k]);
    if (m == nullptr || m->type->cls != Type::kFixed) return false;
    Value one;
    one.type = *m->type;
    if (at + m->offset + one.type.size > v.data.size()) return false;
    one.data.assign(v.data.begin() + at + m->offset, v.data.begin() + at + m->offset + one.type.size);
    if (!as_int64(one, 0, &out[k])) return false;
  }
  return true;
}

}  // namespace h5
}  // namespace htr
