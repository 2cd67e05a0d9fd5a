// A self-contained reader and writer for the subset of the HDF5 file format
// that HTR's restart files use (no HDF5 library is linked).
//
// The reference writes its restart with libhdf5 under default property
// lists: `create` (src/Utils/hdf_helper.rg:199-331) makes one file per
// tile with one contiguous dataset per field, `dumpMasterFile`
// (src/Utils/hdf_helper.rg:845-931) a master file with scalar attributes
// and a `partitions` dataset.  libhdf5's default ("earliest") format for
// that content is what this file implements, after the published HDF5
// File Format Specification (version 3.0):
//
//   - superblock version 0 (a user block before it is allowed);
//   - version-1 object headers with continuation blocks;
//   - when reading, also the newer format's superblock versions 1-3,
//     version-2 object headers ("OHDR"/"OCHK", lookup3 checksums verified)
//     and dense storage of links and attributes (objects of a one-block
//     fractal heap, indexed by a one-leaf version-2 B-tree);
//   - groups stored as a symbol table: a version-1 B-tree of group nodes
//     (type 0), symbol table nodes and a local heap of link names; groups
//     made of link messages are read as well;
//   - datatypes: fixed-point, IEEE floating point, fixed-length strings,
//     compounds (versions 1-3) and arrays (versions 2-3);
//   - dataspaces versions 1-2; data layout versions 1-4, contiguous or
//     compact storage; attribute messages versions 1-3.
//
// The writer makes only the earliest format.  What the reader meets outside
// the subset (chunked, filtered or virtual storage, larger fractal heaps or
// B-trees, variable-length types) is reported as unsupported, never guessed
// at.
#pragma once

#include <cstdint>
#include <cstdio>
#include <functional>
#include <memory>
#include <string>
#include <utility>
#include <vector>

namespace htr {
namespace h5 {

constexpr uint64_t kUndef = ~0ull;

// Outcome of a file operation.  `code` is 0 or one of the htr_status codes
// HTR_ERR_IO, HTR_ERR_FORMAT, HTR_ERR_UNSUPPORTED, HTR_ERR_ARGUMENT.
struct Status {
  int code = 0;
  std::string msg;
  bool ok() const { return code == 0; }
};

struct Type {
  enum Class : int { kFixed = 0, kFloat = 1, kString = 3, kCompound = 6, kArray = 10, kOther = -1 };
  int cls = kOther;
  int raw_class = -1;       // class number as stored (for messages about kOther)
  uint32_t size = 0;        // bytes per element
  bool is_signed = false;   // fixed-point
  bool big_endian = false;  // fixed-point and floating point
  int pad = 0;              // string padding: 0 null-terminated, 1 null-padded, 2 space-padded
  bool ieee64 = false;      // floating point with the IEEE binary64 field layout
  struct Member {
    std::string name;
    uint32_t offset;
    std::shared_ptr<Type> type;
  };
  std::vector<Member> members;  // compound
  std::vector<uint32_t> dims;   // array
  std::shared_ptr<Type> base;   // array

  static Type f64();
  static Type integer(uint32_t bytes, bool is_signed);
  static Type string(uint32_t bytes);
  static Type array(const Type &base, std::vector<uint32_t> dims);
  static Type compound(uint32_t size, std::vector<Member> members);

  // little-endian IEEE binary64, or an array of them; `count` receives the
  // number of doubles per element
  bool is_f64_elements(uint64_t *count) const;
  const Member *member(const std::string &name) const;
};

// An attribute (or a small dataset read whole): type, shape, raw bytes.
struct Value {
  Type type;
  std::vector<uint64_t> dims;  // empty for a scalar
  std::vector<uint8_t> data;
  uint64_t elements() const;
};

struct Dataset {
  std::string name;  // path below the root group, '/'-separated
  Type type;
  std::vector<uint64_t> dims;
  int layout = -1;            // 0 compact, 1 contiguous, 2 chunked, 3 virtual
  bool filtered = false;
  uint64_t address = kUndef;  // absolute file offset of contiguous data
  std::vector<uint8_t> compact;
  std::vector<std::pair<std::string, Value>> attrs;
  uint64_t elements() const;
};

// Writes one file: root attributes and datasets directly below the root.
// Metadata comes first, the datasets' contiguous data after it.
class Writer {
 public:
  void attribute(const std::string &name, Value v);
  // `emit` writes exactly elements(dims) * type.size bytes in storage
  // order (row-major over dims, the element's bytes innermost) and returns
  // false on failure.  `max_dims` also stores the maximum dimensions (equal
  // to the current ones), as H5Screate_simple(rank, dims, dims) does.
  void dataset(const std::string &name, const Type &type, std::vector<uint64_t> dims,
               std::function<bool(FILE *)> emit, bool max_dims = false);
  Status write(const std::string &path) const;

 private:
  struct Out {
    std::string name;
    Type type;
    std::vector<uint64_t> dims;
    bool max_dims;
    std::function<bool(FILE *)> emit;
  };
  std::vector<std::pair<std::string, Value>> attrs_;
  std::vector<Out> sets_;
};

class Reader {
 public:
  Reader() = default;
  Reader(const Reader &) = delete;
  Reader &operator=(const Reader &) = delete;
  ~Reader();

  Status open(const std::string &path);
  const std::vector<Dataset> &datasets() const { return sets_; }
  const std::vector<std::pair<std::string, Value>> &attributes() const { return attrs_; }
  const Dataset *find(const std::string &name) const;
  const Value *attribute(const std::string &name) const;
  // copies `bytes` bytes of the dataset's storage, starting `offset` bytes
  // into it, to `dst`; never-written contiguous storage reads as zeros
  Status read(const Dataset &d, uint64_t offset, uint64_t bytes, void *dst) const;

  // decoding helpers over Values (false if the type does not convert)
  static bool as_int64(const Value &v, uint64_t index, int64_t *out);
  static bool as_double(const Value &v, uint64_t index, double *out);
  static bool as_string(const Value &v, uint64_t index, std::string *out);
  // an int3d-like compound {x, y, z} (or a member path "lo"/"hi" of a
  // rect3d-like compound when `member` is given)
  static bool as_point3(const Value &v, uint64_t index, const char *member, int64_t out[3]);

 private:
  FILE *f_ = nullptr;
  uint64_t size_ = 0;
  uint64_t base_ = 0;
  std::vector<Dataset> sets_;
  std::vector<std::pair<std::string, Value>> attrs_;
  friend struct Parser;
};

}  // namespace h5
}  // namespace htr
