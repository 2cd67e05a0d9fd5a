// Restart files (include/htr_restart.h): the tile and master files of the
// reference's HDF5 restart layout, written and read through h5file.h.
//
// Device fields move through two pinned host buffers and two device slabs:
// a kernel gathers one slab of z-planes of a field from its strided layout
// into file order (z, y, x, component), an asynchronous copy brings it to
// the host, and while the file takes one slab the next one is gathered and
// copied (loading runs the same pipeline backwards).
#include <cuda_runtime.h>

#include <algorithm>
#include <cinttypes>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "h5file.h"
#include "htr_restart.h"

namespace htr {
int set_last_error(int code, const std::string &msg);
}

namespace {

using htr::h5::Reader;
using htr::h5::Status;
using htr::h5::Type;
using htr::h5::Value;

// field data go to and from the files as the host holds them: the files
// store little-endian doubles and int64 rectangles
static_assert(__BYTE_ORDER__ == __ORDER_LITTLE_ENDIAN__, "restart files need a little-endian host");

constexpr size_t kSlabBytes = size_t(64) << 20;
constexpr int kThreads = 256;

int fail(int code, const std::string &msg) { return htr::set_last_error(code, msg); }
int fail(const Status &s) { return htr::set_last_error(s.code, s.msg); }
int cuda_fail(cudaError_t e, const char *where) {
  return htr::set_last_error(HTR_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

// One slab: planes [z0, z0 + nz) of the tile, all x and y, all components.
__global__ void gather_slab(const char *base, int64_t sx, int64_t sy, int64_t sz, int64_t x0, int64_t y0,
                            int64_t z0, int64_t nx, int64_t ny, int comps, int64_t n, double *out) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t c = i % comps, p = i / comps;
    const int64_t x = p % nx, q = p / nx;
    const int64_t y = q % ny, z = q / ny;
    out[i] = *reinterpret_cast<const double *>(base + (x0 + x) * sx + (y0 + y) * sy + (z0 + z) * sz + c * 8);
  }
}

__global__ void scatter_slab(char *base, int64_t sx, int64_t sy, int64_t sz, int64_t x0, int64_t y0, int64_t z0,
                             int64_t nx, int64_t ny, int comps, int64_t n, const double *in) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t c = i % comps, p = i / comps;
    const int64_t x = p % nx, q = p / nx;
    const int64_t y = q % ny, z = q / ny;
    *reinterpret_cast<double *>(base + (x0 + x) * sx + (y0 + y) * sy + (z0 + z) * sz + c * 8) = in[i];
  }
}

struct FieldSpec {
  const char *name;
  htr_field htr_fluid_view::*member;
  int comps;  // 0: nSpec
};

// IOVars (src/prometeo.rg:145-153) and the inflow profile fields
const FieldSpec kIOFields[] = {
    {"rho", &htr_fluid_view::rho, 1},
    {"pressure", &htr_fluid_view::pressure, 1},
    {"temperature", &htr_fluid_view::temperature, 1},
    {"MolarFracs", &htr_fluid_view::MolarFracs, 0},
    {"velocity", &htr_fluid_view::velocity, 3},
    {"dudtBoundary", &htr_fluid_view::dudtBoundary, 3},
    {"dTdtBoundary", &htr_fluid_view::dTdtBoundary, 1},
};
const FieldSpec kProfileFields[] = {
    {"MolarFracs_profile", &htr_fluid_view::MolarFracs_profile, 0},
    {"velocity_profile", &htr_fluid_view::velocity_profile, 3},
    {"temperature_profile", &htr_fluid_view::temperature_profile, 1},
};

struct Field {
  const char *name;
  htr_field f;
  int comps;
};

struct Slab {
  size_t field;
  int64_t z0, nz;
  uint64_t bytes, offset;  // bytes, and offset within the dataset
};

struct Tile {
  htr_rect3 r;
  int64_t nx, ny, nz;
};

int collect(const htr_fluid_view *view, int nSpec, int flags, std::vector<Field> &out) {
  auto add = [&](const FieldSpec &s) -> int {
    const htr_field f = view->*(s.member);
    if (f.base == nullptr) return fail(HTR_ERR_ARGUMENT, std::string("restart field ") + s.name + " is null");
    if (reinterpret_cast<uintptr_t>(f.base) % 8 != 0)
      return fail(HTR_ERR_LAYOUT, std::string("restart field ") + s.name + ": misaligned base");
    for (int i = 0; i < 3; i++)
      if (f.stride[i] % 8 != 0)
        return fail(HTR_ERR_LAYOUT, std::string("restart field ") + s.name + ": stride not a multiple of 8 bytes");
    out.push_back({s.name, f, s.comps ? s.comps : nSpec});
    return HTR_OK;
  };
  for (const auto &s : kIOFields)
    if (int st = add(s)) return st;
  if (flags & HTR_RESTART_PROFILES)
    for (const auto &s : kProfileFields)
      if (int st = add(s)) return st;
  return HTR_OK;
}

std::vector<Slab> slabs_of(const std::vector<Field> &fields, const Tile &t, size_t *cap) {
  std::vector<Slab> out;
  *cap = 0;
  for (size_t k = 0; k < fields.size(); k++) {
    const uint64_t plane = uint64_t(t.nx) * t.ny * fields[k].comps * 8;
    const int64_t per = std::max<int64_t>(1, std::min<int64_t>(t.nz, int64_t(kSlabBytes / plane)));
    for (int64_t z0 = 0; z0 < t.nz; z0 += per) {
      const int64_t nz = std::min(per, t.nz - z0);
      out.push_back({k, z0, nz, plane * nz, plane * z0});
      *cap = std::max<size_t>(*cap, plane * nz);
    }
  }
  return out;
}

// Two pinned host buffers, two device slabs and their events.
struct Staging {
  bool device = false;
  cudaStream_t stream = nullptr;
  size_t cap = 0;
  void *host[2] = {nullptr, nullptr};
  double *dev[2] = {nullptr, nullptr};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  std::vector<char> plain[2];
  int blocks = 0;

  int init(bool on_device, cudaStream_t s, size_t bytes) {
    device = on_device;
    stream = s;
    cap = bytes;
    if (!device) {
      plain[0].resize(cap);
      plain[1].resize(cap);
      host[0] = plain[0].data();
      host[1] = plain[1].data();
      return HTR_OK;
    }
    int dev_id = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev_id);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev_id);
    if (e != cudaSuccess) return cuda_fail(e, "restart staging");
    blocks = std::max(1, sms) * 8;
    for (int b = 0; b < 2; b++) {
      if ((e = cudaMallocHost(&host[b], cap)) != cudaSuccess) return cuda_fail(e, "cudaMallocHost");
      if ((e = cudaMalloc(&dev[b], cap)) != cudaSuccess) return cuda_fail(e, "cudaMalloc");
      if ((e = cudaEventCreateWithFlags(&ev[b], cudaEventDisableTiming)) != cudaSuccess)
        return cuda_fail(e, "cudaEventCreate");
    }
    return HTR_OK;
  }
  int grid(int64_t n) const { return int(std::min<int64_t>(blocks, (n + kThreads - 1) / kThreads)); }
  ~Staging() {
    if (!device) return;
    cudaStreamSynchronize(stream);
    for (int b = 0; b < 2; b++) {
      if (host[b]) cudaFreeHost(host[b]);
      if (dev[b]) cudaFree(dev[b]);
      if (ev[b]) cudaEventDestroy(ev[b]);
    }
  }
};

void host_gather(const Field &f, const Tile &t, const Slab &s, char *out) {
  const char *base = static_cast<const char *>(f.f.base);
  const size_t elem = size_t(f.comps) * 8;
  for (int64_t z = 0; z < s.nz; z++)
    for (int64_t y = 0; y < t.ny; y++)
      for (int64_t x = 0; x < t.nx; x++) {
        std::memcpy(out, base + (t.r.lo[0] + x) * f.f.stride[0] + (t.r.lo[1] + y) * f.f.stride[1] +
                             (t.r.lo[2] + s.z0 + z) * f.f.stride[2], elem);
        out += elem;
      }
}

void host_scatter(const Field &f, const Tile &t, const Slab &s, const char *in) {
  char *base = static_cast<char *>(f.f.base);
  const size_t elem = size_t(f.comps) * 8;
  for (int64_t z = 0; z < s.nz; z++)
    for (int64_t y = 0; y < t.ny; y++)
      for (int64_t x = 0; x < t.nx; x++) {
        std::memcpy(base + (t.r.lo[0] + x) * f.f.stride[0] + (t.r.lo[1] + y) * f.f.stride[1] +
                        (t.r.lo[2] + s.z0 + z) * f.f.stride[2], in, elem);
        in += elem;
      }
}

bool rect_ok(const htr_rect3 &r) {
  for (int i = 0; i < 3; i++)
    if (r.lo[i] > r.hi[i]) return false;
  return true;
}

int tile_of(const htr_rect3 &r, Tile &t) {
  if (!rect_ok(r)) return fail(HTR_ERR_ARGUMENT, "inverted tile rectangle");
  t = {r, r.hi[0] - r.lo[0] + 1, r.hi[1] - r.lo[1] + 1, r.hi[2] - r.lo[2] + 1};
  return HTR_OK;
}

std::string tile_path(const char *dirname, const htr_rect3 &r) {
  char buf[512];
  std::snprintf(buf, sizeof(buf), "%s/%" PRId64 ",%" PRId64 ",%" PRId64 "-%" PRId64 ",%" PRId64 ",%" PRId64 ".hdf",
                dirname, r.lo[0], r.lo[1], r.lo[2], r.hi[0], r.hi[1], r.hi[2]);
  return buf;
}

Type field_type(int comps) {
  return comps == 1 ? Type::f64() : Type::array(Type::f64(), {uint32_t(comps)});
}

Type point3_type() {
  const Type i64 = Type::integer(8, true);
  return Type::compound(24, {{"x", 0, std::make_shared<Type>(i64)},
                             {"y", 8, std::make_shared<Type>(i64)},
                             {"z", 16, std::make_shared<Type>(i64)}});
}

Type rect3_type() {
  const Type p = point3_type();
  return Type::compound(48, {{"lo", 0, std::make_shared<Type>(p)}, {"hi", 24, std::make_shared<Type>(p)}});
}

void put_i64(std::vector<uint8_t> &b, int64_t v) {
  for (int k = 0; k < 8; k++) b.push_back(static_cast<uint8_t>(uint64_t(v) >> (8 * k)));
}

Value scalar(const Type &t, std::vector<uint8_t> bytes) {
  Value v;
  v.type = t;
  v.data = std::move(bytes);
  return v;
}

Value strings(const char *const *s, int n, uint32_t width) {
  Value v;
  v.type = Type::string(width);
  v.dims = {uint64_t(n)};
  v.data.assign(size_t(n) * width, 0);
  for (int i = 0; i < n; i++) {
    const size_t len = std::min<size_t>(std::strlen(s[i]), width - 1);
    std::memcpy(v.data.data() + size_t(i) * width, s[i], len);
  }
  return v;
}

}  // namespace

extern "C" {

int htr_restart_tile_filename(const char *dirname, htr_rect3 tile, char *out, size_t capacity) {
  if (dirname == nullptr || out == nullptr) return fail(HTR_ERR_ARGUMENT, "null argument");
  const std::string p = tile_path(dirname, tile);
  if (p.size() + 1 > capacity) return fail(HTR_ERR_ARGUMENT, "file name buffer too small");
  std::memcpy(out, p.c_str(), p.size() + 1);
  return HTR_OK;
}

int htr_restart_write_tile(const char *dirname, const htr_fluid_view *view, htr_rect3 tile, int nSpec, int flags,
                           htr_stream_t stream) {
  if (dirname == nullptr || view == nullptr) return fail(HTR_ERR_ARGUMENT, "null argument");
  if (nSpec < 1 || nSpec > 1024) return fail(HTR_ERR_ARGUMENT, "nSpec out of range");
  Tile t;
  if (int st = tile_of(tile, t)) return st;
  std::vector<Field> fields;
  if (int st = collect(view, nSpec, flags, fields)) return st;
  size_t cap = 0;
  const std::vector<Slab> slabs = slabs_of(fields, t, &cap);
  const bool on_device = !(flags & HTR_RESTART_HOST_VIEW);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  Staging stage;
  if (int st = stage.init(on_device, s, cap)) return st;

  cudaError_t cerr = cudaSuccess;
  auto enqueue = [&](size_t j) {
    if (j >= slabs.size() || !on_device || cerr != cudaSuccess) return;
    const Slab &sl = slabs[j];
    const Field &f = fields[sl.field];
    const int b = int(j % 2);
    const int64_t n = int64_t(sl.bytes / 8);
    gather_slab<<<stage.grid(n), kThreads, 0, s>>>(static_cast<const char *>(f.f.base), f.f.stride[0], f.f.stride[1],
                                                   f.f.stride[2], t.r.lo[0], t.r.lo[1], t.r.lo[2] + sl.z0, t.nx, t.ny,
                                                   f.comps, n, stage.dev[b]);
    cerr = cudaGetLastError();
    if (cerr == cudaSuccess) cerr = cudaMemcpyAsync(stage.host[b], stage.dev[b], sl.bytes, cudaMemcpyDeviceToHost, s);
    if (cerr == cudaSuccess) cerr = cudaEventRecord(stage.ev[b], s);
  };
  enqueue(0);
  enqueue(1);
  size_t j = 0;
  htr::h5::Writer w;
  for (size_t k = 0; k < fields.size(); k++) {
    w.dataset(fields[k].name, field_type(fields[k].comps), {uint64_t(t.nz), uint64_t(t.ny), uint64_t(t.nx)},
              [&, k](FILE *fp) {
                for (; j < slabs.size() && slabs[j].field == k; j++) {
                  const int b = int(j % 2);
                  if (on_device) {
                    if (cerr == cudaSuccess) cerr = cudaEventSynchronize(stage.ev[b]);
                    if (cerr != cudaSuccess) return false;
                  } else {
                    host_gather(fields[k], t, slabs[j], static_cast<char *>(stage.host[b]));
                  }
                  if (std::fwrite(stage.host[b], 1, slabs[j].bytes, fp) != slabs[j].bytes) return false;
                  enqueue(j + 2);
                }
                return true;
              });
  }
  const Status st = w.write(tile_path(dirname, tile));
  if (cerr != cudaSuccess) return cuda_fail(cerr, "restart tile gather");
  if (!st.ok()) return fail(st);
  return HTR_OK;
}

int htr_restart_read_tile(const char *dirname, const htr_fluid_view *view, htr_rect3 tile, int nSpec, int flags,
                          htr_stream_t stream) {
  if (dirname == nullptr || view == nullptr) return fail(HTR_ERR_ARGUMENT, "null argument");
  if (nSpec < 1 || nSpec > 1024) return fail(HTR_ERR_ARGUMENT, "nSpec out of range");
  Tile t;
  if (int st = tile_of(tile, t)) return st;
  std::vector<Field> fields;
  if (int st = collect(view, nSpec, flags, fields)) return st;
  const std::string path = tile_path(dirname, tile);
  Reader r;
  Status st = r.open(path);
  if (!st.ok()) return fail(st);
  std::vector<const htr::h5::Dataset *> sets;
  for (const auto &f : fields) {
    const htr::h5::Dataset *d = r.find(f.name);
    if (d == nullptr) return fail(HTR_ERR_FORMAT, path + ": no dataset '" + f.name + "'");
    uint64_t comps = 0;
    if (!d->type.is_f64_elements(&comps) || comps != uint64_t(f.comps))
      return fail(HTR_ERR_FORMAT, path + ": dataset '" + f.name + "' is not " + std::to_string(f.comps) +
                                      " little-endian double(s) per point");
    if (d->dims != std::vector<uint64_t>{uint64_t(t.nz), uint64_t(t.ny), uint64_t(t.nx)})
      return fail(HTR_ERR_FORMAT, path + ": dataset '" + f.name + "' does not have the tile's shape");
    sets.push_back(d);
  }
  size_t cap = 0;
  const std::vector<Slab> slabs = slabs_of(fields, t, &cap);
  const bool on_device = !(flags & HTR_RESTART_HOST_VIEW);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  Staging stage;
  if (int e = stage.init(on_device, s, cap)) return e;
  for (size_t j = 0; j < slabs.size(); j++) {
    const Slab &sl = slabs[j];
    const Field &f = fields[sl.field];
    const int b = int(j % 2);
    if (on_device) {
      // the copy out of this buffer two slabs ago must be done
      cudaError_t e = cudaEventSynchronize(stage.ev[b]);
      if (e != cudaSuccess) return cuda_fail(e, "restart tile scatter");
    }
    st = r.read(*sets[sl.field], sl.offset, sl.bytes, stage.host[b]);
    if (!st.ok()) return fail(st);
    if (!on_device) {
      host_scatter(f, t, sl, static_cast<const char *>(stage.host[b]));
      continue;
    }
    cudaError_t e = cudaMemcpyAsync(stage.dev[b], stage.host[b], sl.bytes, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync");
    const int64_t n = int64_t(sl.bytes / 8);
    scatter_slab<<<stage.grid(n), kThreads, 0, s>>>(static_cast<char *>(f.f.base), f.f.stride[0], f.f.stride[1],
                                                    f.f.stride[2], t.r.lo[0], t.r.lo[1], t.r.lo[2] + sl.z0, t.nx,
                                                    t.ny, f.comps, n, stage.dev[b]);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "scatter_slab");
    if ((e = cudaEventRecord(stage.ev[b], s)) != cudaSuccess) return cuda_fail(e, "cudaEventRecord");
  }
  if (on_device) {
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "restart tile load");
  }
  return HTR_OK;
}

int htr_restart_write_master(const char *dirname, const htr_restart_info *info, htr_rect3 bounds,
                             const int64_t tiles[3], const htr_rect3 *partitions, int nSpec,
                             const char *const *species_names, const char *const *versions) {
  if (dirname == nullptr || info == nullptr || tiles == nullptr || partitions == nullptr)
    return fail(HTR_ERR_ARGUMENT, "null argument");
  if (!rect_ok(bounds)) return fail(HTR_ERR_ARGUMENT, "inverted base index space");
  for (int i = 0; i < 3; i++)
    if (tiles[i] < 1) return fail(HTR_ERR_ARGUMENT, "tile counts must be positive");
  if (info->timeStep < INT32_MIN || info->timeStep > INT32_MAX)
    return fail(HTR_ERR_ARGUMENT, "timeStep does not fit the 32-bit attribute");
  if (species_names != nullptr && (nSpec < 1 || nSpec > 1024)) return fail(HTR_ERR_ARGUMENT, "nSpec out of range");
  const uint64_t ntiles = uint64_t(tiles[0]) * tiles[1] * tiles[2];
  for (uint64_t k = 0; k < ntiles; k++) {
    if (!rect_ok(partitions[k])) return fail(HTR_ERR_ARGUMENT, "inverted partition rectangle");
    for (int i = 0; i < 3; i++)
      if (partitions[k].lo[i] < bounds.lo[i] || partitions[k].hi[i] > bounds.hi[i])
        return fail(HTR_ERR_ARGUMENT, "a partition lies outside the base index space");
  }

  htr::h5::Writer w;
  {
    Value v;
    v.type = Type::string(8);  // IO_VERSION, as the reference stores it
    v.data.assign(8, 0);
    std::memcpy(v.data.data(), "1.0.0", 5);
    w.attribute("IO_VERSION", v);
  }
  {
    std::vector<uint8_t> b;
    for (int i = 0; i < 3; i++) put_i64(b, bounds.lo[i]);
    for (int i = 0; i < 3; i++) put_i64(b, bounds.hi[i]);
    w.attribute("baseIndexSpace", scalar(rect3_type(), b));
  }
  {
    std::vector<uint8_t> b;
    for (int i = 0; i < 3; i++) put_i64(b, tiles[i]);
    w.attribute("tilesNumber", scalar(point3_type(), b));
  }
  {
    std::vector<uint8_t> b;
    const uint32_t ts = static_cast<uint32_t>(static_cast<int32_t>(info->timeStep));
    for (int k = 0; k < 4; k++) b.push_back(static_cast<uint8_t>(ts >> (8 * k)));
    w.attribute("timeStep", scalar(Type::integer(4, true), b));
  }
  auto f64 = [](double d) {
    std::vector<uint8_t> b(8);
    std::memcpy(b.data(), &d, 8);
    return b;
  };
  w.attribute("simTime", scalar(Type::f64(), f64(info->simTime)));
  if (species_names != nullptr) w.attribute("SpeciesNames", strings(species_names, nSpec, 21));
  if (versions != nullptr) {
    const size_t len = std::max(std::strlen(versions[0]), std::strlen(versions[1]));
    w.attribute("Versions", strings(versions, 2, uint32_t(len + 1)));
  }
  w.attribute("channelForcing", scalar(Type::f64(), f64(info->channelForcing)));
  std::vector<uint8_t> parts;
  for (uint64_t k = 0; k < ntiles; k++) {
    for (int i = 0; i < 3; i++) put_i64(parts, partitions[k].lo[i]);
    for (int i = 0; i < 3; i++) put_i64(parts, partitions[k].hi[i]);
  }
  w.dataset("partitions", rect3_type(), {uint64_t(tiles[2]), uint64_t(tiles[1]), uint64_t(tiles[0])},
            [&](FILE *fp) { return std::fwrite(parts.data(), 1, parts.size(), fp) == parts.size(); }, true);
  const Status st = w.write(std::string(dirname) + "/master.hdf");
  return st.ok() ? HTR_OK : fail(st);
}

int htr_restart_read_master(const char *dirname, htr_restart_info *info, htr_rect3 *bounds, int64_t tiles[3],
                            htr_rect3 *partitions, int64_t capacity) {
  if (dirname == nullptr || info == nullptr || bounds == nullptr || tiles == nullptr)
    return fail(HTR_ERR_ARGUMENT, "null argument");
  const std::string path = std::string(dirname) + "/master.hdf";
  Reader r;
  Status st = r.open(path);
  if (!st.ok()) return fail(st);
  const Value *ts = r.attribute("timeStep");
  const Value *tm = r.attribute("simTime");
  const Value *cf = r.attribute("channelForcing");
  const Value *bi = r.attribute("baseIndexSpace");
  const Value *tn = r.attribute("tilesNumber");
  if (!ts || !Reader::as_int64(*ts, 0, &info->timeStep)) return fail(HTR_ERR_FORMAT, path + ": no integer timeStep");
  if (!tm || !Reader::as_double(*tm, 0, &info->simTime)) return fail(HTR_ERR_FORMAT, path + ": no double simTime");
  info->channelForcing = 0.0;
  if (cf && !Reader::as_double(*cf, 0, &info->channelForcing))
    return fail(HTR_ERR_FORMAT, path + ": channelForcing is not a double");
  if (!bi || !Reader::as_point3(*bi, 0, "lo", bounds->lo) || !Reader::as_point3(*bi, 0, "hi", bounds->hi))
    return fail(HTR_ERR_FORMAT, path + ": no baseIndexSpace rectangle");
  for (int i = 0; i < 3; i++)
    if (bounds->lo[i] > bounds->hi[i]) return fail(HTR_ERR_FORMAT, path + ": inverted baseIndexSpace");
  if (!tn || !Reader::as_point3(*tn, 0, nullptr, tiles)) return fail(HTR_ERR_FORMAT, path + ": no tilesNumber");
  for (int i = 0; i < 3; i++)
    if (tiles[i] < 1 || tiles[i] > (int64_t(1) << 20)) return fail(HTR_ERR_FORMAT, path + ": bad tilesNumber");
  const uint64_t ntiles = uint64_t(tiles[0]) * tiles[1] * tiles[2];
  if (partitions == nullptr || capacity < int64_t(ntiles)) return HTR_OK;
  const htr::h5::Dataset *d = r.find("partitions");
  if (d == nullptr) return fail(HTR_ERR_FORMAT, path + ": no partitions dataset");
  if (d->dims != std::vector<uint64_t>{uint64_t(tiles[2]), uint64_t(tiles[1]), uint64_t(tiles[0])})
    return fail(HTR_ERR_FORMAT, path + ": partitions do not match tilesNumber");
  // a rectangle of int64 points is 48 bytes; anything far larger is not one
  if (d->type.cls != Type::kCompound || d->type.size == 0 || d->type.size > 4096)
    return fail(HTR_ERR_FORMAT, path + ": partitions are not rectangles");
  Value v;
  v.type = d->type;
  v.dims = d->dims;
  v.data.resize(ntiles * d->type.size);
  st = r.read(*d, 0, v.data.size(), v.data.data());
  if (!st.ok()) return fail(st);
  for (uint64_t k = 0; k < ntiles; k++) {
    if (!Reader::as_point3(v, k, "lo", partitions[k].lo) || !Reader::as_point3(v, k, "hi", partitions[k].hi))
      return fail(HTR_ERR_FORMAT, path + ": partitions are not rectangles");
    // every tile lies inside baseIndexSpace: a tile file read through a
    // rectangle reaching past the grid would write outside the fields
    for (int i = 0; i < 3; i++)
      if (partitions[k].lo[i] > partitions[k].hi[i] || partitions[k].lo[i] < bounds->lo[i] ||
          partitions[k].hi[i] > bounds->hi[i])
        return fail(HTR_ERR_FORMAT, path + ": partition " + std::to_string(k) + " lies outside baseIndexSpace");
  }
  return HTR_OK;
}

int htr_h5_dataset_shape(const char *path, const char *dataset, int *rank, int64_t dims[8],
                         int64_t *doubles_per_element) {
  if (path == nullptr || dataset == nullptr || rank == nullptr || dims == nullptr)
    return fail(HTR_ERR_ARGUMENT, "null argument");
  Reader r;
  const Status st = r.open(path);
  if (!st.ok()) return fail(st);
  const htr::h5::Dataset *d = r.find(dataset);
  if (d == nullptr) return fail(HTR_ERR_FORMAT, std::string(path) + ": no dataset '" + dataset + "'");
  if (d->dims.size() > 8) return fail(HTR_ERR_UNSUPPORTED, "rank above 8");
  *rank = int(d->dims.size());
  for (size_t i = 0; i < d->dims.size(); i++) dims[i] = int64_t(d->dims[i]);
  if (doubles_per_element != nullptr) {
    uint64_t c = 0;
    *doubles_per_element = d->type.is_f64_elements(&c) ? int64_t(c) : 0;
  }
  return HTR_OK;
}

int htr_h5_read_doubles(const char *path, const char *dataset, double *out, int64_t count) {
  if (path == nullptr || dataset == nullptr || out == nullptr) return fail(HTR_ERR_ARGUMENT, "null argument");
  Reader r;
  Status st = r.open(path);
  if (!st.ok()) return fail(st);
  const htr::h5::Dataset *d = r.find(dataset);
  if (d == nullptr) return fail(HTR_ERR_FORMAT, std::string(path) + ": no dataset '" + dataset + "'");
  uint64_t c = 0;
  if (!d->type.is_f64_elements(&c)) return fail(HTR_ERR_FORMAT, std::string("dataset '") + dataset + "' is not double");
  if (count < 0 || uint64_t(count) != d->elements() * c)
    return fail(HTR_ERR_ARGUMENT, std::string("dataset '") + dataset + "' holds " + std::to_string(d->elements() * c) +
                                      " doubles");
  st = r.read(*d, 0, uint64_t(count) * 8, out);
  return st.ok() ? HTR_OK : fail(st);
}

int htr_h5_string_attribute(const char *path, const char *dataset, const char *name, int64_t index, char *out,
                            size_t capacity) {
  if (path == nullptr || name == nullptr || out == nullptr || capacity == 0)
    return fail(HTR_ERR_ARGUMENT, "null argument");
  Reader r;
  const Status st = r.open(path);
  if (!st.ok()) return fail(st);
  const Value *v = nullptr;
  if (dataset == nullptr) {
    v = r.attribute(name);
  } else if (const htr::h5::Dataset *d = r.find(dataset)) {
    for (const auto &a : d->attrs)
      if (a.first == name) v = &a.second;
  }
  std::string s;
  if (v == nullptr || index < 0 || !Reader::as_string(*v, uint64_t(index), &s))
    return fail(HTR_ERR_FORMAT, std::string("no string attribute '") + name + "'");
  if (s.size() + 1 > capacity) return fail(HTR_ERR_ARGUMENT, "string buffer too small");
  std::memcpy(out, s.c_str(), s.size() + 1);
  return HTR_OK;
}

}  // extern "C"
