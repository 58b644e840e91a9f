// fv3g_restart.cu -- restart files of the tracer path: fv_tracer.res.tile<t>.nc
// (every tracer) and fv_core.res.tile<t>.nc (delp among the dynamics fields),
// as fv3atm reads them at start-up and writes them at restart times
// (atmos_model.F90:105,1149-1166) and as the write component lays them out
// (io/module_write_restart_netcdf.F90:244-317: dimensions xaxis_1, yaxis_1,
// zaxis_1 and the unlimited Time; each field (Time, zaxis_1, yaxis_1,
// xaxis_1) with a 'checksum' attribute written as '(Z16)' of FMS mpp_chksum,
// :444-530).
//
// The container is the netCDF classic family, whose published format is a
// big-endian header (dimensions, attributes, variables with their file
// offsets) followed by the raw values: CDF-1 (classic), CDF-2 (64-bit
// offset) and CDF-5 (64-bit data).  The header is parsed on the host; a
// variable's values travel to the GPU as they lie in the file, and one kernel
// swaps the byte order, converts to the state's precision, scatters the
// values into the halo-padded planes and sums their bit patterns for the
// checksum (integer addition modulo 2^64 is exact in any order).  Writing is
// the mirror image.  netCDF-4 (HDF5) files are recognised and refused.
#include <cuda_runtime.h>
#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "fv3g_internal.cuh"

using namespace fv3g;

#define CHECK(expr)             \
  do {                          \
    int rc__ = (expr);          \
    if (rc__ != 0) return rc__; \
  } while (0)

namespace {

enum { NC_BYTE = 1, NC_CHAR, NC_SHORT, NC_INT, NC_FLOAT, NC_DOUBLE, NC_UBYTE, NC_USHORT, NC_UINT, NC_INT64,
       NC_UINT64 };
enum { TAG_DIMENSION = 10, TAG_VARIABLE = 11, TAG_ATTRIBUTE = 12 };

size_t type_size(int t) {
  switch (t) {
    case NC_BYTE: case NC_CHAR: case NC_UBYTE: return 1;
    case NC_SHORT: case NC_USHORT: return 2;
    case NC_INT: case NC_FLOAT: case NC_UINT: return 4;
    case NC_DOUBLE: case NC_INT64: case NC_UINT64: return 8;
    default: return 0;
  }
}

struct NcAttr {
  std::string name;
  int type = 0;
  long long count = 0;
  std::vector<unsigned char> raw;  // values as stored (big-endian), unpadded
};

struct NcVar {
  std::string name;
  std::vector<long long> dimids;
  std::vector<NcAttr> attrs;
  int type = 0;
  long long begin = 0;
  bool record = false;
  long long values = 1;  // per record (record variables) or in all
};

// ---------------------------------------------------------------- parsing --
struct Cursor {
  const unsigned char* p;
  size_t n, off = 0;
  int version;
  bool short_ = false;  // ran past the bytes read so far
  unsigned long long be(int bytes) {
    if (off + bytes > n) {
      short_ = true;
      off = n;
      return 0;
    }
    unsigned long long v = 0;
    for (int b = 0; b < bytes; ++b) v = (v << 8) | p[off + b];
    off += bytes;
    return v;
  }
  long long nonneg() { return (long long)be(version == 5 ? 8 : 4); }  // counts, lengths, sizes
  long long offset() { return (long long)be(version == 1 ? 4 : 8); }
  void skip_padded(size_t len) {
    size_t pad = (len + 3) & ~(size_t)3;
    if (off + pad > n) {
      short_ = true;
      off = n;
    } else {
      off += pad;
    }
  }
  std::string name() {
    long long len = nonneg();
    if (short_ || len < 0 || (size_t)len > n - off) {
      short_ = true;
      return std::string();
    }
    std::string s((const char*)p + off, (size_t)len);
    skip_padded((size_t)len);
    return s;
  }
};

}  // namespace

struct fv3g_ncfile {
  int fd = -1;
  int version = 0;
  long long numrecs = 0, recsize = 0, file_bytes = 0;
  std::vector<std::string> dim_names;
  std::vector<long long> dim_len;  // 0 = the record dimension
  std::vector<NcAttr> gatts;
  std::vector<NcVar> vars;
  // staging of variable reads: two page-locked host buffers and their device twins
  unsigned char* pin[2] = {nullptr, nullptr};
  unsigned char* dev[2] = {nullptr, nullptr};
  size_t stage = 0;
  cudaEvent_t done[2] = {nullptr, nullptr};
  unsigned long long* dsum = nullptr;
  int dsum_n = 0;
  ~fv3g_ncfile() {
    for (int b = 0; b < 2; ++b) {
      if (pin[b]) cudaFreeHost(pin[b]);
      if (dev[b]) cudaFree(dev[b]);
      if (done[b]) cudaEventDestroy(done[b]);
    }
    if (dsum) cudaFree(dsum);
    if (fd >= 0) close(fd);
  }
};

namespace {

int read_at(int fd, void* buf, size_t bytes, long long off) {
  unsigned char* b = (unsigned char*)buf;
  while (bytes > 0) {
    ssize_t r = pread(fd, b, bytes, (off_t)off);
    if (r <= 0) return set_error(FV3G_E_ARG, "short read at offset %lld of a restart file", off);
    b += r;
    bytes -= (size_t)r;
    off += r;
  }
  return 0;
}

int write_at(int fd, const void* buf, size_t bytes, long long off) {
  const unsigned char* b = (const unsigned char*)buf;
  while (bytes > 0) {
    ssize_t r = pwrite(fd, b, bytes, (off_t)off);
    if (r <= 0) return set_error(FV3G_E_ARG, "write failed at offset %lld of a restart file", off);
    b += r;
    bytes -= (size_t)r;
    off += r;
  }
  return 0;
}

// Parse an attribute list (ABSENT or NC_ATTRIBUTE nelems [attr ...]).
bool parse_attrs(Cursor& c, std::vector<NcAttr>& out) {
  const long long tag = (long long)c.be(4);
  const long long count = c.nonneg();
  if (c.short_) return false;
  if (tag == 0 && count == 0) return true;
  if (tag != TAG_ATTRIBUTE || count < 0) return false;
  for (long long a = 0; a < count && !c.short_; ++a) {
    NcAttr at;
    at.name = c.name();
    at.type = (int)c.be(4);
    at.count = c.nonneg();
    const size_t es = type_size(at.type);
    if (c.short_ || es == 0 || at.count < 0) return false;
    const size_t len = (size_t)at.count * es;
    if (len > c.n - c.off) {
      c.short_ = true;
      return false;
    }
    at.raw.assign(c.p + c.off, c.p + c.off + len);
    c.skip_padded(len);
    out.push_back(std::move(at));
  }
  return !c.short_;
}

// Parse the header from the first `n` bytes of the file; returns 1 when more
// bytes are needed, 0 on success, an error code otherwise.
int parse_header(fv3g_ncfile* f, const unsigned char* p, size_t n) {
  Cursor c{p, n, 4, f->version};
  f->dim_names.clear();
  f->dim_len.clear();
  f->gatts.clear();
  f->vars.clear();
  f->numrecs = c.nonneg();
  if (f->version != 5 && f->numrecs == 0xFFFFFFFFLL) f->numrecs = 0;  // streaming: counted below
  long long tag = (long long)c.be(4), count = c.nonneg();
  if (c.short_) return 1;
  if (!(tag == 0 && count == 0)) {
    if (tag != TAG_DIMENSION || count < 0) return set_error(FV3G_E_ARG, "malformed netCDF dimension list");
    for (long long d = 0; d < count; ++d) {
      std::string nm = c.name();
      long long len = c.nonneg();
      if (c.short_) return 1;
      f->dim_names.push_back(nm);
      f->dim_len.push_back(len);
    }
  }
  if (!parse_attrs(c, f->gatts)) return c.short_ ? 1 : set_error(FV3G_E_ARG, "malformed netCDF attribute list");
  tag = (long long)c.be(4);
  count = c.nonneg();
  if (c.short_) return 1;
  if (!(tag == 0 && count == 0)) {
    if (tag != TAG_VARIABLE || count < 0) return set_error(FV3G_E_ARG, "malformed netCDF variable list");
    for (long long v = 0; v < count; ++v) {
      NcVar var;
      var.name = c.name();
      const long long nd = c.nonneg();
      if (c.short_) return 1;
      if (nd < 0 || nd > 64) return set_error(FV3G_E_ARG, "variable %s has %lld dimensions", var.name.c_str(), nd);
      for (long long d = 0; d < nd; ++d) var.dimids.push_back(c.nonneg());
      if (!parse_attrs(c, var.attrs)) return c.short_ ? 1 : set_error(FV3G_E_ARG, "malformed variable attributes");
      var.type = (int)c.be(4);
      (void)c.nonneg();  // vsize: recomputed from the shape (it saturates for large variables)
      var.begin = c.offset();
      if (c.short_) return 1;
      if (type_size(var.type) == 0) return set_error(FV3G_E_ARG, "variable %s has netCDF type %d", var.name.c_str(),
                                                     var.type);
      for (size_t d = 0; d < var.dimids.size(); ++d) {
        const long long id = var.dimids[d];
        if (id < 0 || id >= (long long)f->dim_len.size())
          return set_error(FV3G_E_ARG, "variable %s names dimension %lld", var.name.c_str(), id);
        if (f->dim_len[id] == 0) {
          if (d != 0) return set_error(FV3G_E_ARG, "record dimension not first in %s", var.name.c_str());
          var.record = true;
        } else {
          var.values *= f->dim_len[id];
        }
      }
      f->vars.push_back(std::move(var));
    }
  }
  // record stride: the padded per-record sizes of all record variables,
  // unpadded when there is only one
  int nrec = 0;
  f->recsize = 0;
  for (const NcVar& v : f->vars)
    if (v.record) {
      ++nrec;
      f->recsize += (long long)((v.values * type_size(v.type) + 3) & ~3ULL);
    }
  if (nrec == 1)
    for (const NcVar& v : f->vars)
      if (v.record) f->recsize = v.values * (long long)type_size(v.type);
  return 0;
}

const NcVar* find_var(const fv3g_ncfile* f, const char* name) {
  for (const NcVar& v : f->vars)
    if (v.name == name) return &v;
  return nullptr;
}

const NcAttr* find_attr(const NcVar& v, const char* name) {
  for (const NcAttr& a : v.attrs)
    if (a.name == name) return &a;
  return nullptr;
}

// The 'checksum' text attribute: hexadecimal digits with blanks around them.
bool parse_checksum(const NcAttr& a, unsigned long long* out) {
  if (a.type != NC_CHAR) return false;
  std::string s(a.raw.begin(), a.raw.end());
  size_t b = s.find_first_not_of(" \t\n\r");
  size_t e = s.find_last_not_of(" \t\n\r");
  if (b == std::string::npos) return false;
  s = s.substr(b, e - b + 1);
  if (s.empty() || s.size() > 16) return false;
  unsigned long long v = 0;
  for (char ch : s) {
    int d;
    if (ch >= '0' && ch <= '9') d = ch - '0';
    else if (ch >= 'A' && ch <= 'F') d = ch - 'A' + 10;
    else if (ch >= 'a' && ch <= 'f') d = ch - 'a' + 10;
    else return false;
    v = (v << 4) | (unsigned)d;
  }
  *out = v;
  return true;
}

// Fortran '(Z16)' of a 64-bit integer in a 32-character field, as the
// restart writer stores it: upper-case hexadecimal digits right-justified in
// 16 columns, then 16 blanks.
std::string z16(unsigned long long v) {
  char hex[17];
  snprintf(hex, sizeof hex, "%16llX", v);
  return std::string(hex) + std::string(16, ' ');
}

double host_value(const unsigned char* p, int type) {
  unsigned long long u = 0;
  const size_t es = type_size(type);
  for (size_t b = 0; b < es; ++b) u = (u << 8) | p[b];
  switch (type) {
    case NC_BYTE: return (double)(signed char)u;
    case NC_CHAR: case NC_UBYTE: return (double)u;
    case NC_SHORT: return (double)(short)u;
    case NC_USHORT: return (double)u;
    case NC_INT: return (double)(int)(unsigned)u;
    case NC_UINT: return (double)u;
    case NC_INT64: return (double)(long long)u;
    case NC_UINT64: return (double)u;
    case NC_FLOAT: {
      unsigned w = (unsigned)u;
      float x;
      memcpy(&x, &w, 4);
      return x;
    }
    default: {
      double x;
      memcpy(&x, &u, 8);
      return x;
    }
  }
}

// ------------------------------------------------------------- kernels --
__device__ __forceinline__ unsigned bswap32(unsigned x) { return __byte_perm(x, 0, 0x0123); }
__device__ __forceinline__ unsigned long long bswap64(unsigned long long x) {
  return ((unsigned long long)bswap32((unsigned)x) << 32) | bswap32((unsigned)(x >> 32));
}

template <typename S> struct Bits;
template <> struct Bits<double> {
  using U = unsigned long long;
  static __device__ __forceinline__ double from_be(U w) { return __longlong_as_double((long long)bswap64(w)); }
  static __device__ __forceinline__ U to_be(double v) { return bswap64((U)__double_as_longlong(v)); }
  // mpp_chksum of FP64 data: the bit patterns summed as 64-bit integers
  static __device__ __forceinline__ unsigned long long term(double v) { return (U)__double_as_longlong(v); }
};
template <> struct Bits<float> {
  using U = unsigned;
  static __device__ __forceinline__ float from_be(U w) { return __int_as_float((int)bswap32(w)); }
  static __device__ __forceinline__ U to_be(float v) { return bswap32((U)__float_as_int(v)); }
  // mpp_chksum of FP32 data: the bit patterns as 32-bit integers, sign-extended
  static __device__ __forceinline__ unsigned long long term(float v) {
    return (unsigned long long)(long long)__float_as_int(v);
  }
};

__device__ __forceinline__ void block_sum_add(unsigned long long acc, unsigned long long* sum) {
  __shared__ unsigned long long part[32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) part[warp] = acc;
  __syncthreads();
  if (warp == 0) {
    acc = (lane < (int)(blockDim.x >> 5)) ? part[lane] : 0ULL;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) atomicAdd(sum, acc);
  }
}

// File values (rows of n, nrows = nlev * n, big-endian S) into the planes of
// one (tile, tracer): row r = k*n + j goes to plane k, row j+1, columns 1..n.
template <typename S, typename T>
__global__ void __launch_bounds__(256) k_nc_unpack(const typename Bits<S>::U* __restrict__ src, T* __restrict__ dst,
                                                   PlaneGeom pg, long long plane, int n, long long nrows,
                                                   unsigned long long* __restrict__ sum) {
  unsigned long long acc = 0;
  for (long long r = blockIdx.x; r < nrows; r += gridDim.x) {
    const long long k = r / n;
    const int j = (int)(r - k * n) + 1;
    const typename Bits<S>::U* row = src + r * n;
    T* out = dst + k * plane + pg.at(1, j);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const S v = Bits<S>::from_be(row[i]);
      acc += Bits<S>::term(v);
      out[i] = (T)v;
    }
  }
  block_sum_add(acc, sum);
}

// The mirror image: planes of one (tile, tracer) into big-endian file rows.
template <typename T, typename S>
__global__ void __launch_bounds__(256) k_nc_pack(const T* __restrict__ src, typename Bits<S>::U* __restrict__ dst,
                                                 PlaneGeom pg, long long plane, int n, long long nrows,
                                                 unsigned long long* __restrict__ sum) {
  unsigned long long acc = 0;
  for (long long r = blockIdx.x; r < nrows; r += gridDim.x) {
    const long long k = r / n;
    const int j = (int)(r - k * n) + 1;
    const T* in = src + k * plane + pg.at(1, j);
    typename Bits<S>::U* row = dst + r * n;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const S v = (S)in[i];
      acc += Bits<S>::term(v);
      row[i] = Bits<S>::to_be(v);
    }
  }
  block_sum_add(acc, sum);
}

unsigned row_blocks(long long nrows) { return (unsigned)std::min<long long>(nrows, 152LL * 8); }

template <typename T>
int launch_unpack(int ftype, const void* src, void* dst, const StateFieldView& v, long long nrows,
                  unsigned long long* sum, cudaStream_t s) {
  if (ftype == NC_DOUBLE)
    k_nc_unpack<double, T><<<row_blocks(nrows), 256, 0, s>>>((const unsigned long long*)src, (T*)dst, v.pg, v.plane,
                                                             v.n, nrows, sum);
  else
    k_nc_unpack<float, T><<<row_blocks(nrows), 256, 0, s>>>((const unsigned*)src, (T*)dst, v.pg, v.plane, v.n, nrows,
                                                            sum);
  FV3G_CUDA(cudaGetLastError());
  return 0;
}

template <typename T>
int launch_pack(int ftype, const void* src, void* dst, const StateFieldView& v, long long nrows,
                unsigned long long* sum, cudaStream_t s) {
  if (ftype == NC_DOUBLE)
    k_nc_pack<T, double><<<row_blocks(nrows), 256, 0, s>>>((const T*)src, (unsigned long long*)dst, v.pg, v.plane, v.n,
                                                           nrows, sum);
  else
    k_nc_pack<T, float><<<row_blocks(nrows), 256, 0, s>>>((const T*)src, (unsigned*)dst, v.pg, v.plane, v.n, nrows,
                                                          sum);
  FV3G_CUDA(cudaGetLastError());
  return 0;
}

int ensure_staging(fv3g_ncfile* f, size_t bytes, int nsums) {
  if (f->stage < bytes) {
    for (int b = 0; b < 2; ++b) {
      if (f->pin[b]) cudaFreeHost(f->pin[b]);
      if (f->dev[b]) cudaFree(f->dev[b]);
      f->pin[b] = nullptr;
      f->dev[b] = nullptr;
    }
    f->stage = 0;
    for (int b = 0; b < 2; ++b) {
      FV3G_CUDA(cudaHostAlloc((void**)&f->pin[b], bytes, cudaHostAllocDefault));
      FV3G_CUDA(cudaMalloc((void**)&f->dev[b], bytes));
    }
    f->stage = bytes;
  }
  for (int b = 0; b < 2; ++b)
    if (!f->done[b]) FV3G_CUDA(cudaEventCreateWithFlags(&f->done[b], cudaEventDisableTiming));
  if (f->dsum_n < nsums) {
    if (f->dsum) cudaFree(f->dsum);
    f->dsum = nullptr;
    FV3G_CUDA(cudaMalloc((void**)&f->dsum, sizeof(unsigned long long) * nsums));
    f->dsum_n = nsums;
  }
  return 0;
}

// Where variable `slot` of tile `tile` starts in the state's field.
void* plane_base(const StateFieldView& v, int field, int tile, int slot) {
  long long p = (field == FV3G_FIELD_Q) ? ((long long)tile * v.nq + slot) * v.npz : (long long)tile * v.npz;
  return (char*)v.dev + (size_t)(p * v.plane) * v.esz;
}

int check_slots(int field, const StateFieldView& v, int tile, const int* slots, int nvars) {
  if (tile < 0 || tile >= v.ntiles) return set_error(FV3G_E_ARG, "tile %d outside 0..%d", tile, v.ntiles - 1);
  if (nvars < 1) return set_error(FV3G_E_ARG, "no variables");
  if (field == FV3G_FIELD_DELP) {
    if (nvars != 1) return set_error(FV3G_E_ARG, "delp is one variable");
    return 0;
  }
  if (!slots) return set_error(FV3G_E_ARG, "tracer slots missing");
  for (int i = 0; i < nvars; ++i)
    if (slots[i] < 0 || slots[i] >= v.nq) return set_error(FV3G_E_ARG, "tracer slot %d outside 0..%d", slots[i],
                                                           v.nq - 1);
  return 0;
}

// --------------------------------------------------------------- writing --
struct HeaderWriter {
  std::vector<unsigned char> b;
  int version;
  void be(unsigned long long v, int bytes) {
    for (int k = bytes - 1; k >= 0; --k) b.push_back((unsigned char)(v >> (8 * k)));
  }
  void nonneg(long long v) { be((unsigned long long)v, version == 5 ? 8 : 4); }
  void offset(long long v) { be((unsigned long long)v, version == 1 ? 4 : 8); }
  void pad() {
    while (b.size() % 4) b.push_back(0);
  }
  void name(const std::string& s) {
    nonneg((long long)s.size());
    b.insert(b.end(), s.begin(), s.end());
    pad();
  }
  void text_attr(const std::string& nm, const std::string& value) {
    name(nm);
    be(NC_CHAR, 4);
    nonneg((long long)value.size());
    b.insert(b.end(), value.begin(), value.end());
    pad();
  }
};

struct OutVar {
  std::string name;
  std::vector<int> dims;
  std::vector<std::pair<std::string, std::string>> text;
  int type;
  long long bytes;  // per record for record variables
  bool record;
  long long begin = 0;
};

// Header of the write component's layout with the given offsets (index i of
// vars gets begins[i]); returns its bytes.
std::vector<unsigned char> build_header(int version, int n, int npz, const std::vector<OutVar>& vars) {
  HeaderWriter h{{}, version};
  h.b.insert(h.b.end(), {'C', 'D', 'F', (unsigned char)version});
  h.nonneg(1);  // numrecs
  h.be(TAG_DIMENSION, 4);
  h.nonneg(4);
  const char* dn[4] = {"xaxis_1", "yaxis_1", "zaxis_1", "Time"};
  const long long dl[4] = {n, n, npz, 0};
  for (int d = 0; d < 4; ++d) {
    h.name(dn[d]);
    h.nonneg(dl[d]);
  }
  h.be(TAG_ATTRIBUTE, 4);  // global: NumFilesInSet = 1
  h.nonneg(1);
  h.name("NumFilesInSet");
  h.be(NC_INT, 4);
  h.nonneg(1);
  h.be(1, 4);
  h.be(TAG_VARIABLE, 4);
  h.nonneg((long long)vars.size());
  for (const OutVar& v : vars) {
    h.name(v.name);
    h.nonneg((long long)v.dims.size());
    for (int d : v.dims) h.nonneg(d);
    if (v.text.empty()) {
      h.be(0, 4);
      h.nonneg(0);
    } else {
      h.be(TAG_ATTRIBUTE, 4);
      h.nonneg((long long)v.text.size());
      for (const auto& a : v.text) h.text_attr(a.first, a.second);
    }
    h.be((unsigned long long)v.type, 4);
    const long long vsize = (v.bytes + 3) & ~3LL;
    h.nonneg(version == 5 ? vsize : std::min<long long>(vsize, 0xFFFFFFFFLL));
    h.offset(v.begin);
  }
  return h.b;
}

void put_be_double(std::vector<unsigned char>& out, double x) {
  unsigned long long u;
  memcpy(&u, &x, 8);
  for (int k = 7; k >= 0; --k) out.push_back((unsigned char)(u >> (8 * k)));
}

}  // namespace

extern "C" {

int fv3g_nc_open(const char* path, fv3g_ncfile** out) {
  if (!path || !out) return set_error(FV3G_E_ARG, "null argument");
  *out = nullptr;
  const int fd = open(path, O_RDONLY);
  if (fd < 0) return set_error(FV3G_E_ARG, "cannot open %s", path);
  fv3g_ncfile* f = new fv3g_ncfile;
  f->fd = fd;
  struct stat sb;
  if (fstat(fd, &sb) != 0) {
    delete f;
    return set_error(FV3G_E_ARG, "cannot stat %s", path);
  }
  f->file_bytes = (long long)sb.st_size;
  unsigned char magic[8] = {0};
  if (f->file_bytes < 8 || pread(fd, magic, 8, 0) != 8) {
    delete f;
    return set_error(FV3G_E_ARG, "%s is not a netCDF file", path);
  }
  if (magic[0] == 0x89 && magic[1] == 'H' && magic[2] == 'D' && magic[3] == 'F') {
    delete f;
    return set_error(FV3G_E_UNSUPPORTED, "%s is netCDF-4 (HDF5); convert it to CDF-5 or 64-bit offset first",
                     path);
  }
  if (magic[0] != 'C' || magic[1] != 'D' || magic[2] != 'F' || (magic[3] != 1 && magic[3] != 2 && magic[3] != 5)) {
    delete f;
    return set_error(FV3G_E_ARG, "%s is not a netCDF classic, 64-bit offset or CDF-5 file", path);
  }
  f->version = magic[3];
  size_t want = (size_t)std::min<long long>(f->file_bytes, 1 << 16);
  for (;;) {
    std::vector<unsigned char> buf(want);
    int rc = read_at(fd, buf.data(), want, 0);
    if (rc) {
      delete f;
      return rc;
    }
    rc = parse_header(f, buf.data(), want);
    if (rc == 0) break;
    if (rc != 1 || want == (size_t)f->file_bytes) {
      delete f;
      return rc == 1 ? set_error(FV3G_E_ARG, "truncated netCDF header in %s", path) : rc;
    }
    want = (size_t)std::min<long long>(f->file_bytes, (long long)want * 4);
  }
  if (f->numrecs == 0 && f->recsize > 0) {  // streaming files count their records from the size
    long long first = -1;
    for (const NcVar& v : f->vars)
      if (v.record && (first < 0 || v.begin < first)) first = v.begin;
    if (first >= 0) f->numrecs = (f->file_bytes - first) / f->recsize;
  }
  *out = f;
  return 0;
}

int fv3g_nc_close(fv3g_ncfile* f) {
  delete f;
  return 0;
}

int fv3g_nc_nvars(fv3g_ncfile* f, int* nvars) {
  if (!f || !nvars) return set_error(FV3G_E_ARG, "null argument");
  *nvars = (int)f->vars.size();
  return 0;
}

int fv3g_nc_var_info(fv3g_ncfile* f, int idx, char* name, int len, int* nc_type, int* ndims, long long* shape,
                     int* is_record) {
  if (!f) return set_error(FV3G_E_ARG, "null file");
  if (idx < 0 || idx >= (int)f->vars.size()) return set_error(FV3G_E_ARG, "variable index %d outside 0..%d", idx,
                                                              (int)f->vars.size() - 1);
  const NcVar& v = f->vars[idx];
  if (name && len > 0) {
    const size_t m = std::min(v.name.size(), (size_t)len - 1);
    memcpy(name, v.name.data(), m);
    name[m] = '\0';
  }
  if (nc_type) *nc_type = v.type;
  if (ndims) *ndims = (int)v.dimids.size();
  if (shape)
    for (size_t d = 0; d < v.dimids.size() && d < 8; ++d) {
      const long long l = f->dim_len[v.dimids[d]];
      shape[d] = l == 0 ? f->numrecs : l;
    }
  if (is_record) *is_record = v.record ? 1 : 0;
  return 0;
}

int fv3g_nc_checksum(fv3g_ncfile* f, const char* name, unsigned long long* checksum, int* present) {
  if (!f || !name || !checksum || !present) return set_error(FV3G_E_ARG, "null argument");
  const NcVar* v = find_var(f, name);
  if (!v) return set_error(FV3G_E_ARG, "no variable %s", name);
  const NcAttr* a = find_attr(*v, "checksum");
  *present = 0;
  if (!a) return 0;
  if (!parse_checksum(*a, checksum)) return set_error(FV3G_E_ARG, "unreadable checksum attribute of %s", name);
  *present = 1;
  return 0;
}

int fv3g_nc_read(fv3g_ncfile* f, const char* name, int record, double* out, long long count) {
  if (!f || !name || !out) return set_error(FV3G_E_ARG, "null argument");
  const NcVar* v = find_var(f, name);
  if (!v) return set_error(FV3G_E_ARG, "no variable %s", name);
  if (count != v->values)
    return set_error(FV3G_E_ARG, "variable %s holds %lld values per record, not %lld", name, v->values, count);
  long long off = v->begin;
  if (v->record) {
    if (record < 0 || record >= f->numrecs) return set_error(FV3G_E_ARG, "record %d outside 0..%lld of %s", record,
                                                             f->numrecs - 1, name);
    off += (long long)record * f->recsize;
  }
  const size_t es = type_size(v->type);
  std::vector<unsigned char> raw((size_t)count * es);
  CHECK(read_at(f->fd, raw.data(), raw.size(), off));
  for (long long i = 0; i < count; ++i) out[i] = host_value(raw.data() + (size_t)i * es, v->type);
  return 0;
}

int fv3g_state_read_restart(fv3g_state* st, int field, int tile, fv3g_ncfile* f, const char* const* names,
                            const int* slots, int nvars, int verify, unsigned long long* checksums) {
  if (!st || !f || !names) return set_error(FV3G_E_ARG, "null argument");
  StateFieldView view;
  CHECK(state_field_view(st, field, true, &view));
  CHECK(check_slots(field, view, tile, slots, nvars));
  const long long nrows = (long long)view.npz * view.n, nvals = nrows * view.n;
  std::vector<const NcVar*> vs(nvars);
  size_t most = 0;
  for (int i = 0; i < nvars; ++i) {
    const NcVar* v = names[i] ? find_var(f, names[i]) : nullptr;
    if (!v) return set_error(FV3G_E_ARG, "no variable %s", names[i] ? names[i] : "(null)");
    if (v->type != NC_FLOAT && v->type != NC_DOUBLE)
      return set_error(FV3G_E_UNSUPPORTED, "variable %s is not float or double", v->name.c_str());
    const size_t nd = v->dimids.size() - (v->record ? 1 : 0);
    const long long* dl = f->dim_len.data();
    const std::vector<long long>& id = v->dimids;
    const size_t o = v->record ? 1 : 0;
    if (nd != 3 || dl[id[o]] != view.npz || dl[id[o + 1]] != view.n || dl[id[o + 2]] != view.n)
      return set_error(FV3G_E_ARG, "variable %s is not (zaxis, yaxis, xaxis) = (%d, %d, %d)", v->name.c_str(),
                       view.npz, view.n, view.n);
    if (v->record && f->numrecs < 1) return set_error(FV3G_E_ARG, "variable %s has no record", v->name.c_str());
    vs[i] = v;
    most = std::max(most, (size_t)nvals * type_size(v->type));
  }
  cudaStream_t s = view.stream;
  CHECK(ensure_staging(f, most, nvars));
  FV3G_CUDA(cudaMemsetAsync(f->dsum, 0, sizeof(unsigned long long) * nvars, s));
  for (int i = 0; i < nvars; ++i) {
    const int b = i & 1;
    const size_t bytes = (size_t)nvals * type_size(vs[i]->type);
    if (i >= 2) FV3G_CUDA(cudaEventSynchronize(f->done[b]));  // buffer b's last copy and unpack are done
    CHECK(read_at(f->fd, f->pin[b], bytes, vs[i]->begin));   // record 0; overlaps the GPU work on the other buffer
    FV3G_CUDA(cudaMemcpyAsync(f->dev[b], f->pin[b], bytes, cudaMemcpyHostToDevice, s));
    void* dst = plane_base(view, field, tile, field == FV3G_FIELD_Q ? slots[i] : 0);
    CHECK(view.esz == 8 ? launch_unpack<double>(vs[i]->type, f->dev[b], dst, view, nrows, f->dsum + i, s)
                        : launch_unpack<float>(vs[i]->type, f->dev[b], dst, view, nrows, f->dsum + i, s));
    FV3G_CUDA(cudaEventRecord(f->done[b], s));
  }
  std::vector<unsigned long long> sums(nvars);
  FV3G_CUDA(cudaMemcpyAsync(sums.data(), f->dsum, sizeof(unsigned long long) * nvars, cudaMemcpyDeviceToHost, s));
  FV3G_CUDA(cudaStreamSynchronize(s));
  for (int i = 0; i < nvars; ++i) {
    if (checksums) checksums[i] = sums[i];
    if (!verify) continue;
    const NcAttr* a = find_attr(*vs[i], "checksum");
    if (!a) continue;
    unsigned long long want = 0;
    if (!parse_checksum(*a, &want) || want != sums[i])
      return set_error(FV3G_E_CHECKSUM, "checksum of %s: file says %s, data sums to %016llX", vs[i]->name.c_str(),
                       std::string(a->raw.begin(), a->raw.end()).c_str(), sums[i]);
  }
  return 0;
}

int fv3g_state_write_restart(fv3g_state* st, int field, int tile, const char* path, const char* const* names,
                             const int* slots, int nvars, int nc_type, int version, unsigned long long* checksums) {
  if (!st || !path || !names) return set_error(FV3G_E_ARG, "null argument");
  if (nc_type != NC_FLOAT && nc_type != NC_DOUBLE)
    return set_error(FV3G_E_ARG, "nc_type must be FV3G_NC_FLOAT or FV3G_NC_DOUBLE (got %d)", nc_type);
  if (version != 1 && version != 2 && version != 5)
    return set_error(FV3G_E_ARG, "version must be 1, 2 or 5 (got %d)", version);
  StateFieldView view;
  CHECK(state_field_view(st, field, false, &view));
  CHECK(check_slots(field, view, tile, slots, nvars));
  for (int i = 0; i < nvars; ++i)
    if (!names[i] || !names[i][0]) return set_error(FV3G_E_ARG, "variable %d has no name", i);
  const long long nrows = (long long)view.npz * view.n, nvals = nrows * view.n;
  const long long vbytes = nvals * (long long)type_size(nc_type);
  if (version != 5 && vbytes > 0xFFFFFFFFLL - 4)
    return set_error(FV3G_E_ARG, "a %lld-byte variable needs version 5 (CDF-5)", vbytes);

  // layout: axis variables (fixed), then the record section: Time and the fields
  std::vector<OutVar> vars;
  vars.push_back({"xaxis_1", {0}, {{"axis", "X"}}, NC_DOUBLE, 8LL * view.n, false});
  vars.push_back({"yaxis_1", {1}, {{"axis", "Y"}}, NC_DOUBLE, 8LL * view.n, false});
  vars.push_back({"zaxis_1", {2}, {{"axis", "Z"}}, NC_DOUBLE, 8LL * view.npz, false});
  vars.push_back({"Time", {3}, {{"cartesian_axis", "T"}, {"units", "time level"}, {"long_name", "Time"}}, NC_DOUBLE,
                  8, true});
  for (int i = 0; i < nvars; ++i)
    vars.push_back({names[i], {3, 2, 1, 0}, {{"checksum", z16(0)}}, nc_type, vbytes, true});
  const size_t hbytes = build_header(version, view.n, view.npz, vars).size();
  if (version == 1 && (long long)hbytes + 8LL * (2 * view.n + view.npz + 1) + vbytes * nvars > 0x7FFFFFFFLL)
    return set_error(FV3G_E_ARG, "the file exceeds 2 GiB: use version 2 or 5");
  long long off = (long long)hbytes;
  for (OutVar& v : vars)
    if (!v.record) {
      v.begin = off;
      off += (v.bytes + 3) & ~3LL;
    }
  for (OutVar& v : vars)
    if (v.record) {
      v.begin = off;
      off += (v.bytes + 3) & ~3LL;
    }

  fv3g_ncfile scratch;  // staging buffers only
  const int fd = open(path, O_WRONLY | O_CREAT | O_TRUNC, 0644);
  if (fd < 0) return set_error(FV3G_E_ARG, "cannot create %s", path);
  auto fail = [&](int rc) {
    close(fd);
    return rc;
  };
  int rc = ensure_staging(&scratch, (size_t)vbytes, nvars);
  if (rc) return fail(rc);
  cudaStream_t s = view.stream;
  if (cudaMemsetAsync(scratch.dsum, 0, sizeof(unsigned long long) * nvars, s) != cudaSuccess)
    return fail(set_error(FV3G_E_CUDA, "cudaMemsetAsync failed"));
  // axis values 1..n, 1..npz and Time = 1, big-endian
  for (int a = 0; a < 4; ++a) {
    std::vector<unsigned char> raw;
    const long long cnt = vars[a].bytes / 8;
    for (long long i = 1; i <= cnt; ++i) put_be_double(raw, (double)i);
    if ((rc = write_at(fd, raw.data(), raw.size(), vars[a].begin))) return fail(rc);
  }
  // variable i is packed on the GPU while the host writes variable i-1
  for (int i = 0; i <= nvars; ++i) {
    if (i < nvars) {
      const int b = i & 1;
      const void* src = plane_base(view, field, tile, field == FV3G_FIELD_Q ? slots[i] : 0);
      rc = view.esz == 8 ? launch_pack<double>(nc_type, src, scratch.dev[b], view, nrows, scratch.dsum + i, s)
                         : launch_pack<float>(nc_type, src, scratch.dev[b], view, nrows, scratch.dsum + i, s);
      if (rc) return fail(rc);
      if (cudaMemcpyAsync(scratch.pin[b], scratch.dev[b], (size_t)vbytes, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
          cudaEventRecord(scratch.done[b], s) != cudaSuccess)
        return fail(set_error(FV3G_E_CUDA, "packing %s failed", names[i]));
    }
    if (i > 0) {
      const int b = (i - 1) & 1;
      if (cudaEventSynchronize(scratch.done[b]) != cudaSuccess)
        return fail(set_error(FV3G_E_CUDA, "packing %s failed", names[i - 1]));
      if ((rc = write_at(fd, scratch.pin[b], (size_t)vbytes, vars[4 + i - 1].begin))) return fail(rc);
    }
  }
  std::vector<unsigned long long> sums(nvars);
  if (cudaMemcpy(sums.data(), scratch.dsum, sizeof(unsigned long long) * nvars, cudaMemcpyDeviceToHost) !=
      cudaSuccess)
    return fail(set_error(FV3G_E_CUDA, "reading the checksums failed"));
  for (int i = 0; i < nvars; ++i) {
    vars[4 + i].text[0].second = z16(sums[i]);
    if (checksums) checksums[i] = sums[i];
  }
  const std::vector<unsigned char> header = build_header(version, view.n, view.npz, vars);
  if ((rc = write_at(fd, header.data(), header.size(), 0))) return fail(rc);
  // pad the last record variable to its padded size so the file length matches the layout
  if (off > vars.back().begin + vars.back().bytes) {
    const unsigned char zero[4] = {0, 0, 0, 0};
    if ((rc = write_at(fd, zero, (size_t)(off - vars.back().begin - vars.back().bytes),
                       vars.back().begin + vars.back().bytes)))
      return fail(rc);
  }
  if (close(fd) != 0) return set_error(FV3G_E_ARG, "closing %s failed", path);
  return 0;
}

}  // extern "C"
