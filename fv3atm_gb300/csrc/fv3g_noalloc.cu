// fv3g_noalloc.cu -- column remap on caller-owned device arrays without any
// device allocation by the library.
//
// Some callers cannot let a library allocate GPU memory: a model that keeps
// its own device memory pool (for example a Fortran dynamical core ported with
// OpenACC that hands its device arrays over with host_data use_device) and
// forbids other allocations inside its time loop, or code that must not
// trigger the implicit device synchronisation of cudaMalloc/cudaFree.  For
// them, fv3g_remap_columns_noalloc runs the thread-per-column remap kernel
// (k_remap_scratch, which the tangent-linear remap also uses; map_scalar,
// map1_ppm and the batched remap run the warp-per-column kernel, and the
// tests check this entry against one of those) with its scratch held in one
// file-scope __device__ array of fixed size instead of a buffer obtained
// from cudaMalloc.  The addresses of that array are looked up once per
// device and kept: a device reset after the first call is not supported.
#include <cuda_runtime.h>

#include <mutex>

#include "fv3g_internal.cuh"
#include "fv3g_remap.cuh"

namespace fv3g {
namespace {

// Largest number of columns one call may remap (every call may also use up to
// KMAX source and KMAX target layers).  The arrays below take
// 6 * (KMAX+1) * 1024 doubles + (KMAX+1) * 1024 bytes = 6.5 MB of device memory
// on every GPU that loads the library, until the process exits.
constexpr long long kNoAllocMaxCols = 1024;

static __device__ __align__(256) double g_scratch[6 * (KMAX + 1) * kNoAllocMaxCols];
static __device__ __align__(256) unsigned char g_sched[(KMAX + 1) * kNoAllocMaxCols];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
double* g_scratch_ptr[kMaxDevices] = {};
unsigned char* g_sched_ptr[kMaxDevices] = {};

// Device addresses of the two arrays on the current device.  In host code the
// array names are host-side stand-ins, not device addresses, so the addresses
// are looked up once per device with cudaGetSymbolAddress (with that device
// current) and cached.
int device_scratch(double** scratch, unsigned char** sched) {
  int dev = 0;
  FV3G_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return set_error(FV3G_E_ARG, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_mutex);
  if (g_scratch_ptr[dev] == nullptr) {
    void* a = nullptr;
    void* b = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&a, g_scratch);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(scratch)");
    e = cudaGetSymbolAddress(&b, g_sched);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(schedule)");
    g_scratch_ptr[dev] = (double*)a;
    g_sched_ptr[dev] = (unsigned char*)b;
  }
  *scratch = g_scratch_ptr[dev];
  *sched = g_sched_ptr[dev];
  return 0;
}

}  // namespace
}  // namespace fv3g

using namespace fv3g;

extern "C" int fv3g_remap_columns_noalloc(int ncol, int km, const double* pe1, const double* q1, const double* qs,
                                          int kn, const double* pe2, double* q2, int nfield, int iv, int kord,
                                          double q_min, void* stream) {
  if (!pe1 || !q1 || !pe2 || !q2) return set_error(FV3G_E_ARG, "null array argument");
  if (ncol < 1 || ncol > kNoAllocMaxCols)
    return set_error(FV3G_E_ARG, "fv3g_remap_columns_noalloc handles 1..%lld columns per call (got %d)",
                     kNoAllocMaxCols, ncol);
  if (km < 1 || km > KMAX || kn < 1 || kn > KMAX)
    return set_error(FV3G_E_ARG, "fv3g_remap_columns_noalloc handles 1..%d layers (km=%d, kn=%d)", KMAX, km, kn);
  if (nfield < 1) return set_error(FV3G_E_ARG, "nfield must be positive");
  if (kord != 4 && kord != 9) return set_error(FV3G_E_UNSUPPORTED, "kord %d not implemented (4 and 9 are)", kord);
  if (iv < -2 || iv > 1) return set_error(FV3G_E_ARG, "iv %d outside -2..1", iv);
  if (iv == -2 && qs == nullptr) return set_error(FV3G_E_ARG, "iv -2 needs the surface values qs");
  double* scratch = nullptr;
  unsigned char* sched = nullptr;
  int rc = device_scratch(&scratch, &sched);
  if (rc) return rc;
  // The kernel writes every scratch element of a column before reading it,
  // so nothing has to be cleared between calls.
  RemapArgs<double> r{};
  r.q_in = q1;
  r.q_out = q2;
  r.sQt = 0;
  r.sQk = ncol;
  r.sQq = (long long)ncol * km;
  r.sQqo = (long long)ncol * kn;
  r.nfield = nfield;
  r.pe1 = pe1;
  r.pe2 = pe2;
  r.qs = qs;
  r.pg.pitch = ncol;
  r.pg.rows = 1;
  r.pg.isd = 1;
  r.pg.jsd = 1;
  r.i1 = 1;
  r.j1 = 1;
  r.ni = ncol;
  r.nj = 1;
  r.ncol = ncol;
  r.km = km;
  r.kn = kn;
  r.iv = iv;
  r.q_min = q_min;
  r.scratch = scratch;
  r.sched = sched;
  return launch_remap<double>(r, kord, (cudaStream_t)stream);
}
