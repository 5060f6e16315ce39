// Host-pointer forward transform that allocates no device memory.
//
// kd_coef_host stages its host input and output through device buffers taken
// from the context's scratch arena, which may call cudaMalloc.  This variant
// stages through the fixed file-scope device arrays below instead, for callers
// that cannot let a library allocate GPU memory: applications that reserve
// their whole device memory budget up front and hand it out from their own
// pool, where an allocation by the library fails or breaks the budget, and
// code running between the steps of such an application, where a cudaFree
// would also synchronise the whole device.  Every GPU that loads the library
// holds these arrays until the process exits (2 x 8 MiB of doubles plus
// 64 KiB of table space).  The call allocates nothing: the per-line matrices
// go into the context's matrix pool, which is allocated once when the context
// is created.
//
// The first call on a device looks up the arrays' device addresses there
// (cudaGetSymbolAddress, with that device current); make that first call
// before any stream capture.
//
// The arrays are shared by every call on a device and keep the contents of
// the last call; two calls whose GPU work overlaps (two host threads, or two
// contexts on one device) race on them.  Nothing here needs to start at zero:
// each call overwrites the input staging, the table entries it uses and the
// whole output range it reads back.
#include <cuda_runtime.h>

#include <mutex>
#include <vector>

#include "kadath_gb300.h"
#include "kd_noalloc.hpp"
#include "kd_spectral.hpp"

namespace kd {

static __device__ __align__(256) double g_noalloc_in[KD_NOALLOC_MAX_DOUBLES];
static __device__ __align__(256) double g_noalloc_out[KD_NOALLOC_MAX_DOUBLES];
static __device__ __align__(256) int g_noalloc_tab[KD_NOALLOC_MAX_TABLE];

namespace {

struct DevicePtrs {
  bool ready = false;
  double* in = nullptr;
  double* out = nullptr;
  int* tab = nullptr;
};

// Makes `device` current for its lifetime and restores the caller's device
// on every exit path, exceptions included.
class DeviceGuard {
 public:
  explicit DeviceGuard(int device) {
    cuda_check(cudaGetDevice(&prev_), "cudaGetDevice");
    if (prev_ != device) cuda_check(cudaSetDevice(device), "cudaSetDevice");
    switched_ = prev_ != device;
  }
  ~DeviceGuard() {
    if (switched_) cudaSetDevice(prev_);
  }
  DeviceGuard(const DeviceGuard&) = delete;
  DeviceGuard& operator=(const DeviceGuard&) = delete;

 private:
  int prev_ = -1;
  bool switched_ = false;
};

constexpr int kMaxDevices = 64;
DevicePtrs g_ptrs[kMaxDevices];
std::mutex g_mu;

// Device addresses of the static arrays, resolved once per device with that
// device current (host code must not pass the symbols themselves: on the host
// they are stand-ins, not device addresses).
const DevicePtrs& device_ptrs(int device) {
  if (device < 0 || device >= kMaxDevices) throw KdError(KD_ERR_ARG, "device index out of range");
  std::lock_guard<std::mutex> lock(g_mu);
  DevicePtrs& p = g_ptrs[device];
  if (!p.ready) {
    DeviceGuard guard(device);
    double* in = nullptr;
    double* out = nullptr;
    int* tab = nullptr;
    cuda_check(cudaGetSymbolAddress(reinterpret_cast<void**>(&in), g_noalloc_in), "cudaGetSymbolAddress(in)");
    cuda_check(cudaGetSymbolAddress(reinterpret_cast<void**>(&out), g_noalloc_out), "cudaGetSymbolAddress(out)");
    cuda_check(cudaGetSymbolAddress(reinterpret_cast<void**>(&tab), g_noalloc_tab), "cudaGetSymbolAddress(tab)");
    p.in = in;
    p.out = out;
    p.tab = tab;
    p.ready = true;
  }
  return p;
}

}  // namespace

void coef_host_noalloc(Context& ctx, const Base& base, const int np[3], const int nc[3], int batch,
                       const double* h_in, double* h_out) {
  if (batch <= 0) return;
  const long long n_in = static_cast<long long>(np[0]) * np[1] * np[2];
  const long long n_out = static_cast<long long>(nc[0]) * nc[1] * nc[2];
  if (n_in * batch > KD_NOALLOC_MAX_DOUBLES || n_out * batch > KD_NOALLOC_MAX_DOUBLES)
    throw KdError(KD_ERR_ARG, "kd_coef_host_noalloc: batch * field size exceeds KD_NOALLOC_MAX_DOUBLES");
  // Per-line matrix offsets of the three passes, laid out back to back.
  std::vector<LinePassSpec> specs = coef_specs(ctx, base, np, nc);
  std::vector<int> tab;
  int start[3];
  for (int q = 0; q < 3; q++) {
    start[q] = static_cast<int>(tab.size());
    tab.insert(tab.end(), specs[q].offsets.begin(), specs[q].offsets.end());
  }
  if (static_cast<long long>(tab.size()) > KD_NOALLOC_MAX_TABLE)
    throw KdError(KD_ERR_ARG, "kd_coef_host_noalloc: basis table exceeds KD_NOALLOC_MAX_TABLE");
  const DevicePtrs& p = device_ptrs(ctx.device());
  cudaStream_t s = ctx.stream();
  const double* pool = ctx.pool();  // uploads new matrices into the existing pool (no allocation)
  cuda_check(cudaMemcpyAsync(p.tab, tab.data(), tab.size() * sizeof(int), cudaMemcpyHostToDevice, s), "table upload");
  cuda_check(cudaMemcpyAsync(p.in, h_in, sizeof(double) * n_in * batch, cudaMemcpyHostToDevice, s), "H2D");
  KdItemList list{};
  list.nitems = 1;
  list.prefix[0] = 0;
  list.prefix[1] = batch;
  KdItem& it = list.items[0];
  it.in = p.in;
  it.out = p.out;
  it.in_stride = n_in;
  it.out_stride = n_out;
  it.n0 = np[0];
  it.n1 = np[1];
  it.n2 = np[2];
  it.npass = 3;
  it.scale = 1.0;
  int maxe = static_cast<int>(n_in);
  int d[3] = {np[0], np[1], np[2]};
  for (int q = 0; q < 3; q++) {
    it.pass[q].dim = specs[q].dim;
    it.pass[q].n_in = specs[q].n_in;
    it.pass[q].n_out = specs[q].n_out;
    it.pass[q].mat_ld = specs[q].mat_ld;
    it.pass[q].mat = p.tab + start[q];
    d[specs[q].dim] = specs[q].n_out;
    int e = d[0] * d[1] * d[2];
    if (e > maxe) maxe = e;
  }
  cuda_check(launch_line_passes(list, maxe, pool, s), "line_passes kernel (no-alloc)");
  ctx.launches++;
  cuda_check(cudaMemcpyAsync(h_out, p.out, sizeof(double) * n_out * batch, cudaMemcpyDeviceToHost, s), "D2H");
  cuda_check(cudaStreamSynchronize(s), "sync");
}

}  // namespace kd
