// fhp_energy_matrix_noalloc: the A_H energy matrix of fields and a coefficient
// on one grid, in a single kernel launch whose block partial sums live in a
// fixed scratch array of this translation unit.  Nothing is allocated per
// call, per plan or per device: the scratch is a static device array that
// exists once the library's module is loaded.
//
// Callers this serves: code whose device memory is owned by another allocator
// (a framework's caching allocator, or a pool reserved up front to the limit of
// HBM), where a cudaMalloc from inside the library fails or stalls the device,
// and loops that must not synchronise with the host.
//
// Limits: loads <= 6 and dv <= 6 (36 accumulators per block), at most
// kNoAllocMaxBlocks blocks; the scratch is shared by every call on a device, so
// calls that overlap in time on one device race and must be serialised by the
// caller.  Every call looks up the scratch's device address (no allocation);
// the first call on a device also loads the kernels and should come before
// any stream capture.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "../../include/ffthompy_gb300.h"
#include "fhp_engine.h"
#include "fhp_kernels.cuh"

namespace {

constexpr int kNoAllocMaxBlocks = 1024;
constexpr int kNoAllocHeader = 32;  // doubles (256 bytes): the block ticket counter
constexpr int kNoAllocAcc = fhp::kMaxLoads * fhp::kMaxLoads;
constexpr size_t kNoAllocScratchDoubles =
    kNoAllocHeader + (size_t)kNoAllocMaxBlocks * kNoAllocAcc;  // 36,896 doubles = 288.25 KiB
constexpr int kNoAllocThreads = 128;
constexpr int kMaxDevices = 64;

}  // namespace

// [0, 256 B): unsigned ticket counter, must be zero when a launch starts (the
// entry point clears it on the stream before each launch);
// [256 B, ...): per-block partial sums, each written before it is read.
static __device__ __align__(256) double fhp_noalloc_scratch[kNoAllocScratchDoubles];

namespace {

// A_H partials per block (the sum of k_energy), then the last block to finish
// adds the partials of all blocks in block order and writes AH.
template <int COEF>
__global__ void __launch_bounds__(kNoAllocThreads)
    k_energy_oneshot(const double* __restrict__ X, const double* __restrict__ A,
                     fhp::GridDims g, int add_macro, double scale, double* scratch,
                     double* __restrict__ AH) {
  using namespace fhp;
  __shared__ double red[(kNoAllocThreads / 32) * kNoAllocAcc];
  __shared__ int is_last;
  const int L = g.L, dv = g.dv, n = L * L;
  double acc[kNoAllocAcc];
  for (int i = 0; i < kNoAllocAcc; ++i) acc[i] = 0.;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < g.M; v += stride) {
    double u[kMaxLoads][kMaxDv];
    for (int l = 0; l < L; ++l)
      for (int c = 0; c < dv; ++c)
        u[l][c] = X[(long long)(l * dv + c) * g.M + v] + ((add_macro && c == l) ? 1. : 0.);
    for (int i = 0; i < L; ++i) {
      double q[kMaxDv];
      coef_apply<double, COEF>(A, g.M, v, dv, u[i], q);
      for (int j = 0; j < L; ++j) {
        double s = 0.;
        for (int c = 0; c < dv; ++c) s += q[c] * u[j][c];
        acc[i * L + j] += s;
      }
    }
  }
  double* partials = scratch + kNoAllocHeader;
  block_sum_n(acc, n, red, partials + (long long)blockIdx.x * n);
  // publish this block's partials before taking a ticket
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned int* ticket = reinterpret_cast<unsigned int*>(scratch);
    is_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  if (threadIdx.x < n) {
    double s = 0.;
    for (unsigned int b = 0; b < gridDim.x; ++b)
      s += __ldcg(partials + (long long)b * n + threadIdx.x);
    AH[threadIdx.x] = s * scale;
  }
}

struct DeviceScratch {
  bool ready = false;
  double* ptr = nullptr;
  int nsm = 0;
};

std::mutex g_setup_mu;
DeviceScratch g_setup[kMaxDevices];

int fail(int status, const char* msg) {
  fhp::set_error(msg);
  return status;
}

// Once per device, with that device current: the SM count and the kernels
// loaded.  The scratch's device address is looked up on every call (no
// allocation, and a cached address would go stale if the device's primary
// context were reset and created again).
int scratch_for_current_device(DeviceScratch& out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return fail(FHP_CUDA, "cudaGetDevice failed");
  if (dev < 0 || dev >= kMaxDevices) return fail(FHP_BAD_ARG, "device index beyond 63");
  double* p = nullptr;
  cudaError_t ea = cudaGetSymbolAddress((void**)&p, fhp_noalloc_scratch);
  if (ea != cudaSuccess) {
    fhp::set_error(std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(ea));
    return FHP_CUDA;
  }
  std::lock_guard<std::mutex> g(g_setup_mu);
  DeviceScratch& d = g_setup[dev];
  if (!d.ready) {
    int nsm = 0;
    cudaError_t e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaFuncAttributes fa;
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_energy_oneshot<fhp::COEF_ISO>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_energy_oneshot<fhp::COEF_SYM>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_energy_oneshot<fhp::COEF_FULL>);
    if (e != cudaSuccess) {
      fhp::set_error(std::string("no-alloc energy set-up: ") + cudaGetErrorString(e));
      return FHP_CUDA;
    }
    d.nsm = nsm > 0 ? nsm : 1;
    d.ready = true;
  }
  d.ptr = p;
  out = d;
  return FHP_OK;
}

}  // namespace

extern "C" int fhp_energy_matrix_noalloc(int dim, const int* n, int dv, int loads, int kind,
                                         const double* A, const double* X, int add_macro,
                                         double* AH, void* stream) {
  if (dim != 2 && dim != 3) return fail(FHP_BAD_ARG, "dim must be 2 or 3");
  if (!n || !A || !X || !AH) return fail(FHP_BAD_ARG, "n, A, X and AH are required");
  if (loads < 1 || loads > fhp::kMaxLoads)
    return fail(FHP_BAD_ARG,
                "loads must be in 1..6: the fixed scratch holds 6 x 6 accumulators per block");
  if (dv < 1 || dv > fhp::kMaxDv) return fail(FHP_BAD_ARG, "dv must be in 1..6");
  if (kind != FHP_COEF_ISO && kind != FHP_COEF_SYM && kind != FHP_COEF_FULL)
    return fail(FHP_BAD_ARG, "kind must be FHP_COEF_ISO, FHP_COEF_SYM or FHP_COEF_FULL");
  long long M = 1;
  for (int i = 0; i < dim; ++i) {
    if (n[i] < 1) return fail(FHP_BAD_ARG, "grid sizes must be positive");
    M *= n[i];
  }
  DeviceScratch d;
  int st = scratch_for_current_device(d);
  if (st != FHP_OK) return st;
  fhp::GridDims g{};
  g.dim = dim;
  g.n0 = dim == 3 ? n[0] : 1;
  g.n1 = n[dim - 2];
  g.n2 = n[dim - 1];
  g.n2h = g.n2 / 2 + 1;
  g.dv = dv;
  g.L = loads;
  g.M = M;
  long long nb = (M + kNoAllocThreads - 1) / kNoAllocThreads;
  nb = std::min<long long>(nb, std::min<long long>(4LL * d.nsm, kNoAllocMaxBlocks));
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(d.ptr, 0, kNoAllocHeader * sizeof(double), s);
  if (e != cudaSuccess) {
    fhp::set_error(std::string("clearing the ticket: ") + cudaGetErrorString(e));
    return FHP_CUDA;
  }
  const double scale = 1.0 / (double)M;
  switch (kind) {
    case FHP_COEF_ISO:
      k_energy_oneshot<fhp::COEF_ISO><<<(unsigned)nb, kNoAllocThreads, 0, s>>>(X, A, g, add_macro,
                                                                             scale, d.ptr, AH);
      break;
    case FHP_COEF_SYM:
      k_energy_oneshot<fhp::COEF_SYM><<<(unsigned)nb, kNoAllocThreads, 0, s>>>(X, A, g, add_macro,
                                                                             scale, d.ptr, AH);
      break;
    default:
      k_energy_oneshot<fhp::COEF_FULL><<<(unsigned)nb, kNoAllocThreads, 0, s>>>(X, A, g, add_macro,
                                                                              scale, d.ptr, AH);
      break;
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    fhp::set_error(std::string("no-alloc energy launch: ") + cudaGetErrorString(e));
    return FHP_CUDA;
  }
  return FHP_OK;
}
