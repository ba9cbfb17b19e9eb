// budget_noalloc.cu - lexgb_budget_noalloc: the FP64 global budgets of lexgb_budget for callers
// that cannot allocate device memory.
//
// Who cannot allocate: code that runs where cudaMalloc is not allowed or not wanted - inside a
// host framework that owns every device byte through its own pool (an XLA/JAX custom call, a
// TensorRT or Triton-server plugin), in a path being recorded into a CUDA graph (cudaMalloc is
// not a capturable operation), or in a latency-critical loop where cudaMalloc's implicit
// device synchronisation is unacceptable.  They pass the state, the base columns and the output
// in memory they already own; the per-block partial sums go to a fixed array compiled into this
// library instead of a context allocation.
//
// Scratch: g_budget_scratch below, LEXGB_NOALLOC_MAX_BLOCKS x 4 doubles (256 KiB), present on
// every GPU that loads the library until the process exits.  One block reduces a fixed run of
// 2048 cells, so a grid may have at most 8192 * 2048 = 16,777,216 cells (e.g. 256^3); larger
// grids are rejected with LEXGB_ERR_ARG.  Every call writes each partial slot it later reads, so
// nothing has to start at zero; all calls share the one array, so calls whose kernels overlap on
// the GPU (different streams, or different threads without ordering) race and must not be
// issued concurrently.
//
// Set-up: the device address of the array is looked up with cudaGetSymbolAddress once per
// device, by the first call made while that device is current; make that first call before any
// stream capture.  The address is kept for the life of the process: after a cudaDeviceReset of a
// device (which unloads this library's device code there) the kept address no longer names the
// array, so a process that resets a device must not call lexgb_budget_noalloc on it again.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/lexgb.h"
#include "lexgb_internal.cuh"

namespace lexgb {
void record_error(const std::string& msg);
}

namespace {

using namespace lexgb;

constexpr int kThreads = 256;
constexpr int kCellsPerBlock = 2048;
constexpr int kMaxBlocks = LEXGB_NOALLOC_MAX_BLOCKS;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_budget_scratch[kMaxBlocks * 4];

std::mutex g_mu;
double* g_scratch_ptr[kMaxDevices] = {nullptr};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// same per-cell contributions as the context's budget: air mass, vapour mass, kinetic energy,
// rho0*theta (get_rho, one_step_integration.py:941-947)
__global__ void __launch_bounds__(kThreads) k_budget_fixed(Dims d, double dV, double theta_ref,
                                                         const float* __restrict__ T, const float* __restrict__ u,
                                                         const float* __restrict__ v, const float* __restrict__ w,
                                                         const float* __restrict__ p, const float* __restrict__ q,
                                                         const double* __restrict__ rho0_col,
                                                         const double* __restrict__ pi0_col,
                                                         double* __restrict__ partial) {
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  const long long n = d.cells();
  const long long begin = (long long)blockIdx.x * kCellsPerBlock;
  const long long end = begin + kCellsPerBlock < n ? begin + kCellsPerBlock : n;
  for (long long t = begin + threadIdx.x; t < end; t += kThreads) {
    const int i = (int)(t % d.nx);
    const int j = (int)((t / d.nx) % d.ny);
    const int k = (int)(t / ((long long)d.nx * d.ny));
    const double th = theta_ref + (double)T[t];
    const double qv = (double)q[t];
    const double pi = pi0_col[k + 1] + (double)p[t];
    const double pr = pow(pi, kCp / kRd) * kP00;
    const double rho = pr / kRd / ((1.0 + kRepsm1 * qv) * (pi * th));
    const double r0 = rho0_col[k + 1];
    const double uc = 0.5 * ((double)u[t] + (double)u[d.at(wrap(i + 1, d.nx), j, k)]);
    const double vc = 0.5 * ((double)v[t] + (double)v[d.at(i, wrap(j + 1, d.ny), k)]);
    const double wc = 0.5 * ((double)w[t] + (double)w[d.at(i, j, k + 1)]);
    acc[0] += rho * dV;
    acc[1] += rho * qv * dV;
    acc[2] += 0.5 * r0 * (uc * uc + vc * vc + wc * wc) * dV;
    acc[3] += r0 * th * dV;
  }
  __shared__ double sm[4][kThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    const double s = warp_sum(acc[m]);
    if (lane == 0) sm[m][wid] = s;
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      double s = lane < kThreads / 32 ? sm[m][lane] : 0.0;
      s = warp_sum(s);
      if (lane == 0) partial[blockIdx.x * 4 + m] = s;
    }
  }
}

__global__ void __launch_bounds__(kThreads) k_budget_sum(int nblocks, const double* __restrict__ partial,
                                                       double* __restrict__ out) {
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int b = threadIdx.x; b < nblocks; b += kThreads)
#pragma unroll
    for (int m = 0; m < 4; ++m) acc[m] += partial[b * 4 + m];
  __shared__ double sm[4][kThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    const double s = warp_sum(acc[m]);
    if (lane == 0) sm[m][wid] = s;
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      double s = lane < kThreads / 32 ? sm[m][lane] : 0.0;
      s = warp_sum(s);
      if (lane == 0) out[m] = s;
    }
  }
}

// device address of g_budget_scratch for the current device (looked up once per device)
int scratch_for_current_device(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    record_error(std::string("lexgb_budget_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
    return LEXGB_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    record_error("lexgb_budget_noalloc: device index out of range");
    return LEXGB_ERR_ARG;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_budget_scratch);
    if (e != cudaSuccess || !ptr) {
      record_error(std::string("lexgb_budget_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      return LEXGB_ERR_CUDA;
    }
    g_scratch_ptr[dev] = static_cast<double*>(ptr);
  }
  *out = g_scratch_ptr[dev];
  return LEXGB_OK;
}

}  // namespace

extern "C" int lexgb_budget_noalloc(int nx, int ny, int nz, double dx, double dy, double dz, double theta_ref,
                                    const float* const fields[6], const double* rho0_col, const double* pi0_col,
                                    double* out, void* stream) {
  if (nx < 4 || ny < 4 || nz < 6) {
    record_error("lexgb_budget_noalloc: grid too small: need nx, ny >= 4 and nz >= 6");
    return LEXGB_ERR_ARG;
  }
  if (!fields || !rho0_col || !pi0_col || !out) {
    record_error("lexgb_budget_noalloc: null argument");
    return LEXGB_ERR_ARG;
  }
  for (int f = 0; f < 6; ++f)
    if (!fields[f]) {
      record_error("lexgb_budget_noalloc: null field pointer");
      return LEXGB_ERR_ARG;
    }
  const long long cells = (long long)nx * ny * nz;
  const long long nblocks = (cells + kCellsPerBlock - 1) / kCellsPerBlock;
  if (nblocks > kMaxBlocks || (long long)nx * ny * (nz + 1) >= (1LL << 31)) {
    record_error("lexgb_budget_noalloc: " + std::to_string(cells) + " cells exceed the maximum of " +
                 std::to_string((long long)kMaxBlocks * kCellsPerBlock) +
                 " cells that its fixed scratch array (LEXGB_NOALLOC_MAX_BLOCKS partial sums) can reduce");
    return LEXGB_ERR_ARG;
  }
  double* scratch = nullptr;
  const int s = scratch_for_current_device(&scratch);
  if (s != LEXGB_OK) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const Dims d{nx, ny, nz};
  k_budget_fixed<<<(unsigned)nblocks, kThreads, 0, st>>>(d, dx * dy * dz, theta_ref, fields[0], fields[1],
                                                        fields[2], fields[3], fields[4], fields[5], rho0_col,
                                                        pi0_col, scratch);
  k_budget_sum<<<1, kThreads, 0, st>>>((int)nblocks, scratch, out);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    record_error(std::string("lexgb_budget_noalloc: launch: ") + cudaGetErrorString(e));
    return LEXGB_ERR_CUDA;
  }
  return LEXGB_OK;
}
