// kernels_cnn.cu - the learned SGS correction's 3-D CNN (simpleCNN, dl_models.py:19-30):
// four 3x3x3 convolutions (5 -> 32 -> 32 -> 32 -> 5 channels, zero padding, tanh-GELU between).
//
// Activations are stored channels-innermost, [z][y][x][C] in BF16, with C padded to a multiple of
// 16 for a convolution's input (the k16 of the MMA) and of 8 for its output (the n8).  Weights
// are [27 offsets][Cout][Cin] BF16 (Cin innermost), offset (dz+1)*9 + (dy+1)*3 + (dx+1).
//
//   k_conv3d       implicit GEMM on the BF16 tensor cores (mma.sync m16n8k16, FP32 accumulation):
//                  a warp owns 16 consecutive x points and every output channel; for each of the
//                  27 offsets and 16-channel slice it loads the shifted input rows as the A
//                  fragment and the weights as B.  Epilogue: + bias, optional FP32 pre-activation,
//                  optional GELU, BF16 and/or FP32 output.  The input gradient of a convolution is
//                  the same kernel run with the offsets mirrored and Cin/Cout swapped.
//   k_gelu_bwd     g = dy * GELU'(pre), to BF16 with the channel padding of the next backward conv
//   k_conv3d_dw    weight gradient dW[o][co][ci] = sum_p g[p][co] x[p+o][ci], FP32 on the CUDA
//                  cores (a small reduction: 27 * Cout * Cin outputs); each block reduces a slab of
//                  points for one offset and adds its partial sums atomically
//   k_bias_grad    db[co] = sum_p g[p][co]
//   k_adam         Adam update of FP32 master weights and their BF16 copies
//   k_sgs_pack     the network's input from the device-layout state (dl_models.py:125-155)
//   k_sgs_unpack   the scaled, re-staggered correction added to the state
//                  (one_sprint_functions.py:136-151)
#include <cuda_bf16.h>
#include <stdint.h>

#include "lexgb_cnn.cuh"

namespace lexgb {

namespace {

__device__ __forceinline__ float gelu_tanh(float x) {
  const float k0 = 0.7978845608028654f;  // sqrt(2/pi)
  return 0.5f * x * (1.f + tanhf(k0 * (x + 0.044715f * x * x * x)));
}
__device__ __forceinline__ float gelu_tanh_grad(float x) {
  const float k0 = 0.7978845608028654f;
  const float u = k0 * (x + 0.044715f * x * x * x);
  const float t = tanhf(u);
  return 0.5f * (1.f + t) + 0.5f * x * (1.f - t * t) * k0 * (1.f + 3.f * 0.044715f * x * x);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t ld32(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

// NT: output-channel tiles of 8 (Cout = 8 * NT).  One warp: 16 points x Cout.
template <int NT>
__global__ void __launch_bounds__(128) k_conv3d(int nx, int ny, int nz, int cin, const __nv_bfloat16* __restrict__ x,
                                                const __nv_bfloat16* __restrict__ w, const float* __restrict__ bias,
                                                float* __restrict__ pre, __nv_bfloat16* __restrict__ ybf,
                                                float* __restrict__ yf, int gelu, int creal) {
  constexpr int COUT = 8 * NT;
  const int lane = threadIdx.x & 31;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int rows_x = nx / 16;
  const long long ntiles = (long long)rows_x * ny * nz;
  if (warp >= ntiles) return;
  const int tx = (int)(warp % rows_x), y = (int)((warp / rows_x) % ny), z = (int)(warp / ((long long)rows_x * ny));
  const int x0 = tx * 16;
  const int g = lane >> 2, t = lane & 3;
  float acc[NT][4];
#pragma unroll
  for (int n = 0; n < NT; ++n)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[n][q] = 0.f;
  for (int off = 0; off < 27; ++off) {
    const int dz = off / 9 - 1, dy = (off / 3) % 3 - 1, dx = off % 3 - 1;
    const int zz = z + dz, yy = y + dy;
    if (zz < 0 || zz >= nz || yy < 0 || yy >= ny) continue;  // zero padding: the whole slice is 0
    const int xa = x0 + g + dx, xb = x0 + g + 8 + dx;
    const bool va = xa >= 0 && xa < nx, vb = xb >= 0 && xb < nx;
    const long long rowbase = ((long long)zz * ny + yy) * nx;
    const __nv_bfloat16* pa = x + (rowbase + (va ? xa : 0)) * cin;
    const __nv_bfloat16* pb = x + (rowbase + (vb ? xb : 0)) * cin;
    const __nv_bfloat16* wo = w + (long long)off * COUT * cin;
    for (int kc = 0; kc < cin; kc += 16) {
      uint32_t a[4];
      a[0] = va ? ld32(pa + kc + 2 * t) : 0u;
      a[1] = vb ? ld32(pb + kc + 2 * t) : 0u;
      a[2] = va ? ld32(pa + kc + 2 * t + 8) : 0u;
      a[3] = vb ? ld32(pb + kc + 2 * t + 8) : 0u;
#pragma unroll
      for (int n = 0; n < NT; ++n) {
        const __nv_bfloat16* pw = wo + (long long)(n * 8 + g) * cin + kc + 2 * t;
        uint32_t b[2] = {ld32(pw), ld32(pw + 8)};
        mma_bf16(acc[n], a, b);
      }
    }
  }
  // epilogue: rows g and g+8, channels n*8 + 2t, 2t+1
  const long long p0 = (((long long)z * ny + y) * nx + x0 + g), p1 = p0 + 8;
#pragma unroll
  for (int n = 0; n < NT; ++n) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int co = n * 8 + 2 * t + (q & 1);
      const long long p = q < 2 ? p0 : p1;
      float v = acc[n][q] + (bias ? bias[co] : 0.f);
      if (pre) pre[p * COUT + co] = v;
      if (gelu) v = gelu_tanh(v);
      if (co >= creal) v = 0.f;  // padding channels stay zero
      if (ybf) ybf[p * COUT + co] = __float2bfloat16(v);
      if (yf) yf[p * COUT + co] = v;
    }
  }
}

// g[p][c] = dy[p][c] * GELU'(pre[p][c]) for c < C (pre and dy have C channels, FP32), written
// as BF16 with Cpad >= C channels (the padding zero)
__global__ void k_gelu_bwd(long long npts, int C, int Cpad, const float* __restrict__ dy, const float* __restrict__ pre,
                           __nv_bfloat16* __restrict__ g) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npts * Cpad) return;
  const long long p = t / Cpad;
  const int c = (int)(t - p * Cpad);
  float v = 0.f;
  if (c < C) v = dy[p * C + c] * (pre ? gelu_tanh_grad(pre[p * C + c]) : 1.f);
  g[t] = __float2bfloat16(v);
}

// dW[off][co][ci] += sum over a slab of points p of g[p][co] * x[p+off][ci] (zero outside).
// Block: one offset, SLAB consecutive points, threads over (co, ci).
constexpr int SLAB = 128;  // (cin + cout) * SLAB * 4 B <= 32 KB of shared memory
__global__ void k_conv3d_dw(int nx, int ny, int nz, int cin, int cout, int gstride, const __nv_bfloat16* __restrict__ x,
                            const __nv_bfloat16* __restrict__ g, float* __restrict__ dw) {
  extern __shared__ float sm[];
  float* gs = sm;                 // [SLAB][cout]
  float* xs = sm + SLAB * cout;   // [SLAB][cin]
  const int off = blockIdx.y;
  const int dz = off / 9 - 1, dy = (off / 3) % 3 - 1, dx = off % 3 - 1;
  const long long npts = (long long)nx * ny * nz;
  const long long p0 = (long long)blockIdx.x * SLAB;
  for (int e = threadIdx.x; e < SLAB * cout; e += blockDim.x) {
    const long long p = p0 + e / cout;
    gs[e] = p < npts ? __bfloat162float(g[p * gstride + e % cout]) : 0.f;
  }
  for (int e = threadIdx.x; e < SLAB * cin; e += blockDim.x) {
    const long long p = p0 + e / cin;
    float v = 0.f;
    if (p < npts) {
      const int i = (int)(p % nx), j = (int)((p / nx) % ny), k = (int)(p / ((long long)nx * ny));
      const int ii = i + dx, jj = j + dy, kk = k + dz;
      if (ii >= 0 && ii < nx && jj >= 0 && jj < ny && kk >= 0 && kk < nz)
        v = __bfloat162float(x[(((long long)kk * ny + jj) * nx + ii) * cin + e % cin]);
    }
    xs[e] = v;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < cout * cin; e += blockDim.x) {
    const int co = e / cin, ci = e % cin;
    float acc = 0.f;
    for (int q = 0; q < SLAB; ++q) acc += gs[q * cout + co] * xs[q * cin + ci];
    atomicAdd(&dw[((long long)off * cout + co) * cin + ci], acc);
  }
}

// db[co] += sum_p g[p][co]
__global__ void k_bias_grad(long long npts, int cout, int gstride, const __nv_bfloat16* __restrict__ g,
                            float* __restrict__ db) {
  const int co = threadIdx.x % cout;
  const int lanes = blockDim.x / cout;
  float acc = 0.f;
  for (long long p = (long long)blockIdx.x * lanes + threadIdx.x / cout; p < npts; p += (long long)gridDim.x * lanes)
    acc += __bfloat162float(g[p * gstride + co]);
  if (threadIdx.x < lanes * cout) atomicAdd(&db[co], acc);
}

// Adam (bias-corrected moments) on FP32 master parameters, with an optional BF16 copy
__global__ void k_adam(long long n, float* __restrict__ w, const float* __restrict__ gw, float* __restrict__ m,
                       float* __restrict__ v, __nv_bfloat16* __restrict__ wbf, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const float gg = gw[t];
  const float mm = b1 * m[t] + (1.f - b1) * gg;
  const float vv = b2 * v[t] + (1.f - b2) * gg * gg;
  m[t] = mm;
  v[t] = vv;
  const float ww = w[t] - lr * (mm / c1) / (sqrtf(vv / c2) + eps);
  w[t] = ww;
  if (wbf) wbf[t] = __float2bfloat16(ww);
}

// Input of the network, one thread per cell, 16 BF16 channels (32 bytes):
//   (theta, ui, vi, wi, qv, 0 x 11), each (value - lo[f][k]) / rin[f][k]
// with theta = T + theta_ref and the winds averaged to the cell centre (u, v periodic).  The
// arithmetic is the element-wise sequence of the PyTorch packing of the same state, rounded
// the same way (no contractions), so both give the same BF16 inputs.
__global__ void k_sgs_pack(int nx, int ny, int nz, const float* __restrict__ T, const float* __restrict__ u,
                           const float* __restrict__ v, const float* __restrict__ w, const float* __restrict__ q,
                           float theta_ref, const float* __restrict__ lo, const float* __restrict__ rin,
                           uint4* __restrict__ x16) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long plane = (long long)nx * ny;
  if (t >= plane * nz) return;
  const int i = (int)(t % nx), j = (int)((t / nx) % ny), k = (int)(t / plane);
  const long long tu = t - i + (i + 1 == nx ? 0 : i + 1);
  const long long tv = t + (long long)((j + 1 == ny ? 0 : j + 1) - j) * nx;
  float f[5];
  f[0] = __fadd_rn(T[t], theta_ref);
  f[1] = __fmul_rn(0.5f, __fadd_rn(u[t], u[tu]));
  f[2] = __fmul_rn(0.5f, __fadd_rn(v[t], v[tv]));
  f[3] = __fmul_rn(0.5f, __fadd_rn(w[t], w[t + plane]));
  f[4] = q[t];
  __nv_bfloat16 h[6];
#pragma unroll
  for (int c = 0; c < 5; ++c) h[c] = __float2bfloat16_rn(__fdiv_rn(__fsub_rn(f[c], lo[c * nz + k]), rin[c * nz + k]));
  h[5] = __float2bfloat16_rn(0.f);
  uint4 a, b = make_uint4(0u, 0u, 0u, 0u);
  a.x = (uint32_t)__bfloat16_as_ushort(h[0]) | ((uint32_t)__bfloat16_as_ushort(h[1]) << 16);
  a.y = (uint32_t)__bfloat16_as_ushort(h[2]) | ((uint32_t)__bfloat16_as_ushort(h[3]) << 16);
  a.z = (uint32_t)__bfloat16_as_ushort(h[4]) | ((uint32_t)__bfloat16_as_ushort(h[5]) << 16);
  a.w = 0u;
  x16[2 * t] = a;
  x16[2 * t + 1] = b;
}

// The correction corr[p][0..4] (FP32, 8 channels a point) times the output range rout[f][p],
// back on the grid: theta and qv at the cell, u (v) at the west (south) face as the mean of the
// two cells beside it (periodic), w at the interior faces 1..nz-1 as the mean of the cells below
// and above (the bottom and lid faces are not corrected).  One thread per cell; it writes only
// its own cell and its own west, south and bottom faces.
__global__ void k_sgs_unpack(int nx, int ny, int nz, const float* __restrict__ corr, const float* __restrict__ rout,
                             float* __restrict__ T, float* __restrict__ u, float* __restrict__ v, float* __restrict__ w,
                             float* __restrict__ q) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long plane = (long long)nx * ny, cells = plane * nz;
  if (t >= cells) return;
  const int i = (int)(t % nx), j = (int)((t / nx) % ny), k = (int)(t / plane);
  auto c = [&](long long p, int f) { return __fmul_rn(corr[p * 8 + f], rout[f * cells + p]); };
  const long long tu = t - i + (i == 0 ? nx - 1 : i - 1);
  const long long tv = t + (long long)((j == 0 ? ny - 1 : j - 1) - j) * nx;
  T[t] = __fadd_rn(T[t], c(t, 0));
  u[t] = __fadd_rn(u[t], __fmul_rn(0.5f, __fadd_rn(c(t, 1), c(tu, 1))));
  v[t] = __fadd_rn(v[t], __fmul_rn(0.5f, __fadd_rn(c(t, 2), c(tv, 2))));
  if (k > 0) w[t] = __fadd_rn(w[t], __fmul_rn(0.5f, __fadd_rn(c(t - plane, 3), c(t, 3))));
  q[t] = __fadd_rn(q[t], c(t, 4));
}
}  // namespace

cudaError_t launch_sgs_pack(int nx, int ny, int nz, const float* T, const float* u, const float* v, const float* w,
                            const float* q, float theta_ref, const float* lo, const float* rin, void* x16,
                            cudaStream_t st) {
  const long long n = (long long)nx * ny * nz;
  k_sgs_pack<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(nx, ny, nz, T, u, v, w, q, theta_ref, lo, rin,
                                                          (uint4*)x16);
  return cudaGetLastError();
}

cudaError_t launch_sgs_unpack(int nx, int ny, int nz, const float* corr, const float* rout, float* T, float* u,
                              float* v, float* w, float* q, cudaStream_t st) {
  const long long n = (long long)nx * ny * nz;
  k_sgs_unpack<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(nx, ny, nz, corr, rout, T, u, v, w, q);
  return cudaGetLastError();
}
}  // namespace lexgb

// ------------------------------------------------------------------------------------------------
// C ABI (include/lexgb.h); device pointers, ordered on `stream` (0: the legacy default stream)
// ------------------------------------------------------------------------------------------------
namespace lexgb {
void record_error(const std::string& msg);
}

namespace {
int cnn_status(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return LEXGB_OK;
  lexgb::record_error(std::string(what) + ": " + cudaGetErrorString(e));
  return LEXGB_ERR_CUDA;
}
int cnn_arg(const char* msg) {
  lexgb::record_error(msg);
  return LEXGB_ERR_ARG;
}
}  // namespace

extern "C" int lexgb_cnn_conv3d(int nx, int ny, int nz, int cin, int cout, const void* x, const void* w,
                                const float* bias, float* pre, void* y_bf16, float* y_f32, int gelu, int creal,
                                void* stream) {
  using namespace lexgb;
  if (nx <= 0 || ny <= 0 || nz <= 0 || nx % 16) return cnn_arg("lexgb_cnn_conv3d: need nx a positive multiple of 16");
  if (cin <= 0 || cin % 16) return cnn_arg("lexgb_cnn_conv3d: cin must be a positive multiple of 16");
  if (!(cout == 8 || cout == 16 || cout == 32)) return cnn_arg("lexgb_cnn_conv3d: cout must be 8, 16 or 32");
  if (!x || !w || (!y_bf16 && !y_f32 && !pre)) return cnn_arg("lexgb_cnn_conv3d: null argument");
  const long long warps = (long long)(nx / 16) * ny * nz;
  const unsigned blocks = (unsigned)((warps + 3) / 4);
  cudaStream_t st = (cudaStream_t)stream;
  const __nv_bfloat16* xb = (const __nv_bfloat16*)x;
  const __nv_bfloat16* wb = (const __nv_bfloat16*)w;
  __nv_bfloat16* yb = (__nv_bfloat16*)y_bf16;
  if (cout == 8)
    k_conv3d<1><<<blocks, 128, 0, st>>>(nx, ny, nz, cin, xb, wb, bias, pre, yb, y_f32, gelu, creal);
  else if (cout == 16)
    k_conv3d<2><<<blocks, 128, 0, st>>>(nx, ny, nz, cin, xb, wb, bias, pre, yb, y_f32, gelu, creal);
  else
    k_conv3d<4><<<blocks, 128, 0, st>>>(nx, ny, nz, cin, xb, wb, bias, pre, yb, y_f32, gelu, creal);
  return cnn_status(cudaGetLastError(), "lexgb_cnn_conv3d");
}

extern "C" int lexgb_cnn_gelu_bwd(long long npts, int c, int cpad, const float* dy, const float* pre, void* g_bf16,
                                  void* stream) {
  using namespace lexgb;
  if (npts <= 0 || c <= 0 || cpad < c || !dy || !g_bf16) return cnn_arg("lexgb_cnn_gelu_bwd: bad argument");
  const long long n = npts * cpad;
  k_gelu_bwd<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(npts, c, cpad, dy, pre,
                                                                           (__nv_bfloat16*)g_bf16);
  return cnn_status(cudaGetLastError(), "lexgb_cnn_gelu_bwd");
}

extern "C" int lexgb_cnn_conv3d_dw(int nx, int ny, int nz, int cin, int cout, int gstride, const void* x,
                                   const void* g, float* dw, float* db, void* stream) {
  using namespace lexgb;
  if (nx <= 0 || ny <= 0 || nz <= 0 || cin <= 0 || cout <= 0 || cin > 32 || cout > 32 || 256 % cout ||
      gstride < cout || !x || !g || !dw)
    return cnn_arg("lexgb_cnn_conv3d_dw: bad argument (cin, cout <= 32, cout divides 256, gstride >= cout)");
  const long long npts = (long long)nx * ny * nz;
  cudaStream_t st = (cudaStream_t)stream;
  dim3 grid((unsigned)((npts + SLAB - 1) / SLAB), 27);
  const size_t smem = (size_t)SLAB * (cin + cout) * sizeof(float);
  k_conv3d_dw<<<grid, 256, smem, st>>>(nx, ny, nz, cin, cout, gstride, (const __nv_bfloat16*)x,
                                       (const __nv_bfloat16*)g, dw);
  if (db) k_bias_grad<<<256, 256, 0, st>>>(npts, cout, gstride, (const __nv_bfloat16*)g, db);
  return cnn_status(cudaGetLastError(), "lexgb_cnn_conv3d_dw");
}

extern "C" int lexgb_cnn_adam(long long n, float* w, const float* gw, float* m, float* v, void* w_bf16, float lr,
                              float beta1, float beta2, float eps, int step, void* stream) {
  using namespace lexgb;
  if (n <= 0 || !w || !gw || !m || !v || step < 1) return cnn_arg("lexgb_cnn_adam: bad argument");
  const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
  k_adam<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(n, w, gw, m, v, (__nv_bfloat16*)w_bf16, lr,
                                                                       beta1, beta2, eps, c1, c2);
  return cnn_status(cudaGetLastError(), "lexgb_cnn_adam");
}
