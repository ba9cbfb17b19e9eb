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
//   k_sgs_unpack   the re-staggered, scaled correction added to the state
//                  (dl_models.py:158-182, one_sprint_functions.py:136-151)
#include <cuda_bf16.h>
#include <stdint.h>

#include "lexgb_cnn.cuh"

namespace lexgb {

namespace {

__device__ __forceinline__ float gelu_tanh(float x) {
  const float k0 = 0.7978845608028654f;  // sqrt(2/pi)
  return 0.5f * x * (1.f + tanhf(k0 * (x + 0.044715f * x * x * x)));
}
// forward GELU with the hardware tanh (tanh.approx.f32, relative error about 2^-11, below the
// BF16 precision the activations are stored in)
__device__ __forceinline__ float tanh_fast(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float gelu_tanh_fast(float x) {
  const float k0 = 0.7978845608028654f;  // sqrt(2/pi)
  return 0.5f * x * (1.f + tanh_fast(k0 * (x + 0.044715f * x * x * x)));
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

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const __nv_bfloat16* p) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(a));
}
__device__ __forceinline__ void ldsm_x2(uint32_t (&r)[2], const __nv_bfloat16* p) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];" : "=r"(r[0]), "=r"(r[1]) : "r"(a));
}

// programmatic dependent launch: let the next kernel of the stream start its prologue / wait
// until the previous kernel has completed and its writes are visible (both no-ops for kernels
// launched without the programmatic-serialisation attribute)
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// 16-byte asynchronous copy global -> shared; valid = false writes zeros (no bytes read)
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, bool valid) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(sa), "l"(gmem), "r"(valid ? 16 : 0));
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Shared-memory convolution (CIN 16 or 32, COUT 8, 16 or 32): a persistent block of 12 warps
// stages the layer's weights once ([27][COUT][CIN + 8]: the 8 padding channels put the 16-byte
// rows of an 8x8 matrix in distinct banks), then loops over tiles of 16 x 8 x 1 points (x, y, z),
// staging each tile's input with its halo ([3][10][18][CIN + 8], zero outside the grid) by
// cp.async.  Warp (d, r) takes the 9 offsets of the input plane z + d - 1 for rows y0 + r and
// y0 + r + 4, 16 points each, and every output channel (one A fragment feeds COUT / 8 MMAs, one
// B fragment two); fragments are read with ldmatrix.  The three planes' partial sums meet in
// shared memory and are added in plane order.
constexpr int CONV_RP = 4, CONV_MR = 2, CONV_TY = CONV_RP * CONV_MR, CONV_WARPS = 3 * CONV_RP;

template <int CIN, int COUT>
struct ConvSmem {
  static constexpr int CP = CIN + 8;
  static constexpr int NT = COUT / 8;
  static constexpr int THREADS = 32 * CONV_WARPS;
  static constexpr int W_ELEMS = 27 * COUT * CP;
  static constexpr int A_BYTES = 3 * (CONV_TY + 2) * 18 * CP * 2;
  static constexpr int PS = COUT + 4;                          // partial-sum row stride (floats)
  static constexpr int P_BYTES = CONV_TY * 16 * PS * 4;         // [128 points][PS]
  static constexpr size_t BYTES = (size_t)W_ELEMS * 2 + (A_BYTES > P_BYTES ? A_BYTES : P_BYTES);
};

template <int CIN, int COUT>
__global__ void __launch_bounds__(ConvSmem<CIN, COUT>::THREADS)
    k_conv3d_smem(int nx, int ny, int nz, const __nv_bfloat16* __restrict__ x, const __nv_bfloat16* __restrict__ w,
                  const float* __restrict__ bias, float* __restrict__ pre, __nv_bfloat16* __restrict__ ybf,
                  float* __restrict__ yf, int gelu, int creal, int early_weights) {
  using L = ConvSmem<CIN, COUT>;
  constexpr int CP = L::CP, NT = L::NT, KC = CIN / 16, CH = CIN / 8;  // CH: 16-byte chunks a row
  extern __shared__ __align__(16) __nv_bfloat16 conv_smem[];
  __nv_bfloat16* Ws = conv_smem;
  __nv_bfloat16* As = conv_smem + L::W_ELEMS;
  float* Ps = reinterpret_cast<float*>(As);  // partial sums, after the tile's reads of As
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int dz = wid / CONV_RP, rp = wid % CONV_RP;
  // early_weights: the weights are not written by the previous kernel of the stream, so their
  // staging overlaps that kernel's tail (launched as a programmatic dependent); the input is
  // read only after pdl_wait
  pdl_launch_dependents();
  if (!early_weights) pdl_wait();
  for (int e = tid; e < 27 * COUT * CH; e += L::THREADS) {
    const int row = e / CH, c = e % CH;
    cp_async16(Ws + row * CP + c * 8, w + (long long)row * CIN + c * 8, true);
  }
  if (early_weights) pdl_wait();
  const int tiles_x = nx / 16, tiles_y = (ny + CONV_TY - 1) / CONV_TY;
  const long long ntiles = (long long)tiles_x * tiles_y * nz;
  const int g = lane >> 2, t = lane & 3;
  // ldmatrix row addresses: A (x4): matrix m = lane/8 -> rows (m & 1) * 8 + lane % 8, k half m >> 1
  const int a_row = ((lane >> 3) & 1) * 8 + (lane & 7), a_k = (lane >> 4) * 8;
  // B (x4, two n8 tiles): matrix m -> tile m >> 1, k half m & 1; (x2) matrix m -> k half m
  const int b_row = (lane >> 4) * 8 + (lane & 7), b_k = ((lane >> 3) & 1) * 8;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int tx = (int)(tile % tiles_x), ty = (int)((tile / tiles_x) % tiles_y);
    const int z = (int)(tile / ((long long)tiles_x * tiles_y));
    const int x0 = tx * 16, y0 = ty * CONV_TY;
    __syncthreads();  // the previous tile's reads of As / Ps are done
    for (int e = tid; e < 3 * (CONV_TY + 2) * 18 * CH; e += L::THREADS) {
      const int c = e % CH, q = e / CH;
      const int hx = q % 18, hy = (q / 18) % (CONV_TY + 2), hz = q / (18 * (CONV_TY + 2));
      const int xx = x0 + hx - 1, yy = y0 + hy - 1, zz = z + hz - 1;
      const bool in = xx >= 0 && xx < nx && yy >= 0 && yy < ny && zz >= 0 && zz < nz;
      cp_async16(As + q * CP + c * 8, in ? x + (((long long)zz * ny + yy) * nx + xx) * CIN + c * 8 : x, in);
    }
    cp_async_wait_all();
    __syncthreads();
    const int ya = y0 + rp, yb = ya + CONV_RP;  // the warp's two rows
    const bool plane = z + dz - 1 >= 0 && z + dz - 1 < nz;
    float acc[CONV_MR][NT][4];
#pragma unroll
    for (int m = 0; m < CONV_MR; ++m)
#pragma unroll
      for (int n = 0; n < NT; ++n)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[m][n][q] = 0.f;
    if (plane && ya < ny) {
#pragma unroll 1
      for (int dy = 0; dy < 3; ++dy) {
        const bool ina = ya + dy - 1 >= 0 && ya + dy - 1 < ny, inb = yb + dy - 1 >= 0 && yb + dy - 1 < ny;
        if (!ina && !inb) continue;
        const __nv_bfloat16* arow = As + ((dz * (CONV_TY + 2) + rp + dy) * 18) * CP;
#pragma unroll
        for (int dx = 0; dx < 3; ++dx) {
          const __nv_bfloat16* wo = Ws + ((dz * 9 + dy * 3 + dx) * COUT) * CP;
#pragma unroll
          for (int kc = 0; kc < KC; ++kc) {
            uint32_t a[CONV_MR][4];
#pragma unroll
            for (int m = 0; m < CONV_MR; ++m)
              ldsm_x4(a[m], arow + (m * CONV_RP * 18 + dx + a_row) * CP + kc * 16 + a_k);
            if constexpr (NT == 1) {
              uint32_t b[2];
              ldsm_x2(b, wo + (lane & 7) * CP + kc * 16 + ((lane >> 3) & 1) * 8);
#pragma unroll
              for (int m = 0; m < CONV_MR; ++m) mma_bf16(acc[m][0], a[m], b);
            } else {
#pragma unroll
              for (int n2 = 0; n2 < NT / 2; ++n2) {
                uint32_t b4[4];
                ldsm_x4(b4, wo + (n2 * 16 + b_row) * CP + kc * 16 + b_k);
                const uint32_t b0[2] = {b4[0], b4[1]}, b1[2] = {b4[2], b4[3]};
#pragma unroll
                for (int m = 0; m < CONV_MR; ++m) {
                  mma_bf16(acc[m][2 * n2], a[m], b0);
                  mma_bf16(acc[m][2 * n2 + 1], a[m], b1);
                }
              }
            }
          }
        }
      }
    }
    __syncthreads();  // every warp is done with As: it becomes the partial sums [point][channel]
    // planes added in order: plane 0 writes (zeros where it does not exist), 1 and 2 add
    constexpr int PS = L::PS;
#pragma unroll 1
    for (int d = 0; d < 3; ++d) {
      if (dz == d && (d == 0 || (plane && ya < ny))) {
#pragma unroll
        for (int m = 0; m < CONV_MR; ++m)
#pragma unroll
          for (int n = 0; n < NT; ++n)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              float2* pp = reinterpret_cast<float2*>(Ps + ((rp + m * CONV_RP) * 16 + g + 8 * h) * PS + n * 8 + 2 * t);
              float2 v = make_float2(acc[m][n][2 * h], acc[m][n][2 * h + 1]);
              if (d > 0) {
                const float2 o = *pp;
                v = make_float2(o.x + v.x, o.y + v.y);
              }
              *pp = v;
            }
      }
      __syncthreads();
    }
    // epilogue over the whole block: channel pairs of the tile's 128 points
    for (int e = tid; e < CONV_TY * 16 * (COUT / 2); e += L::THREADS) {
      const int pt = e / (COUT / 2), co = (e % (COUT / 2)) * 2;
      const int y = y0 + pt / 16;
      if (y >= ny) continue;
      const long long p = ((long long)z * ny + y) * nx + x0 + (pt % 16);
      const float2 sum = *reinterpret_cast<const float2*>(Ps + pt * PS + co);
      float v0 = sum.x + (bias ? bias[co] : 0.f), v1 = sum.y + (bias ? bias[co + 1] : 0.f);
      if (pre) *reinterpret_cast<float2*>(pre + p * COUT + co) = make_float2(v0, v1);
      if (gelu) {
        v0 = gelu_tanh_fast(v0);
        v1 = gelu_tanh_fast(v1);
      }
      if (co >= creal) v0 = 0.f;
      if (co + 1 >= creal) v1 = 0.f;
      if (ybf) *reinterpret_cast<__nv_bfloat162*>(ybf + p * COUT + co) = __floats2bfloat162_rn(v0, v1);
      if (yf) *reinterpret_cast<float2*>(yf + p * COUT + co) = make_float2(v0, v1);
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
// Network input of one cell, as dl_models.phys_state_tuple2array makes it (dl_models.py:125-155):
// every field is min-max normalised on its own grid points with per-level constants lo[f][l] and
// rin[f][l] (stride nz+1: w's constants are per face level 0..nz), then the normalised winds are
// averaged to the cell centre (unstagger_uvw).  16 BF16 channels, 5 used.
__global__ void k_sgs_pack(int nx, int ny, int nz, const float* __restrict__ T, const float* __restrict__ u,
                           const float* __restrict__ v, const float* __restrict__ w, const float* __restrict__ q,
                           float theta_ref, const float* __restrict__ lo, const float* __restrict__ rin,
                           uint4* __restrict__ x16) {
  pdl_launch_dependents();
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long plane = (long long)nx * ny;
  if (t >= plane * nz) return;
  const int i = (int)(t % nx), j = (int)((t / nx) % ny), k = (int)(t / plane);
  const long long tu = t - i + (i + 1 == nx ? 0 : i + 1);
  const long long tv = t + (long long)((j + 1 == ny ? 0 : j + 1) - j) * nx;
  const int L = nz + 1;
  auto nrm = [&](float x, int f, int l) { return __fdiv_rn(__fsub_rn(x, lo[f * L + l]), rin[f * L + l]); };
  float f[5];
  f[0] = nrm(__fadd_rn(T[t], theta_ref), 0, k);
  f[1] = __fmul_rn(0.5f, __fadd_rn(nrm(u[t], 1, k), nrm(u[tu], 1, k)));
  f[2] = __fmul_rn(0.5f, __fadd_rn(nrm(v[t], 2, k), nrm(v[tv], 2, k)));
  f[3] = __fmul_rn(0.5f, __fadd_rn(nrm(w[t], 3, k), nrm(w[t + plane], 3, k + 1)));
  f[4] = nrm(q[t], 4, k);
  __nv_bfloat16 h[6];
#pragma unroll
  for (int c = 0; c < 5; ++c) h[c] = __float2bfloat16_rn(f[c]);
  h[5] = __float2bfloat16_rn(0.f);
  uint4 a, b = make_uint4(0u, 0u, 0u, 0u);
  a.x = (uint32_t)__bfloat16_as_ushort(h[0]) | ((uint32_t)__bfloat16_as_ushort(h[1]) << 16);
  a.y = (uint32_t)__bfloat16_as_ushort(h[2]) | ((uint32_t)__bfloat16_as_ushort(h[3]) << 16);
  a.z = (uint32_t)__bfloat16_as_ushort(h[4]) | ((uint32_t)__bfloat16_as_ushort(h[5]) << 16);
  a.w = 0u;
  x16[2 * t] = a;
  x16[2 * t + 1] = b;
}

// The correction corr[p][0..4] (FP32, 8 channels a point) back on the grid as
// dl_models.correct_array2tuple and one_sprint_functions.py:139-151 apply it: theta and qv at the
// cell; u (v) on the west (south) face i >= 1 as the mean of the two cells beside it and on face 0
// the value of face nx-1 (stagger_uvw copies the face next to the far end onto the end face,
// dl_models.py:172-182); w on the interior faces 1..nz-1 as the mean of the cells below and above
// (bottom and lid untouched); each times the output range at its own point, rout[f][l][j][i]
// (stride nz+1 levels: cells for theta and qv, west / south faces for u / v, faces 0..nz for w).
// One thread per cell; it writes only its own cell and its own west, south and bottom faces.
__global__ void k_sgs_unpack(int nx, int ny, int nz, const float* __restrict__ corr, const float* __restrict__ rout,
                             float* __restrict__ T, float* __restrict__ u, float* __restrict__ v, float* __restrict__ w,
                             float* __restrict__ q) {
  pdl_wait();
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long plane = (long long)nx * ny, cells = plane * nz, rstride = plane * (nz + 1);
  if (t >= cells) return;
  const int i = (int)(t % nx), j = (int)((t / nx) % ny), k = (int)(t / plane);
  auto c = [&](long long p, int f) { return corr[p * 8 + f]; };
  auto r = [&](long long p, int f) { return rout[f * rstride + p]; };
  // the two cells beside the west (south) face; face 0 takes cells nx-2, nx-1 (ny-2, ny-1)
  const long long ua = i > 0 ? t - 1 : t + (nx - 2), ub = i > 0 ? t : t + (nx - 1);
  const long long va = j > 0 ? t - nx : t + (long long)(ny - 2) * nx, vb = j > 0 ? t : t + (long long)(ny - 1) * nx;
  T[t] = __fadd_rn(T[t], __fmul_rn(c(t, 0), r(t, 0)));
  u[t] = __fadd_rn(u[t], __fmul_rn(__fmul_rn(0.5f, __fadd_rn(c(ua, 1), c(ub, 1))), r(t, 1)));
  v[t] = __fadd_rn(v[t], __fmul_rn(__fmul_rn(0.5f, __fadd_rn(c(va, 2), c(vb, 2))), r(t, 2)));
  if (k > 0) w[t] = __fadd_rn(w[t], __fmul_rn(__fmul_rn(0.5f, __fadd_rn(c(t - plane, 3), c(t, 3))), r(t, 3)));
  q[t] = __fadd_rn(q[t], __fmul_rn(c(t, 4), r(t, 4)));
}
}  // namespace

// Persistent-grid size of k_conv3d_smem<CIN, COUT> (resident blocks on the current device), set
// up once per device: the dynamic shared-memory opt-in and the occupancy query are not stream
// operations, so they run here (conv_prepare) before any graph capture.
constexpr int CONV_MAX_DEVICES = 64;

template <int CIN, int COUT>
cudaError_t conv_grid(int* cap) {
  static int grid_cap[CONV_MAX_DEVICES] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= CONV_MAX_DEVICES) return cudaErrorInvalidDevice;
  if (!grid_cap[dev]) {
    using L = ConvSmem<CIN, COUT>;
    e = cudaFuncSetAttribute(k_conv3d_smem<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L::BYTES);
    if (e != cudaSuccess) return e;
    int sms = 0, per = 0;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_conv3d_smem<CIN, COUT>, L::THREADS, L::BYTES)) !=
        cudaSuccess)
      return e;
    grid_cap[dev] = sms * (per > 0 ? per : 1);
  }
  *cap = grid_cap[dev];
  return cudaSuccess;
}

// pdl: launch as a programmatic dependent of the previous kernel of the stream, staging the
// weights before waiting for it (the caller guarantees that kernel does not write them)
template <int CIN, int COUT>
cudaError_t launch_conv_smem(int nx, int ny, int nz, const __nv_bfloat16* x, const __nv_bfloat16* w,
                             const float* bias, float* pre, __nv_bfloat16* ybf, float* yf, int gelu, int creal,
                             cudaStream_t st, bool pdl) {
  int cap = 0;
  cudaError_t e = conv_grid<CIN, COUT>(&cap);
  if (e != cudaSuccess) return e;
  const long long ntiles = (long long)(nx / 16) * ((ny + CONV_TY - 1) / CONV_TY) * nz;
  using L = ConvSmem<CIN, COUT>;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(ntiles < cap ? ntiles : cap));
  cfg.blockDim = dim3(L::THREADS);
  cfg.dynamicSmemBytes = L::BYTES;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, k_conv3d_smem<CIN, COUT>, nx, ny, nz, x, w, bias, pre, ybf, yf, gelu, creal,
                            pdl ? 1 : 0);
}

// which convolution kernel launch_cnn_conv3d uses (LEXGB_CNN_AUTO: tcgen05 where the grid fits its
// 8 x 16 tiles and has at least kConvTcMinPoints points, else mma.sync); process-wide, set by
// lexgb_cnn_set_kernel
int g_conv_kernel = LEXGB_CNN_AUTO;
constexpr long long kConvTcMinPoints = 1ll << 18;   // below: too few tiles for the tcgen05 pipeline

cudaError_t launch_cnn_conv3d(int nx, int ny, int nz, int cin, int cout, const void* x, const void* w,
                              const float* bias, float* pre, void* ybf, float* yf, int gelu, int creal,
                              cudaStream_t st, bool pdl) {
  const bool big = (long long)nx * ny * nz >= kConvTcMinPoints;
  if (conv_tc_fits(nx, ny, nz, cin, cout, x, pre, ybf, yf) &&
      (g_conv_kernel == LEXGB_CNN_TCGEN05 || (g_conv_kernel == LEXGB_CNN_AUTO && big)))
    return launch_conv_tc(nx, ny, nz, cin, cout, x, w, bias, pre, ybf, yf, gelu, creal, st, pdl);
  if (g_conv_kernel == LEXGB_CNN_TCGEN05) return cudaErrorInvalidValue;
  if (!(cin == 16 || cin == 32) || !(cout == 8 || cout == 16 || cout == 32) || nx % 16) return cudaErrorInvalidValue;
  const __nv_bfloat16* xb = (const __nv_bfloat16*)x;
  const __nv_bfloat16* wb = (const __nv_bfloat16*)w;
  __nv_bfloat16* yb = (__nv_bfloat16*)ybf;
#define LEXGB_CONV(CI, CO) launch_conv_smem<CI, CO>(nx, ny, nz, xb, wb, bias, pre, yb, yf, gelu, creal, st, pdl)
  if (cin == 16) return cout == 8 ? LEXGB_CONV(16, 8) : cout == 16 ? LEXGB_CONV(16, 16) : LEXGB_CONV(16, 32);
  return cout == 8 ? LEXGB_CONV(32, 8) : cout == 16 ? LEXGB_CONV(32, 16) : LEXGB_CONV(32, 32);
#undef LEXGB_CONV
}

cudaError_t conv_prepare() {
  int cap;
  cudaError_t e;
  if ((e = conv_tc_prepare()) != cudaSuccess) return e;
  if ((e = conv_grid<16, 8>(&cap)) != cudaSuccess) return e;
  if ((e = conv_grid<16, 16>(&cap)) != cudaSuccess) return e;
  if ((e = conv_grid<16, 32>(&cap)) != cudaSuccess) return e;
  if ((e = conv_grid<32, 8>(&cap)) != cudaSuccess) return e;
  if ((e = conv_grid<32, 16>(&cap)) != cudaSuccess) return e;
  return conv_grid<32, 32>(&cap);
}

cudaError_t launch_sgs_pack(int nx, int ny, int nz, const float* T, const float* u, const float* v, const float* w,
                            const float* q, float theta_ref, const float* lo, const float* rin, void* x16,
                            cudaStream_t st) {
  const long long n = (long long)nx * ny * nz;
  k_sgs_pack<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(nx, ny, nz, T, u, v, w, q, theta_ref, lo, rin,
                                                          (uint4*)x16);
  return cudaGetLastError();
}

cudaError_t launch_sgs_unpack(int nx, int ny, int nz, const float* corr, const float* rout, float* T, float* u,
                              float* v, float* w, float* q, cudaStream_t st, bool pdl) {
  const long long n = (long long)nx * ny * nz;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)((n + 255) / 256));
  cfg.blockDim = dim3(256);
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, k_sgs_unpack, nx, ny, nz, corr, rout, T, u, v, w, q);
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
  if (cin == 16 || cin == 32)
    return cnn_status(launch_cnn_conv3d(nx, ny, nz, cin, cout, x, w, bias, pre, y_bf16, y_f32, gelu, creal, st, false),
                      "lexgb_cnn_conv3d");
  if (cout == 8)
    k_conv3d<1><<<blocks, 128, 0, st>>>(nx, ny, nz, cin, xb, wb, bias, pre, yb, y_f32, gelu, creal);
  else if (cout == 16)
    k_conv3d<2><<<blocks, 128, 0, st>>>(nx, ny, nz, cin, xb, wb, bias, pre, yb, y_f32, gelu, creal);
  else
    k_conv3d<4><<<blocks, 128, 0, st>>>(nx, ny, nz, cin, xb, wb, bias, pre, yb, y_f32, gelu, creal);
  return cnn_status(cudaGetLastError(), "lexgb_cnn_conv3d");
}

extern "C" int lexgb_cnn_set_kernel(int which) {
  using namespace lexgb;
  if (which != LEXGB_CNN_AUTO && which != LEXGB_CNN_MMA && which != LEXGB_CNN_TCGEN05)
    return cnn_arg("lexgb_cnn_set_kernel: unknown kernel");
  g_conv_kernel = which;
  return LEXGB_OK;
}

extern "C" int lexgb_cnn_take_timeouts(unsigned int* n) {
  using namespace lexgb;
  if (!n) return cnn_arg("lexgb_cnn_take_timeouts: null output");
  return cnn_status(conv_tc_take_timeouts(n), "lexgb_cnn_take_timeouts");
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
  if (g_conv_kernel != LEXGB_CNN_MMA && conv_dw_tc_fits(nx, ny, nz, cin, cout, gstride, x, g, dw)) {
    const cudaError_t e = launch_conv_dw_tc(nx, ny, nz, cin, cout, gstride, x, g, dw, st);
    if (e != cudaSuccess) return cnn_status(e, "lexgb_cnn_conv3d_dw (tcgen05)");
  } else if (g_conv_kernel == LEXGB_CNN_TCGEN05) {
    return cnn_arg("lexgb_cnn_conv3d_dw: the tcgen05 kernel needs cin 16 or 32, gstride 16 or 32, cout <= gstride "
                   "and 16-byte aligned x and g");
  } else {
    dim3 grid((unsigned)((npts + SLAB - 1) / SLAB), 27);
    const size_t smem = (size_t)SLAB * (cin + cout) * sizeof(float);
    k_conv3d_dw<<<grid, 256, smem, st>>>(nx, ny, nz, cin, cout, gstride, (const __nv_bfloat16*)x,
                                         (const __nv_bfloat16*)g, dw);
  }
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
