// kernels_cnn_tc.cu - the learned SGS correction's 3x3x3 convolution on the 5th-generation tensor
// cores (tcgen05.mma, accumulators in tensor memory), as an implicit GEMM per tile of points, one
// input plane at a time:
//
//   D[128 points][3 NP] += A[128 points][Cin] (input plane p shifted by (dy, dx))
//                          x B[Cin][3 NP]     (the weights of the taps (dz, dy, dx), dz = -1, 0, +1)
//
// so that one MMA adds plane p's share to the three output levels it feeds (p+1, p, p-1): each
// input tile is read by the tensor cores 9 x Cin/16 times per plane instead of 27 x Cin/16.
// A block owns a column of 8 (x) x 16 (y) points and marches up a chunk of levels, with its
// warps specialised:
//   warp 4 (producer)  loads each input plane the chunk needs (10 x 18 points with the one-point
//                      halo, zero outside the grid by the tensor map's out-of-bounds fill) by TMA
//                      (cp.async.bulk.tensor, one box per 8-channel group) into a ring of plane
//                      slots; a slot's full barrier completes on the bytes' arrival;
//   warp 5 (MMA)       for plane p issues the 9 x Cin/16 MMAs (M = 128, N = 3 NP, K = 16, BF16
//                      in, FP32 accumulate) into the columns of output levels p+1, p, p-1: the
//                      tensor memory is a ring of Q level slots of NP columns in descending level
//                      order, so the three are adjacent (where they wrap round the ring, the MMA
//                      is split in two; never in a chunk of at most Q - 5 levels); it frees the
//                      plane's slot and marks level p-1 summed;
//   warps 0-3          (the four tensor-memory lane quarters) zero the ring first (the windows of
//                      neighbouring planes overlap, so every MMA accumulates), then for each level
//                      wait for it, read their 32 rows (tcgen05.ld), zero the level slot again if
//                      a later level of the chunk uses it, hand it back to the MMA warp and apply
//                      the epilogue of k_conv3d_smem (bias, FP32 pre-activation, GELU, padding
//                      channels zero, BF16 / FP32 output).
// Every wait is bounded: one that gives up counts a timeout in g_tc_timeouts and sets the block's
// abort flag, which ends the other roles' waits; the block then waits (bounded) for the MMAs it
// issued and the copies in flight, frees its tensor memory and returns.
//
// Shared-memory layouts (16-byte pieces; the tensor cores' canonical K-major layout without
// swizzle, core matrix = 8 rows of 16 bytes):
//   weights  Wsm[9][CIN/8][3 NP][8]        (dy dx), input group, row t NP + co of tap (t - 1, dy,
//                                          dx) and output channel co; core matrix = 8 rows x 8
//                                          inputs; K step 3 NP x 16 B (LBO), next 8 rows 128 B (SBO)
//   planes   Psm[R][CIN/8][18][10][8]      slot, channel group (its box padded to 128-byte
//                                          alignment), row, x; core matrix = 8 consecutive x
//                                          points; K step = the next channel group's box (LBO),
//                                          next row of the tile 160 B (SBO)
#include <cuda.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include "lexgb_cnn.cuh"

namespace lexgb {

__device__ unsigned int g_tc_timeouts = 0;   // bounded waits of k_conv3d_tc that gave up

namespace {

constexpr int TC_TX = 8, TC_TY = 16, TC_HX = TC_TX + 2, TC_HY = TC_TY + 2;
constexpr int TC_THREADS = 192;               // 4 epilogue warps, the producer, the MMA warp
constexpr long long TC_POLLS = 1ll << 24;     // mbarrier polls before a wait gives up
constexpr int TC_BOX_BYTES = TC_HY * TC_HX * 16;                  // one channel group's box: 2880
constexpr int TC_GROUP_BYTES = (TC_BOX_BYTES + 127) / 128 * 128;  // padded to 128 bytes: 2944

template <int CIN, int COUT>
struct TcLayout {
  static constexpr int NP = COUT < 16 ? 16 : COUT;  // output channels of one level in N (16 or 32)
  static constexpr int N3 = 3 * NP;                 // N of the MMA: output levels p+1, p, p-1
  static constexpr int CG = CIN / 8;                // channel groups of 8 (16 bytes)
  static constexpr int R = 4;                       // plane slots (each plane is read once)
  static constexpr int TMEM_COLS = 256;             // two blocks per SM
  static constexpr int Q = TMEM_COLS / NP;          // level slots of NP columns (8 or 16)
  static constexpr int W_BYTES = 9 * CG * N3 * 16;
  static constexpr int PLANE_BYTES = CG * TC_GROUP_BYTES;
  static constexpr int P_BYTES = R * PLANE_BYTES;
  static constexpr int A_LBO = TC_GROUP_BYTES;      // next channel group
  static constexpr int A_SBO = TC_HX * 16;          // next row of the tile (8 points on)
  static constexpr int B_LBO = N3 * 16;             // next input-channel group
  static constexpr int B_SBO = 128;                 // next 8 rows of N
  static constexpr int EPI = 4;                     // epilogue warps (one per tensor-memory lane quarter)
  static constexpr int THREADS = 32 * (EPI + 2);    // + the producer and the MMA warp
  static constexpr int NBAR = 2 * R + 2 * Q + 1;    // full[R], empty[R], summed[Q], freed[Q], done
  static constexpr int BAR_BYTES = NBAR * 8 + 16;
  // + alignment slack, barriers, tensor-memory address, abort flag, bias; at least 80 KB, so that
  // no more blocks share an SM than its tensor memory holds
  static constexpr size_t NEED = 128 + (size_t)W_BYTES + P_BYTES + BAR_BYTES + NP * 4;
  static constexpr size_t BYTES = NEED < 80 * 1024 ? 80 * 1024 : NEED;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void cp16(uint32_t dst, const void* src, bool valid) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(valid ? 16 : 0));
}

// canonical K-major, no-swizzle shared-memory matrix descriptor
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= 1ull << 46;  // descriptor version
  return d;         // base offset 0, swizzle none
}

// instruction descriptor of kind::f16: D FP32, A and B BF16, both K-major, M x N
__host__ __device__ constexpr uint32_t tc_idesc(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16_tc(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                            uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// Bounded wait for phase `parity` of an mbarrier; gives up early when the block's abort flag is set.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, const volatile int* abort) {
  for (long long i = 0; i < TC_POLLS; ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if ((i & 1023) == 1023 && *abort) return false;
  }
  return false;
}

// Bounded wait with a back-off between polls (about a second at most), for the warps that wait out
// the whole of a block's work; gives up early when the block's abort flag is set (if checked).
__device__ __forceinline__ bool mbar_wait_long(uint32_t bar, uint32_t parity, const volatile int* abort) {
  for (long long i = 0; i < (1ll << 22); ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if (abort && *abort) return false;
    __nanosleep(256);
  }
  return false;
}

// a 4-D box (channel, x, y, z) of a tensor map into shared memory, completing on an mbarrier
__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap* map, int c, int x, int y, int z,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
      "%5}], [%6];" ::"r"(dst),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(c), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}

__device__ __forceinline__ float gelu_fast(float x) {
  const float k0 = 0.7978845608028654f;  // sqrt(2/pi)
  float t;
  asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(k0 * (x + 0.044715f * x * x * x)));
  return 0.5f * x * (1.f + t);
}

__device__ __forceinline__ void tmem_load16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}


__device__ __forceinline__ void tmem_zero16(uint32_t taddr) {
  const uint32_t z = 0;
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1};" ::"r"(taddr),
      "r"(z)
      : "memory");
}
__device__ __forceinline__ void tmem_zero8(uint32_t taddr) {
  const uint32_t z = 0;
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%1,%1,%1,%1,%1,%1,%1};" ::"r"(taddr), "r"(z)
               : "memory");
}
__device__ __forceinline__ void tmem_load8(uint32_t taddr, float* v) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}
// CW consecutive columns of this warp's lanes: load / zero
template <int CW>
__device__ __forceinline__ void tmem_load_cols(uint32_t taddr, float* v) {
#pragma unroll
  for (int c = 0; c < CW; c += 16) {
    if (CW - c >= 16) tmem_load16(taddr + (uint32_t)c, v + c);
    else tmem_load8(taddr + (uint32_t)c, v + c);
  }
}
template <int CW>
__device__ __forceinline__ void tmem_zero_cols(uint32_t taddr) {
#pragma unroll
  for (int c = 0; c < CW; c += 16) {
    if (CW - c >= 16) tmem_zero16(taddr + (uint32_t)c);
    else tmem_zero8(taddr + (uint32_t)c);
  }
}

template <int CIN, int COUT>
__global__ void __launch_bounds__(TcLayout<CIN, COUT>::THREADS, 1)
    k_conv3d_tc(const __grid_constant__ CUtensorMap xmap, int nx, int ny, int nz, int zc,
                const __nv_bfloat16* __restrict__ w, const float* __restrict__ bias, float* __restrict__ pre,
                __nv_bfloat16* __restrict__ ybf, float* __restrict__ yf, int gelu, int creal, int early_weights) {
  using L = TcLayout<CIN, COUT>;
  constexpr int NP = L::NP, N3 = L::N3, CG = L::CG, R = L::R, Q = L::Q, EPI = L::EPI;
  constexpr int H = EPI / 4, CW = NP / H;   // channel parts of a level; columns of one part
  extern __shared__ unsigned char tc_raw[];
  const uint32_t raw_s = smem_u32(tc_raw);
  unsigned char* smem = tc_raw + ((128u - (raw_s & 127u)) & 127u);   // 128-byte aligned for TMA
  const uint32_t w_s = smem_u32(smem), p_s = w_s + L::W_BYTES, bar_s = p_s + L::P_BYTES;
  auto full = [&](int s) { return bar_s + 8u * s; };
  auto empty = [&](int s) { return bar_s + 8u * (R + s); };
  auto summed = [&](int q) { return bar_s + 8u * (2 * R + q); };       // a level slot's sums are complete
  auto freed = [&](int q) { return bar_s + 8u * (2 * R + Q + q); };    // ... read (and zeroed if reused)
  const uint32_t done = bar_s + 8u * (2 * R + 2 * Q);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + L::W_BYTES + L::P_BYTES + L::NBAR * 8);
  volatile int* abort = reinterpret_cast<volatile int*>(tslot + 1);
  float* bsm = reinterpret_cast<float*>(smem + L::W_BYTES + L::P_BYTES + L::BAR_BYTES);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (warp == EPI + 1) {  // tensor memory: Q level slots of NP columns
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(L::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < R; ++s) {
      mbar_init(full(s), 1);
      mbar_init(empty(s), 1);
    }
    for (int q = 0; q < Q; ++q) {
      mbar_init(summed(q), 1);
      mbar_init(freed(q), EPI);
    }
    mbar_init(done, 1);
    *abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // weights Wsm[dy dx][cg][n][8] from w[tap][COUT][CIN]: row n = t NP + co holds the tap
  // (dz = t - 1, dy, dx) of output channel co (rows co >= COUT zero), so that one MMA on input
  // plane p adds to output levels p+1 (t = 0), p (t = 1) and p-1 (t = 2)
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  if (!early_weights) asm volatile("griddepcontrol.wait;" ::: "memory");
  for (int e = tid; e < 9 * CG * N3; e += L::THREADS) {
    const int n = e % N3, cg = (e / N3) % CG, yx = e / (N3 * CG);
    const int t = n / NP, co = n % NP;
    const bool ok = co < COUT;
    const int tap = t * 9 + yx;
    cp16(w_s + (uint32_t)e * 16u, w + ((long long)(tap * COUT + (ok ? co : 0)) * CIN + cg * 8), ok);
  }
  if (tid < NP) bsm[tid] = (bias && tid < COUT) ? bias[tid] : 0.f;
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  // epilogue warp w: lanes 32 (w % 4) .., channels CW (w / 4) .. of every level
  const uint32_t lanes = (uint32_t)(32 * (warp & 3)) << 16;
  const int part = (warp >> 2) * CW;
  // the MMA windows of neighbouring planes overlap, so they all accumulate: zero the slots first
  if (warp < EPI) {
    for (int q = 0; q < Q; ++q) tmem_zero_cols<CW>(tmem + lanes + (uint32_t)(q * NP + part));
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
  }
  asm volatile("cp.async.wait_all;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // weights -> the tensor cores
  if (early_weights) asm volatile("griddepcontrol.wait;" ::: "memory");   // the input is ready
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

  const int tiles_x = nx / TC_TX, tiles_y = ny / TC_TY;
  const int tx = blockIdx.x % tiles_x, ty = (blockIdx.x / tiles_x) % tiles_y, ch = blockIdx.x / (tiles_x * tiles_y);
  const int x0 = tx * TC_TX, y0 = ty * TC_TY, z0 = ch * zc, z1 = min(z0 + zc, nz);
  const int p0 = z0 - 1;   // first plane of the chunk; plane p uses slot (p - p0) % R, fill (p - p0) / R
  // Output level z (z0 - 2 .. z1 + 1; the four outside z0 .. z1 - 1 are scratch that the planes at
  // the chunk's ends add to) lives in level slot Q - 1 - (z - z0 + 2) mod Q, its (z - z0 + 2) / Q-th
  // use: the slots of levels p+1, p, p-1 follow one another except where they wrap round (never in
  // a chunk of at most Q - 5 levels).
  const int zb = z0 - 2;
  auto lslot = [&](int z) { return Q - 1 - (z - zb) % Q; };
  auto luse = [&](int z) { return (z - zb) / Q; };

  if (warp == EPI) {
    // ---------------- producer: planes z0-1 .. z1 ----------------
    if (lane == 0) {
      int p = p0;
      for (; p <= z1; ++p) {
        const int s = (p - p0) % R, k = (p - p0) / R;
        if (k > 0 && !mbar_wait(empty(s), (k - 1) & 1, abort)) {
          atomicAdd(&g_tc_timeouts, 1u);
          *abort = 1;
          break;
        }
        mbar_expect_tx(full(s), CG * TC_BOX_BYTES);
        for (int cg = 0; cg < CG; ++cg)
          tma_load_4d(p_s + s * L::PLANE_BYTES + cg * TC_GROUP_BYTES, &xmap, cg * 8, x0 - 1, y0 - 1, p, full(s));
      }
      // the copies this thread issued have landed before the block's memory goes (bounded)
      for (int q = p - 1; q >= p0 && q >= p - R; --q) mbar_wait_long(full((q - p0) % R), ((q - p0) / R) & 1, nullptr);
    }
  } else if (warp == EPI + 1) {
    // ---------------- MMA issuer: one plane at a time ----------------
    if (lane == 0) {
      // descriptors: the start address is the low field (16-byte units), so an operand at a fixed
      // offset from a base is the base's descriptor plus the offset / 16
      const uint64_t b0 = smem_desc(w_s, L::B_LBO, L::B_SBO);
      bool ok = true;
      for (int p = p0; p <= z1 && ok; ++p) {
        const int s = (p - p0) % R, k = (p - p0) / R;
        ok = mbar_wait(full(s), k & 1, abort);
        // level p+1 is new in its slot: the level that used the slot before has been read and zeroed
        if (ok && luse(p + 1) > 0) ok = mbar_wait(freed(lslot(p + 1)), (luse(p + 1) - 1) & 1, abort);
        if (!ok) {
          atomicAdd(&g_tc_timeouts, 1u);
          *abort = 1;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int q0 = lslot(p + 1);   // slots q0, q0 + 1, q0 + 2 (mod Q) <- t = 0, 1, 2
        // the rows t < split go to columns q0 NP.., the rest to column 0 (the window wraps)
        const int split = q0 + 3 <= Q ? 3 : Q - q0;
        const uint32_t c_hi = tmem + (uint32_t)(q0 * NP), c_lo = tmem;
        const uint64_t a0 = smem_desc(p_s + s * L::PLANE_BYTES, L::A_LBO, L::A_SBO);
#pragma unroll
        for (int dy = 0; dy < 3; ++dy)
#pragma unroll
          for (int dx = 0; dx < 3; ++dx)
#pragma unroll
            for (int ks = 0; ks < CIN / 16; ++ks) {
              const uint64_t ad = a0 + (uint64_t)((2 * ks * TC_GROUP_BYTES + (dy * TC_HX + dx) * 16) >> 4);
              const uint64_t bd = b0 + (uint64_t)((((dy * 3 + dx) * CG + 2 * ks) * N3 * 16) >> 4);
              if (split == 3) {
                mma_bf16_tc(c_hi, ad, bd, tc_idesc(128, N3), 1u);
              } else if (split == 2) {
                mma_bf16_tc(c_hi, ad, bd, tc_idesc(128, 2 * NP), 1u);
                mma_bf16_tc(c_lo, ad, bd + (uint64_t)((2 * NP * 16) >> 4), tc_idesc(128, NP), 1u);
              } else {
                mma_bf16_tc(c_hi, ad, bd, tc_idesc(128, NP), 1u);
                mma_bf16_tc(c_lo, ad, bd + (uint64_t)((NP * 16) >> 4), tc_idesc(128, 2 * NP), 1u);
              }
            }
        mma_commit(empty(s));               // plane p is not read again
        mma_commit(summed(lslot(p - 1)));   // level p-1 has all three of its planes
      }
      mma_commit(done);
      mbar_wait_long(done, 0, nullptr);   // the MMAs are complete before the tensor memory goes
    }
  } else {
    // ---------------- epilogue: warps 0 .. EPI-1 ----------------
    const int r = 32 * (warp & 3) + lane;   // row r <-> point (x0 + r % 8, y0 + r / 8)
    for (int z = zb; z < z1; ++z) {
      const int q = lslot(z);
      if (!__all_sync(0xffffffffu, mbar_wait(summed(q), luse(z) & 1, abort))) {   // warp-uniform
        if (lane == 0) {
          atomicAdd(&g_tc_timeouts, 1u);
          *abort = 1;
        }
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      float v[CW];
      const bool real = z >= z0;
      const uint32_t cols = tmem + lanes + (uint32_t)(q * NP + part);
      if (real) {
        tmem_load_cols<CW>(cols, v);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      }
      if (z + Q <= z1 + 1) {   // the slot's next level is in this chunk: zero it for that level
        tmem_zero_cols<CW>(cols);
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(freed(q));
      if (!real || part >= COUT) continue;
      // the point's channels part .. part + CW - 1 (those below COUT) as 16-byte stores
      const long long p = ((long long)z * ny + y0 + r / TC_TX) * nx + x0 + r % TC_TX;
      constexpr int CN = CW < COUT ? CW : COUT;   // channels of this part below COUT (COUT % CW == 0 or COUT < CW)
#pragma unroll
      for (int c = 0; c < CN; ++c) v[c] += bsm[part + c];
      if (pre) {
#pragma unroll
        for (int c = 0; c < CN; c += 4)
          *reinterpret_cast<float4*>(pre + p * COUT + part + c) = make_float4(v[c], v[c + 1], v[c + 2], v[c + 3]);
      }
#pragma unroll
      for (int c = 0; c < CN; ++c) {
        const float t = gelu ? gelu_fast(v[c]) : v[c];
        v[c] = part + c < creal ? t : 0.f;
      }
      if (ybf) {
#pragma unroll
        for (int c = 0; c < CN; c += 8) {
          uint4 qq;
          __nv_bfloat162 h0 = __floats2bfloat162_rn(v[c], v[c + 1]);
          __nv_bfloat162 h1 = __floats2bfloat162_rn(v[c + 2], v[c + 3]);
          __nv_bfloat162 h2 = __floats2bfloat162_rn(v[c + 4], v[c + 5]);
          __nv_bfloat162 h3 = __floats2bfloat162_rn(v[c + 6], v[c + 7]);
          qq.x = *reinterpret_cast<uint32_t*>(&h0);
          qq.y = *reinterpret_cast<uint32_t*>(&h1);
          qq.z = *reinterpret_cast<uint32_t*>(&h2);
          qq.w = *reinterpret_cast<uint32_t*>(&h3);
          *reinterpret_cast<uint4*>(ybf + p * COUT + part + c) = qq;
        }
      }
      if (yf) {
#pragma unroll
        for (int c = 0; c < CN; c += 4)
          *reinterpret_cast<float4*>(yf + p * COUT + part + c) = make_float4(v[c], v[c + 1], v[c + 2], v[c + 3]);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == EPI + 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(L::TMEM_COLS) : "memory");
  }
}

// ---------------------------------------------------------------------------------------------
// Weight gradient on the tensor cores:
//
//   dW[tap][co][ci] += sum over points p of g[p][co] x[p + off(tap)][ci]
//
// as D[M][N] += A[M][K] B[K][N] with K = the 128 points of an 8 (x) x 16 (y) tile at one level,
// N = the gradient's channels co (16 or 32) and M = 128 rows (dy shift s, input channel ci): the
// rows of A are the input plane read 16 / CG (4 or 8) rows apart, so one MMA covers the y offsets
// -1, 0, +1 (and spare shifts whose rows are dropped).  Each of the nine (dz, dx) offset pairs has
// its own accumulator in tensor memory; a block keeps them over all the (tile, level chunk) items
// it takes and adds them to dW once, at the end.  Both operands are MN-major (the channels are
// the contiguous 16 bytes of a core matrix; its 8 rows are 8 consecutive points along x):
//   x planes  Xsm[HY][CG][10][8]   halo rows y0-1 .. y0+14+SH, all channel groups of a row
//                                  together (a 5-D tensor map with the channel group as its own
//                                  dimension), so the next M block (next channel group, or the
//                                  next row after the last group) is 160 bytes on (SBO) and the
//                                  next K block (the next row of the tile) one halo row on (LBO)
//   gradient  Gsm[NP/8][16][8][8]  next N block = next channel group, 2048 bytes (SBO); next K
//                                  block = next row, 128 bytes (LBO)
// Warp 4 loads plane p of x (with its halo; zero outside the grid) and, for the levels of the
// item, plane p of g into one slot of a ring; warp 5 issues the 72 MMAs of a level (3 dz x 3 dx x
// 8 pairs of rows); warps 0-3 wait for the last MMA, read their lane quarter of the nine
// accumulators and add the rows of the y offsets -1..+1 to dW (atomicAdd).
template <int CG, int NP>
struct DwLayout {
  static constexpr int SH = 16 / CG;                        // y shifts in the 128 rows of M
  static constexpr int HY = TC_TY + SH - 1;                 // halo rows of an x plane
  static constexpr int ROW_BYTES = CG * TC_HX * 16;         // one halo row, all channel groups
  static constexpr int X_BYTES = HY * ROW_BYTES;
  static constexpr int X_PAD = (X_BYTES + 127) / 128 * 128;
  static constexpr int G_GROUP = TC_TY * TC_TX * 16;        // one 8-channel group of a gradient tile
  static constexpr int G_BYTES = NP / 8 * G_GROUP;
  static constexpr int SLOT = X_PAD + G_BYTES;
  static constexpr int R = 6;                               // ring slots
  static constexpr int TMEM_COLS = 9 * NP <= 256 ? 256 : 512;
  static constexpr int BAR_BYTES = (2 * R + 1) * 8 + 16;
  // + 4 KB after the barriers: an operand's core matrices, read with the two descriptor strides
  // either way round, stay inside the allocation
  static constexpr size_t NEED = 128 + (size_t)R * SLOT + BAR_BYTES + 4096;
  // at most 512 / TMEM_COLS blocks per SM, so that no block waits for another's tensor memory
  static constexpr size_t FLOOR = TMEM_COLS == 512 ? 120 * 1024 : 80 * 1024;
  static constexpr size_t BYTES = NEED < FLOOR ? FLOOR : NEED;
};

// a 5-D box into shared memory, completing on an mbarrier
__device__ __forceinline__ void tma_load_5d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            int c4, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
      "%5, %6}], [%7];" ::"r"(dst),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(bar)
      : "memory");
}

template <int CG, int NP>
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_conv3d_dw_tc(const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap gmap, int nx,
                   int ny, int nz, int zc, int cin, int cout, float* __restrict__ dw) {
  using L = DwLayout<CG, NP>;
  constexpr int R = L::R;
  extern __shared__ unsigned char tc_raw[];
  const uint32_t raw_s = smem_u32(tc_raw);
  unsigned char* smem = tc_raw + ((128u - (raw_s & 127u)) & 127u);
  const uint32_t ring_s = smem_u32(smem), bar_s = ring_s + R * L::SLOT;
  auto slot = [&](long long j) { return ring_s + (uint32_t)(j % R) * L::SLOT; };
  auto full = [&](long long j) { return bar_s + 8u * (uint32_t)(j % R); };
  auto empty = [&](long long j) { return bar_s + 8u * (R + (uint32_t)(j % R)); };
  const uint32_t done = bar_s + 8u * (2 * R);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + R * L::SLOT + (2 * R + 1) * 8);
  volatile int* abort = reinterpret_cast<volatile int*>(tslot + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (warp == 5) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(L::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < R; ++s) {
      mbar_init(full(s), 1);
      mbar_init(empty(s), 1);
    }
    mbar_init(done, 1);
    *abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;

  const int tiles_x = (nx + TC_TX - 1) / TC_TX, tiles_y = (ny + TC_TY - 1) / TC_TY;
  const int chunks = (nz + zc - 1) / zc, items = tiles_x * tiles_y * chunks;

  if (warp == 4) {
    // ---------------- producer ----------------
    if (lane == 0) {
      long long j = 0;
      bool ok = true;
      for (int it = blockIdx.x; it < items && ok; it += gridDim.x) {
        const int x0 = (it % tiles_x) * TC_TX, y0 = ((it / tiles_x) % tiles_y) * TC_TY;
        const int z0 = (it / (tiles_x * tiles_y)) * zc, z1 = min(z0 + zc, nz);
        for (int p = z0 - 1; p <= z1; ++p, ++j) {
          if (j >= R && !mbar_wait(empty(j), (uint32_t)((j / R - 1) & 1), abort)) {
            atomicAdd(&g_tc_timeouts, 1u);
            *abort = 1;
            ok = false;
            break;
          }
          const bool with_g = p >= z0 && p < z1;
          mbar_expect_tx(full(j), L::X_BYTES + (with_g ? L::G_BYTES : 0));
          tma_load_5d(slot(j), &xmap, 0, x0 - 1, 0, y0 - 1, p, full(j));
          if (with_g)
            for (int cg = 0; cg < NP / 8; ++cg)
              tma_load_4d(slot(j) + L::X_PAD + cg * L::G_GROUP, &gmap, cg * 8, x0, y0, p, full(j));
        }
      }
      // the copies this thread issued have landed before the block's memory goes (bounded)
      for (long long jj = j - 1; jj >= 0 && jj >= j - R; --jj) mbar_wait_long(full(jj), (uint32_t)((jj / R) & 1), nullptr);
    }
  } else if (warp == 5) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      constexpr uint32_t idesc = tc_idesc(128, NP) | (1u << 15) | (1u << 16);   // A and B MN-major
      long long j = 0;
      bool ok = true, first = true;
      for (int it = blockIdx.x; it < items && ok; it += gridDim.x) {
        const int z0 = (it / (tiles_x * tiles_y)) * zc, z1 = min(z0 + zc, nz);
        const long long jb = j;   // load index of plane z0 - 1
        for (int z = z0; z < z1 && ok; ++z) {
          const long long jz = jb + (z - z0);   // plane z - 1; planes z and z + 1 follow
          for (int q = (z == z0 ? 0 : 2); q <= 2 && ok; ++q) ok = mbar_wait(full(jz + q), (uint32_t)(((jz + q) / R) & 1), abort);
          if (!ok) {
            atomicAdd(&g_tc_timeouts, 1u);
            *abort = 1;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint64_t b0 = smem_desc(slot(jz + 1) + L::X_PAD, 128, L::G_GROUP);
#pragma unroll
          for (int dz = 0; dz < 3; ++dz) {
            const uint64_t a0 = smem_desc(slot(jz + dz), L::ROW_BYTES, TC_HX * 16);
#pragma unroll
            for (int dx = 0; dx < 3; ++dx)
#pragma unroll
              for (int m = 0; m < 8; ++m) {
                const uint64_t ad = a0 + (uint64_t)((2 * m * L::ROW_BYTES + dx * 16) >> 4);
                const uint64_t bd = b0 + (uint64_t)((2 * m * 128) >> 4);
                mma_bf16_tc(tmem + (uint32_t)((dz * 3 + dx) * NP), ad, bd, idesc, (first && m == 0) ? 0u : 1u);
              }
          }
          first = false;
          mma_commit(empty(jz));   // plane z - 1 is not read again
        }
        if (!ok) break;
        mma_commit(empty(jb + (z1 - z0)));       // planes z1 - 1 and z1
        mma_commit(empty(jb + (z1 - z0) + 1));
        j = jb + (z1 - z0) + 2;
      }
      mma_commit(done);
      mbar_wait_long(done, 0, nullptr);   // the MMAs are complete before the tensor memory goes
    }
  } else {
    // ---------------- warps 0-3: the accumulators into dW ----------------
    const bool got = __all_sync(0xffffffffu, mbar_wait_long(done, 0, abort));
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int r = 32 * warp + lane, b = r >> 3, s = b / CG, ci = (b % CG) * 8 + (r & 7);
    if (got && !*abort && (4 * warp) / CG <= 2) {   // the warp holds rows of the y offsets -1..+1
      const bool mine = s <= 2 && ci < cin;
#pragma unroll 1
      for (int acc = 0; acc < 9; ++acc) {
        float v[NP];
#pragma unroll
        for (int c = 0; c < NP; c += 16) tmem_load16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(acc * NP + c), v + c);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (mine) {
          const int tap = (acc / 3) * 9 + s * 3 + acc % 3;
          float* d = dw + (long long)tap * cout * cin + ci;
#pragma unroll
          for (int co = 0; co < NP; ++co)
            if (co < cout) atomicAdd(d + (long long)co * cin, v[co]);
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 5) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(L::TMEM_COLS) : "memory");
  }
}

constexpr int TC_MAX_DEVICES = 64;

template <int CIN, int COUT>
cudaError_t tc_grid(int* cap) {
  static int grid_cap[TC_MAX_DEVICES] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= TC_MAX_DEVICES) return cudaErrorInvalidDevice;
  if (!grid_cap[dev]) {
    using L = TcLayout<CIN, COUT>;
    e = cudaFuncSetAttribute(k_conv3d_tc<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L::BYTES);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_conv3d_tc<CIN, COUT>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return e;
    int sms = 0, per = 0;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_conv3d_tc<CIN, COUT>, L::THREADS, L::BYTES)) !=
        cudaSuccess)
      return e;
    grid_cap[dev] = sms * (per < 1 ? 1 : per);
  }
  *cap = grid_cap[dev];
  return cudaSuccess;
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn tc_encoder() {
  static EncodeTiledFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
    else
      cudaGetLastError();
  }
  return fn;
}

// activations [z][y][x][cin] BF16 as a 4-D tensor (channel, x, y, z); box = one 8-channel group of
// a 10 x 18 plane with halo; out-of-bounds elements read as zero
bool make_xmap(CUtensorMap* map, const void* x, int nx, int ny, int nz, int cin) {
  EncodeTiledFn enc = tc_encoder();
  if (!enc) return false;
  const cuuint64_t dims[4] = {(cuuint64_t)cin, (cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
  const cuuint64_t strides[3] = {(cuuint64_t)cin * 2, (cuuint64_t)nx * cin * 2, (cuuint64_t)ny * nx * cin * 2};
  const cuuint32_t box[4] = {8, TC_HX, TC_HY, 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(x), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int CIN, int COUT>
cudaError_t launch_tc(int nx, int ny, int nz, const void* x, const __nv_bfloat16* w, const float* bias, float* pre,
                      __nv_bfloat16* ybf, float* yf, int gelu, int creal, cudaStream_t st, bool pdl) {
  int cap = 0;
  cudaError_t e = tc_grid<CIN, COUT>(&cap);
  if (e != cudaSuccess) return e;
  CUtensorMap xmap;
  if (!make_xmap(&xmap, x, nx, ny, nz, CIN)) return cudaErrorInvalidValue;
  // level chunks of at least 4 levels: the count whose blocks fill their waves of resident blocks
  // best (ties: fewer chunks, since every chunk stages the weights and two extra planes)
  using L = TcLayout<CIN, COUT>;
  const int tiles = (nx / TC_TX) * (ny / TC_TY);
  int zc = nz;
  double best = -1.0;
  for (int nch = 1; nch <= (nz + 3) / 4; ++nch) {
    const int z = (nz + nch - 1) / nch;
    const long long blocks = (long long)tiles * ((nz + z - 1) / z);
    const double fill = (double)blocks / ((double)((blocks + cap - 1) / cap) * cap);
    if (fill > best + 1e-9) {
      best = fill;
      zc = z;
    }
  }
  if ((long long)tiles * ((nz + zc - 1) / zc) > 0x7fffffffll) return cudaErrorInvalidValue;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(tiles * ((nz + zc - 1) / zc)));
  cfg.blockDim = dim3(L::THREADS);
  cfg.dynamicSmemBytes = L::BYTES;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, k_conv3d_tc<CIN, COUT>, xmap, nx, ny, nz, zc, w, bias, pre, ybf, yf, gelu, creal,
                            pdl ? 1 : 0);
}


// activations [z][y][x][cin] BF16 as a 5-D tensor (8 channels, x, channel group, y, z): a box is a
// plane tile of 10 x hy points with all cin / 8 groups of each row side by side
bool make_dw_xmap(CUtensorMap* map, const void* x, int nx, int ny, int nz, int cin, int hy) {
  EncodeTiledFn enc = tc_encoder();
  if (!enc) return false;
  const cuuint64_t dims[5] = {8, (cuuint64_t)nx, (cuuint64_t)(cin / 8), (cuuint64_t)ny, (cuuint64_t)nz};
  const cuuint64_t strides[4] = {(cuuint64_t)cin * 2, 16, (cuuint64_t)nx * cin * 2, (cuuint64_t)ny * nx * cin * 2};
  const cuuint32_t box[5] = {8, TC_HX, (cuuint32_t)(cin / 8), (cuuint32_t)hy, 1};
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(x), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// gradient [z][y][x][c] BF16 as a 4-D tensor (channel, x, y, z); box = one 8-channel group of an
// 8 x 16 tile
bool make_dw_gmap(CUtensorMap* map, const void* g, int nx, int ny, int nz, int c) {
  EncodeTiledFn enc = tc_encoder();
  if (!enc) return false;
  const cuuint64_t dims[4] = {(cuuint64_t)c, (cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
  const cuuint64_t strides[3] = {(cuuint64_t)c * 2, (cuuint64_t)nx * c * 2, (cuuint64_t)ny * nx * c * 2};
  const cuuint32_t box[4] = {8, TC_TX, TC_TY, 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(g), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int CG, int NP>
cudaError_t dw_grid(int* cap) {
  static int grid_cap[TC_MAX_DEVICES] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= TC_MAX_DEVICES) return cudaErrorInvalidDevice;
  if (!grid_cap[dev]) {
    using L = DwLayout<CG, NP>;
    e = cudaFuncSetAttribute(k_conv3d_dw_tc<CG, NP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L::BYTES);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_conv3d_dw_tc<CG, NP>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return e;
    int sms = 0, per = 0;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_conv3d_dw_tc<CG, NP>, TC_THREADS, L::BYTES)) !=
        cudaSuccess)
      return e;
    per = per < 1 ? 1 : per;
    if (per > 512 / L::TMEM_COLS) per = 512 / L::TMEM_COLS;
    grid_cap[dev] = sms * per;
  }
  *cap = grid_cap[dev];
  return cudaSuccess;
}

template <int CG, int NP>
cudaError_t launch_dw(int nx, int ny, int nz, int cin, int cout, const void* x, const void* g, float* dw,
                      cudaStream_t st) {
  using L = DwLayout<CG, NP>;
  int cap = 0;
  cudaError_t e = dw_grid<CG, NP>(&cap);
  if (e != cudaSuccess) return e;
  CUtensorMap xmap, gmap;
  if (!make_dw_xmap(&xmap, x, nx, ny, nz, cin, L::HY) || !make_dw_gmap(&gmap, g, nx, ny, nz, NP))
    return cudaErrorInvalidValue;
  // level chunks: the count that ends soonest when every block takes ceil(items / blocks) items
  // of chunk + 1 plane times (ties: fewer items, each of which loads two extra planes)
  const long long tiles = (long long)((nx + TC_TX - 1) / TC_TX) * ((ny + TC_TY - 1) / TC_TY);
  int zc = nz;
  long long best = -1;
  for (int nch = 1; nch <= nz; ++nch) {
    const int z = (nz + nch - 1) / nch;
    const long long items = tiles * ((nz + z - 1) / z), blocks = items < cap ? items : cap;
    const long long cost = (items + blocks - 1) / blocks * (z + 1);
    if (best < 0 || cost < best) {
      best = cost;
      zc = z;
    }
  }
  const long long items = tiles * ((nz + zc - 1) / zc);
  if (items > 0x7fffffffll) return cudaErrorInvalidValue;
  const unsigned blocks = (unsigned)(items < cap ? items : cap);
  k_conv3d_dw_tc<CG, NP><<<blocks, TC_THREADS, L::BYTES, st>>>(xmap, gmap, nx, ny, nz, zc, cin, cout, dw);
  return cudaGetLastError();
}
}  // namespace

bool conv_tc_fits(int nx, int ny, int nz, int cin, int cout, const void* x, const void* pre, const void* ybf,
                  const void* yf) {
  const uintptr_t align = (uintptr_t)x | (uintptr_t)pre | (uintptr_t)ybf | (uintptr_t)yf;   // 16-byte TMA / stores
  return (cin == 16 || cin == 32) && (cout == 8 || cout == 16 || cout == 32) && nx > 0 && ny > 0 && nz > 0 &&
         nx % TC_TX == 0 && ny % TC_TY == 0 && (align & 15) == 0 && tc_encoder() != nullptr;
}

cudaError_t launch_conv_tc(int nx, int ny, int nz, int cin, int cout, const void* x, const void* w, const float* bias,
                           float* pre, void* ybf, float* yf, int gelu, int creal, cudaStream_t st, bool pdl) {
  if (!conv_tc_fits(nx, ny, nz, cin, cout, x, pre, ybf, yf)) return cudaErrorInvalidValue;
  const __nv_bfloat16* wb = (const __nv_bfloat16*)w;
  __nv_bfloat16* yb = (__nv_bfloat16*)ybf;
#define LEXGB_TC(CI, CO) launch_tc<CI, CO>(nx, ny, nz, x, wb, bias, pre, yb, yf, gelu, creal, st, pdl)
  if (cin == 16) return cout == 8 ? LEXGB_TC(16, 8) : cout == 16 ? LEXGB_TC(16, 16) : LEXGB_TC(16, 32);
  return cout == 8 ? LEXGB_TC(32, 8) : cout == 16 ? LEXGB_TC(32, 16) : LEXGB_TC(32, 32);
#undef LEXGB_TC
}

cudaError_t conv_tc_prepare() {
  int cap;
  cudaError_t e;
  if ((e = tc_grid<16, 8>(&cap)) != cudaSuccess) return e;
  if ((e = tc_grid<16, 16>(&cap)) != cudaSuccess) return e;
  if ((e = tc_grid<16, 32>(&cap)) != cudaSuccess) return e;
  if ((e = tc_grid<32, 8>(&cap)) != cudaSuccess) return e;
  if ((e = tc_grid<32, 16>(&cap)) != cudaSuccess) return e;
  if ((e = tc_grid<32, 32>(&cap)) != cudaSuccess) return e;
  if ((e = dw_grid<2, 16>(&cap)) != cudaSuccess) return e;
  if ((e = dw_grid<2, 32>(&cap)) != cudaSuccess) return e;
  if ((e = dw_grid<4, 16>(&cap)) != cudaSuccess) return e;
  return dw_grid<4, 32>(&cap);
}

bool conv_dw_tc_fits(int nx, int ny, int nz, int cin, int cout, int gstride, const void* x, const void* g,
                     const float* dw) {
  const uintptr_t align = (uintptr_t)x | (uintptr_t)g;   // 16-byte TMA bases
  return (cin == 16 || cin == 32) && (gstride == 16 || gstride == 32) && cout > 0 && cout <= gstride && nx > 0 &&
         ny > 0 && nz > 0 && (align & 15) == 0 && dw && tc_encoder() != nullptr;
}

cudaError_t launch_conv_dw_tc(int nx, int ny, int nz, int cin, int cout, int gstride, const void* x, const void* g,
                              float* dw, cudaStream_t st) {
  if (!conv_dw_tc_fits(nx, ny, nz, cin, cout, gstride, x, g, dw)) return cudaErrorInvalidValue;
  if (cin == 16) return gstride == 16 ? launch_dw<2, 16>(nx, ny, nz, cin, cout, x, g, dw, st)
                                      : launch_dw<2, 32>(nx, ny, nz, cin, cout, x, g, dw, st);
  return gstride == 16 ? launch_dw<4, 16>(nx, ny, nz, cin, cout, x, g, dw, st)
                       : launch_dw<4, 32>(nx, ny, nz, cin, cout, x, g, dw, st);
}

cudaError_t conv_tc_take_timeouts(unsigned int* n) {
  unsigned int zero = 0;
  cudaError_t e = cudaMemcpyFromSymbol(n, g_tc_timeouts, sizeof(unsigned int));
  if (e != cudaSuccess) return e;
  return cudaMemcpyToSymbol(g_tc_timeouts, &zero, sizeof(unsigned int));
}

}  // namespace lexgb
