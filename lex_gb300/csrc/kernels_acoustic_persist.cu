// kernels_acoustic_persist.cu - all acoustic sub-steps of one RK stage in one persistent kernel
// (sound_rk_step1/2, one_step_integration.py:638-675, :757-794).
//
// Each block owns a tile of 32 x 8 columns over every level and keeps that tile's pi' in shared
// memory from the first sub-step to the last.  u, v and w alternate between two global buffers
// (the tile's own values stay in L2); the per-stage inputs R_u, R_v, R_w, theta_rho and pi'_s are
// read every sub-step.  Inputs reach shared memory by TMA: slabs of 8 levels x 8 rows x 32 columns
// (cp.async.bulk.tensor, one box per field, exactly the tile, so no halo and no wrap) into a
// two-slot ring whose completion is tracked by an mbarrier per slot; the next slab's boxes are in
// flight while the current one is computed.  Values beyond the tile (the column west of it, the
// row south of it, the level below a slab) come by warp shuffles or plain loads.
//
// One sub-step in a block:
//   phase V  new u on the west faces, v on the south faces and w on the bottom faces of every cell
//            (to the sub-step's output buffers), from the old pi'; the blocks on the tile's east and
//            north edges also compute the neighbouring tiles' first face (u on x = tile end, v on
//            y = tile end) into small shared arrays;
//   phase P  new pi' of every cell (in place in shared memory) from the new winds;
//   the tile's edge pi' values go to an edge buffer for the neighbours, then a grid-wide barrier.
// The arithmetic of every face and cell is the same expression as k_acoustic_vec's.
//
// Every wait is bounded: a grid-barrier wait or an mbarrier wait that exceeds its poll limit
// records LEXGB_ERR_TIMEOUT in the context's status word and the block returns with no copy in
// flight (the state is then invalid; the host reports the status).  The launch is cooperative, so
// all blocks are resident.
#include <cuda.h>

#include "../../include/lexgb.h"
#include "lexgb_internal.cuh"

namespace lexgb {

// tensor maps of the fields the kernel stages by TMA; U/V/W indexed like PersistIO::u/v/w
struct PersistMaps {
  CUtensorMap trho, Ru, Rv, Rw, ps;
  CUtensorMap U[4], V[4], W[4];
};

namespace {

constexpr int PTX = 32, PTY = 8, SL = 8, PQX = PTX / 4;  // tile 32 x 8 columns, slabs of 8 levels
constexpr int PNT = PQX * PTY * SL;                       // 512 threads: one quad of one level each
constexpr int NFV = 7, NFP = 4;                           // ring fields of phase V and phase P
constexpr int BOX = SL * PTY * PTX;                       // floats in one field's box (8 KB)
constexpr unsigned FULL = 0xffffffffu;
// polls of an mbarrier wait for a slab's TMA boxes before it is reported as a timeout (a slab
// arrives within microseconds; the limit only bounds a wait that would otherwise never end)
constexpr long long kRingPolls = 1LL << 22;
constexpr float kHalfCpP = (float)(0.5 * kCp);
constexpr float kRdCvP = (float)(kRd / kCv);

struct Smem {  // offsets (floats) of the dynamic shared-memory regions
  int ring, ue, vn, bars;
  size_t bytes;
};

__host__ __device__ __forceinline__ Smem smem_layout(int nz) {
  Smem s;
  s.ring = nz * PTY * PTX;                 // pi' occupies [0, ring)
  s.ue = s.ring + 2 * NFV * BOX;           // ring: 2 slots x 7 boxes
  s.vn = s.ue + nz * PTY;                  // u on the tile's east face [nz][8]
  s.bars = s.vn + nz * PTX;                // v on the row north of the tile [nz][32]
  s.bytes = (size_t)s.bars * sizeof(float) + 2 * sizeof(unsigned long long) + 16;  // + the barrier flag
  return s;
}

__device__ __forceinline__ float pgfp(float tra, float trb, float pa, float pb, float rd) {
  return -kHalfCpP * (tra + trb) * ((pa - pb) * rd);
}
__device__ __forceinline__ float4 ldg4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }
__device__ __forceinline__ float4 ldcg4(const float* p) { return __ldcg(reinterpret_cast<const float4*>(p)); }
__device__ __forceinline__ void st4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
__device__ __forceinline__ float4 zero4() { return make_float4(0.f, 0.f, 0.f, 0.f); }
__device__ __forceinline__ float at(const float4& v, int l) { return l == 0 ? v.x : (l == 1 ? v.y : (l == 2 ? v.z : v.w)); }

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_relaxed(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// ---- mbarrier and TMA (PTX) ----
__device__ __forceinline__ unsigned saddr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}
// one 3-D box (x, y, z = first column, row, level) of a tensor map into shared memory
__device__ __forceinline__ void tma_load_3d(unsigned dst, const CUtensorMap* map, int x, int y, int z, unsigned bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(dst),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}

// Grid-wide barrier over a monotone arrival counter (zeroed before the launch): arrival number
// `target` = blocks * (barrier index + 1).  Returns false when the wait gave up or another block
// already recorded a failure.
__device__ bool grid_sync(unsigned* bar, int* status, unsigned target, long long limit, int* ok) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(bar, 1u);
    int good = 1;
    long long it = 0;
    while (ld_acquire(bar) < target) {
      if (++it > limit || ld_relaxed(status) != 0) {
        atomicCAS(status, 0, LEXGB_ERR_TIMEOUT);
        good = 0;
        break;
      }
      __nanosleep(32);
    }
    __threadfence();
    *ok = good;
  }
  __syncthreads();
  return *ok != 0;
}

// Wait for the ring slot's mbarrier to complete its current phase (bounded).  On a timeout the
// status is recorded and the wait goes on (bounded again), so that the block does not leave
// while the slab's copies may still be writing its shared memory.
__device__ __forceinline__ bool ring_wait(unsigned bar, unsigned parity, long long limit, int* status) {
  long long it = 0;
  while (!mbar_try_wait(bar, parity)) {
    if (++it > limit) {
      atomicCAS(status, 0, LEXGB_ERR_TIMEOUT);
      for (long long j = 0; j < limit && !mbar_try_wait(bar, parity); ++j) __nanosleep(64);
      return false;
    }
  }
  return true;
}

__global__ void __launch_bounds__(PNT, 1)
    k_acoustic_persist(Dims d, Phys ph, Cols c, PersistIO a, const __grid_constant__ PersistMaps m) {
  extern __shared__ __align__(128) float sm[];
  const int nx = d.nx, ny = d.ny, nz = d.nz, plane = nx * ny;
  const Smem L = smem_layout(nz);
  float* sP = sm;                      // pi' [nz][8][32]
  float* ring = sm + L.ring;           // [2][7][SL][8][32]
  float* sUE = sm + L.ue;              // [nz][8]
  float* sVN = sm + L.vn;              // [nz][32]
  unsigned long long* bars = reinterpret_cast<unsigned long long*>(sm + L.bars);
  const unsigned bar0 = saddr(&bars[0]), bar1 = saddr(&bars[1]);
  int* sync_ok = reinterpret_cast<int*>(bars + 2);
  const int tiles_x = nx / PTX;
  const int tx0 = (blockIdx.x % tiles_x) * PTX, ty0 = (blockIdx.x / tiles_x) * PTY;
  const int tid = threadIdx.x, qx = tid & 7, jj = (tid >> 3) & 7, kk = tid >> 6;
  const int i0 = tx0 + 4 * qx, j = ty0 + jj;
  const int jm = wrap(j - 1, ny), jp = wrap(j + 1, ny);
  const int iw = wrap(i0 - 1, nx), ie = wrap(i0 + 4, nx);
  const int ns = (nz + SL - 1) / SL;   // slabs
  const float dtau = a.dtau, rdx = ph.rdx, rdy = ph.rdy, rdz = ph.rdz;
  const long long lim = a.spin_limit;   // grid-barrier polls
  const int own = (kk * PTY + jj) * PQX + qx;   // this thread's quad in a box (float4 index)

  if (tid == 0) {
    mbar_init(bar0, 1);
    mbar_init(bar1, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int idx = tid; idx < PQX * PTY * nz; idx += PNT) {
    const int q = idx % PQX, r = (idx / PQX) % PTY, k = idx / (PQX * PTY);
    reinterpret_cast<float4*>(sP)[idx] = ldcg4(a.p0 + (k * ny + ty0 + r) * nx + tx0 + 4 * q);
  }
  __syncthreads();
  unsigned par0 = 0, par1 = 0;   // phase parity of each ring slot's mbarrier

  // issue the boxes of slab n (fields of the phase) into ring slot n & 1
  auto issue = [&](const CUtensorMap* const* maps, int nf, int n) {
    const unsigned bar = (n & 1) ? bar1 : bar0;
    float* slot = ring + (n & 1) * NFV * BOX;
    mbar_expect_tx(bar, (unsigned)(nf * BOX * sizeof(float)));
    for (int f = 0; f < nf; ++f) tma_load_3d(saddr(slot + f * BOX), maps[f], tx0, ty0, n * SL, bar);
  };
  auto wait_slot = [&](int n) -> bool {
    const bool odd = n & 1;
    const bool okw = ring_wait(odd ? bar1 : bar0, odd ? par1 : par0, kRingPolls, a.status);
    if (odd) par1 ^= 1u; else par0 ^= 1u;
    return okw;
  };

  for (int s = 0; s < a.nsub; ++s) {
    const bool last = s == a.nsub - 1;
    const int src = s == 0 ? 0 : 1 + ((s - 1) & 1), dst = last ? 3 : 1 + (s & 1);
    const float* us = a.u[src];
    const float* vs = a.v[src];
    const float* hs = s == 0 ? a.p0 : a.hb[(s - 1) & 1];
    float* ud = a.u[dst];
    float* vd = a.v[dst];
    float* wd = a.w[dst];
    float* hd = a.hb[s & 1];
    bool good = true;

    // ---------------- phase V: winds on the west, south and bottom faces ----------------
    {
      const CUtensorMap* maps[NFV] = {&m.trho, &m.U[src], &m.Ru, &m.V[src], &m.Rv, &m.W[src], &m.Rw};
      if (tid == 0) {
        issue(maps, NFV, 0);
        if (ns > 1) issue(maps, NFV, 1);
      }
      for (int n = 0; n < ns; ++n) {
        const int k = n * SL + kk;
        const bool live = k < nz;
        const int r0 = k * plane + j * nx + i0;
        // loads that do not come from the ring, issued before waiting for it
        float tWg = 0.f, pWg = 0.f;
        float4 tSg = zero4(), pSg = zero4(), tBg = zero4();
        float uEo = 0.f, ruE = 0.f, tE = 0.f, pE = 0.f;
        float4 vNo = zero4(), rvN = zero4(), tN = zero4(), pN = zero4();
        if (live) {
          if (qx == 0) {
            tWg = __ldg(a.trho + k * plane + j * nx + iw);
            pWg = __ldcg(hs + k * plane + j * nx + iw);
          }
          if (jj == 0) {
            tSg = ldg4(a.trho + k * plane + jm * nx + i0);
            pSg = ldcg4(hs + k * plane + jm * nx + i0);
          }
          if (kk == 0 && k > 0) tBg = ldg4(a.trho + r0 - plane);
          if (qx == PQX - 1) {  // u on the east tile's first face (x = tile end), for phase P
            const int re = k * plane + j * nx + ie;
            uEo = __ldcg(us + re); ruE = __ldg(a.Ru + re); tE = __ldg(a.trho + re); pE = __ldcg(hs + re);
          }
          if (jj == PTY - 1) {  // v on the north tile's first row, for phase P
            const int rn = k * plane + jp * nx + i0;
            vNo = ldcg4(vs + rn); rvN = ldg4(a.Rv + rn); tN = ldg4(a.trho + rn); pN = ldcg4(hs + rn);
          }
        }
        good = wait_slot(n) && good;
        const float4* slot = reinterpret_cast<const float4*>(ring + (n & 1) * NFV * BOX);
        if (live) {
          const float4 T = slot[0 * BOX / 4 + own], U = slot[1 * BOX / 4 + own], RU = slot[2 * BOX / 4 + own];
          const float4 Vv = slot[3 * BOX / 4 + own], RV = slot[4 * BOX / 4 + own];
          const float4 W = slot[5 * BOX / 4 + own], RW = slot[6 * BOX / 4 + own];
          const float4 P = reinterpret_cast<const float4*>(sP)[(k * PTY + jj) * PQX + qx];
          float tW = __shfl_up_sync(FULL, T.w, 1, 8), pW = __shfl_up_sync(FULL, P.w, 1, 8);
          if (qx == 0) { tW = tWg; pW = pWg; }
          const float4 tS = jj > 0 ? slot[0 * BOX / 4 + own - PQX] : tSg;
          const float4 pS = jj > 0 ? reinterpret_cast<const float4*>(sP)[(k * PTY + jj - 1) * PQX + qx] : pSg;
          const float4 tB = kk > 0 ? slot[0 * BOX / 4 + own - PQX * PTY] : tBg;
          const float4 pB = k > 0 ? reinterpret_cast<const float4*>(sP)[((k - 1) * PTY + jj) * PQX + qx] : zero4();
          float4 un, vn, wn;
          un.x = U.x + (pgfp(T.x, tW, P.x, pW, rdx) + RU.x) * dtau;
          un.y = U.y + (pgfp(T.y, T.x, P.y, P.x, rdx) + RU.y) * dtau;
          un.z = U.z + (pgfp(T.z, T.y, P.z, P.y, rdx) + RU.z) * dtau;
          un.w = U.w + (pgfp(T.w, T.z, P.w, P.z, rdx) + RU.w) * dtau;
          vn.x = Vv.x + (pgfp(T.x, tS.x, P.x, pS.x, rdy) + RV.x) * dtau;
          vn.y = Vv.y + (pgfp(T.y, tS.y, P.y, pS.y, rdy) + RV.y) * dtau;
          vn.z = Vv.z + (pgfp(T.z, tS.z, P.z, pS.z, rdy) + RV.z) * dtau;
          vn.w = Vv.w + (pgfp(T.w, tS.w, P.w, pS.w, rdy) + RV.w) * dtau;
          if (k > 0) {
            wn.x = W.x + (pgfp(T.x, tB.x, P.x, pB.x, rdz) + RW.x) * dtau;
            wn.y = W.y + (pgfp(T.y, tB.y, P.y, pB.y, rdz) + RW.y) * dtau;
            wn.z = W.z + (pgfp(T.z, tB.z, P.z, pB.z, rdz) + RW.z) * dtau;
            wn.w = W.w + (pgfp(T.w, tB.w, P.w, pB.w, rdz) + RW.w) * dtau;
          } else {
            wn = zero4();  // bottom face
          }
          st4(ud + r0, un);
          st4(vd + r0, vn);
          st4(wd + r0, wn);
          if (k == nz - 1) st4(wd + r0 + plane, zero4());  // lid face
          if (qx == PQX - 1) sUE[k * PTY + jj] = uEo + (pgfp(tE, T.w, pE, P.w, rdx) + ruE) * dtau;
          if (jj == PTY - 1) {
            float4 v2;
            v2.x = vNo.x + (pgfp(tN.x, T.x, pN.x, P.x, rdy) + rvN.x) * dtau;
            v2.y = vNo.y + (pgfp(tN.y, T.y, pN.y, P.y, rdy) + rvN.y) * dtau;
            v2.z = vNo.z + (pgfp(tN.z, T.z, pN.z, P.z, rdy) + rvN.z) * dtau;
            v2.w = vNo.w + (pgfp(tN.w, T.w, pN.w, P.w, rdy) + rvN.w) * dtau;
            reinterpret_cast<float4*>(sVN)[k * PQX + qx] = v2;
          }
        }
        __syncthreads();   // the slot is read; the next copies may overwrite it
        if (tid == 0 && n + 2 < ns) issue(maps, NFV, n + 2);
      }
    }
    // the winds just written are read back by TMA (async proxy) in phase P and the next sub-step
    asm volatile("fence.proxy.async.global;" ::: "memory");
    __syncthreads();

    // ---------------- phase P: pi' of every cell from the new winds ----------------
    {
      const CUtensorMap* maps[NFP] = {&m.U[dst], &m.V[dst], &m.W[dst], &m.ps};
      if (tid == 0) {
        issue(maps, NFP, 0);
        if (ns > 1) issue(maps, NFP, 1);
      }
      for (int n = 0; n < ns; ++n) {
        const int k = n * SL + kk;
        const bool live = k < nz;
        const int r0 = k * plane + j * nx + i0;
        const bool has_b = k > 0, has_t = k + 1 < nz;
        float sWg = 0.f, sEg = 0.f;
        float4 sSg = zero4(), sNg = zero4(), SBg = zero4(), STg = zero4(), wTg = zero4();
        if (live) {
          if (qx == 0) sWg = __ldg(a.ps + k * plane + j * nx + iw);
          if (qx == PQX - 1) sEg = __ldg(a.ps + k * plane + j * nx + ie);
          if (jj == 0) sSg = ldg4(a.ps + k * plane + jm * nx + i0);
          if (jj == PTY - 1) sNg = ldg4(a.ps + k * plane + jp * nx + i0);
          if (kk == 0 && has_b) SBg = ldg4(a.ps + r0 - plane);
          if (kk == SL - 1 && has_t) {
            STg = ldg4(a.ps + r0 + plane);
            wTg = ldcg4(wd + r0 + plane);
          }
        }
        good = wait_slot(n) && good;
        const float4* slot = reinterpret_cast<const float4*>(ring + (n & 1) * NFV * BOX);
        if (live) {
          const float4 UN = slot[0 * BOX / 4 + own], VN = slot[1 * BOX / 4 + own];
          const float4 wB = has_b ? slot[2 * BOX / 4 + own] : zero4();
          const float4 S0 = slot[3 * BOX / 4 + own];
          float uE = __shfl_down_sync(FULL, UN.x, 1, 8);
          if (qx == PQX - 1) uE = sUE[k * PTY + jj];
          float sW = __shfl_up_sync(FULL, S0.w, 1, 8), sE = __shfl_down_sync(FULL, S0.x, 1, 8);
          if (qx == 0) sW = sWg;
          if (qx == PQX - 1) sE = sEg;
          const float4 vN = jj < PTY - 1 ? slot[1 * BOX / 4 + own + PQX] : reinterpret_cast<const float4*>(sVN)[k * PQX + qx];
          const float4 sS = jj > 0 ? slot[3 * BOX / 4 + own - PQX] : sSg;
          const float4 sN = jj < PTY - 1 ? slot[3 * BOX / 4 + own + PQX] : sNg;
          const float4 SB = !has_b ? zero4() : (kk > 0 ? slot[3 * BOX / 4 + own - PQX * PTY] : SBg);
          const float4 ST = !has_t ? zero4() : (kk < SL - 1 ? slot[3 * BOX / 4 + own + PQX * PTY] : STg);
          const float4 wT = !has_t ? zero4() : (kk < SL - 1 ? slot[2 * BOX / 4 + own + PQX * PTY] : wTg);
          float4* pp = &reinterpret_cast<float4*>(sP)[(k * PTY + jj) * PQX + qx];
          const float4 P = *pp;
          const float rho = c.rho[k], rhoi = c.rho_inv[k], rfb = c.rho_face[k], rft = c.rho_face[k + 1];
          const float dzb = c.dpi0dz[k], dzt = c.dpi0dz[k + 1], pi0 = c.pi0[k];
          const float un[5] = {UN.x, UN.y, UN.z, UN.w, uE};
          const float sc[6] = {sW, S0.x, S0.y, S0.z, S0.w, sE};
          float outp[4];
#pragma unroll
          for (int l = 0; l < 4; ++l) {
            const float vs_ = at(VN, l), vn_ = at(vN, l);
            const float wb = has_b ? at(wB, l) : 0.f;
            const float wt = has_t ? at(wT, l) : 0.f;
            const float div = (un[l + 1] - un[l]) * rdx + (vn_ - vs_) * rdy + (wt - wb) * rdz;
            const float s0 = sc[l + 1];
            const float gxw = (s0 - sc[l]) * rdx, gxe = (sc[l + 2] - s0) * rdx;
            const float gys = (s0 - at(sS, l)) * rdy, gyn = (at(sN, l) - s0) * rdy;
            const float wzb = has_b ? wb * (dzb + (s0 - at(SB, l)) * rdz) : 0.f;
            const float wzt = has_t ? wt * (dzt + (at(ST, l) - s0) * rdz) : 0.f;
            const float ap = -(0.5f * (un[l + 1] * gxe + un[l] * gxw) + 0.5f * (vn_ * gyn + vs_ * gys) +
                               (0.5f * wzb * rfb + 0.5f * wzt * rft) * rhoi);
            const float dpdt = -kRdCvP * ((pi0 + s0) * div) + ap;
            outp[l] = at(P, l) + (kDivDamp * dpdt) * dtau;
          }
          const float4 pn = make_float4(outp[0], outp[1], outp[2], outp[3]);
          *pp = pn;
          if (!last) {  // the tile's edge values for the neighbouring tiles' next sub-step
            if (jj == 0 || jj == PTY - 1) {
              st4(hd + r0, pn);
            } else {
              if (qx == 0) hd[r0] = pn.x;
              if (qx == PQX - 1) hd[r0 + 3] = pn.w;
            }
          }
        }
        __syncthreads();
        if (tid == 0 && n + 2 < ns) issue(maps, NFP, n + 2);
      }
    }
    if (!good) return;   // an mbarrier wait gave up: no copy is in flight (all slabs were waited for)
    // (the test mode waits for one arrival more than there are blocks: the wait can only give up)
    const unsigned target = gridDim.x * (unsigned)(s + 1) + (a.unreachable ? 1u : 0u);
    if (!last && !grid_sync(a.bar, a.status, target, lim, sync_ok)) return;
  }

  // the stage's pi' from shared memory (u, v and w were written by the last sub-step)
  __syncthreads();
  for (int idx = tid; idx < PQX * PTY * nz; idx += PNT) {
    const int q = idx % PQX, r = (idx / PQX) % PTY, k = idx / (PQX * PTY);
    st4(a.po + (k * ny + ty0 + r) * nx + tx0 + 4 * q, reinterpret_cast<const float4*>(sP)[idx]);
  }
}

typedef CUresult (*EncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encoder() {
  static EncodeTiled fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiled>(p);
    else
      cudaGetLastError();
  }
  return fn;
}

// box of 32 columns x 8 rows x 8 levels over a field of `levels` levels (x fastest)
bool make_map(CUtensorMap* map, const float* base, const Dims& d, int levels) {
  EncodeTiled enc = encoder();
  if (!enc) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)d.nx, (cuuint64_t)d.ny, (cuuint64_t)levels};
  const cuuint64_t strides[2] = {(cuuint64_t)d.nx * sizeof(float), (cuuint64_t)d.nx * d.ny * sizeof(float)};
  const cuuint32_t box[3] = {PTX, PTY, SL};
  const cuuint32_t estr[3] = {1, 1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

size_t acoustic_persist_smem(const Dims& d) { return smem_layout(d.nz).bytes; }

// Blocks the persistent kernel needs for this grid, or 0 when it cannot run it: nx a multiple of
// 32 and ny of 8, the tile's pi' and the TMA ring within the shared memory of a block, every block
// resident at once (one per SM), cooperative launches and the tensor-map encoder available.
int acoustic_persist_blocks(const Dims& d) {
  if (d.nx % PTX != 0 || d.ny % PTY != 0 || d.nz < 2 || !encoder()) return 0;
  int dev = 0, coop = 0, sms = 0, maxsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) ||
      cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev)) {
    cudaGetLastError();
    return 0;
  }
  const size_t smem = acoustic_persist_smem(d);
  if (!coop || smem + 64 > (size_t)maxsm) return 0;
  if (cudaFuncSetAttribute(k_acoustic_persist, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_acoustic_persist, PNT, smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  const int blocks = (d.nx / PTX) * (d.ny / PTY);
  return blocks <= per_sm * sms ? blocks : 0;
}

cudaError_t launch_acoustic_persist(const Dims& d, const Phys& ph, const Cols& c, const PersistIO& io,
                                    cudaStream_t st, const cudaAccessPolicyWindow* win) {
  PersistMaps m;
  bool ok = make_map(&m.trho, io.trho, d, d.nz) && make_map(&m.Ru, io.Ru, d, d.nz) &&
            make_map(&m.Rv, io.Rv, d, d.nz) && make_map(&m.Rw, io.Rw, d, d.nz + 1) && make_map(&m.ps, io.ps, d, d.nz);
  for (int b = 0; b < 4 && ok; ++b)
    ok = make_map(&m.U[b], io.u[b], d, d.nz) && make_map(&m.V[b], io.v[b], d, d.nz) &&
         make_map(&m.W[b], io.w[b], d, d.nz + 1);
  if (!ok) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(io.bar, 0, sizeof(unsigned), st);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((d.nx / PTX) * (d.ny / PTY));
  cfg.blockDim = dim3(PNT);
  cfg.dynamicSmemBytes = acoustic_persist_smem(d);
  cfg.stream = st;
  cudaLaunchAttribute attr[2];
  int na = 0;
  attr[na].id = cudaLaunchAttributeCooperative;
  attr[na].val.cooperative = 1;
  ++na;
  if (win) {
    attr[na].id = cudaLaunchAttributeAccessPolicyWindow;
    attr[na].val.accessPolicyWindow = *win;
    ++na;
  }
  cfg.attrs = attr;
  cfg.numAttrs = na;
  e = cudaLaunchKernelEx(&cfg, k_acoustic_persist, d, ph, c, io, m);
  return e != cudaSuccess ? e : cudaGetLastError();
}

}  // namespace lexgb
