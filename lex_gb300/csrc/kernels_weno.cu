// kernels_weno.cu - slow-mode WENO5 advection of one RK stage, tiled in 3-D.
//
// Flux-form advection of the prognostic fields (advection.py:9-149, fluxes :305-1281):
//
//   tendency(phi) = ( -sum_d d(m_d * phi_face)/dx_d + phi * div_at_phi ) / rho_at_phi
//
// Two kernels: k_weno_scalars advects theta and qv together (their mass fluxes are the same
// rho0*u, rho0*v, rho0*w on the cell faces), k_weno_momentum advects u, v and w together (their
// mass fluxes are averages of the three winds, all staged in shared memory).
//
// A block owns a 32 x 4 x 4 box of points, one thread per point.  It stages each field on the
// box plus halo in shared memory (periodic in x and y, clamped in z; x rows are widened to 40
// floats starting at i0-4 so that rows move as aligned float4s when nx % 4 == 0), evaluates
// every x, y and z face flux of the box exactly once - each thread its point's west, south and
// bottom faces, whole warps the box's north, top and east edge faces - and forms each point's
// tendency from its six face fluxes.  Everything a thread's own faces and its point need from
// global memory is loaded before the first barrier; the upwind stencil is selected from the
// sign of the mass flux before the reconstruction.
//
// Outputs (one_step_integration.py:258-296):
//   theta, qv : phi_next = phi^0 + dt_s * adv (+ dt_s * sgs); optional record of adv (+ sgs)
//   u         : R_u = adv + f v (Coriolis, pressure_gradient_coriolis.py:80-113) + sgs_u
//   v         : R_v = adv - f u + sgs_v
//   w         : R_w = adv + b8w (buoyancy at faces, pressure_equations.py:162-172) + sgs_w, with
//               adv = 0 on the bottom and lid faces (advection.py:146-147); wmode 1: adv only,
//               wmode 2: b8w only (diagnostics).
#include "lexgb_internal.cuh"

namespace lexgb {

namespace {

constexpr int TX = 32, TY = 4, TZ = 4, HALO = 3, HX = 4;
constexpr int NT = TX * TY * TZ;
constexpr int BX3 = TX + 2 * HX, BY3 = TY + 2 * HALO, BZ3 = TZ + 2 * HALO;  // 40 x 10 x 10
constexpr int NWARP = NT / 32;

typedef float Box[BZ3][BY3][BX3];
typedef float FluxX[TZ][TY][TX + 1];
typedef float FluxY[TZ][TY + 1][TX];
typedef float FluxZ[TZ + 1][TY][TX];

__device__ __forceinline__ int pmod(int i, int n) {
  i %= n;
  return i < 0 ? i + n : i;
}

#define LD(p, idx) __ldg((p) + (idx))

// global index tables of the box's halo coordinates (box column lx <-> x = i0 - 4 + lx,
// row ly <-> y = j0 - 3 + ly, layer lz <-> level k0 - 3 + lz)
struct Idx {
  int x[BX3];   // wrapped x
  int y[BY3];   // wrapped y, times nx
  int zc[BZ3];  // cell level clamped to 0..nz-1, times nx*ny
  int zw[BZ3];  // face level clamped to 0..nz, times nx*ny
};

__device__ __forceinline__ void build_idx(Idx& ix, int tid, int i0, int j0, int k0, const Dims& d) {
  if (tid < BX3) {
    ix.x[tid] = pmod(i0 - HX + tid, d.nx);
  } else if (tid < BX3 + BY3) {
    ix.y[tid - BX3] = pmod(j0 - HALO + (tid - BX3), d.ny) * d.nx;
  } else if (tid < BX3 + BY3 + BZ3) {
    const int lz = tid - BX3 - BY3;
    const int k = k0 - HALO + lz;
    ix.zc[lz] = clampi(k, 0, d.nz - 1) * d.plane();
    ix.zw[lz] = clampi(k, 0, d.nz) * d.plane();
  }
}

// Staging of NF fields on their boxes with all loads in flight before any shared store.
// vec4: rows move as 10 aligned float4s (nx % 4 == 0, so a 4-group never straddles the periodic
// seam); otherwise warp-per-row scalar loads.
constexpr int ROWS = BY3 * BZ3;
constexpr int NQ4 = ROWS * (BX3 / 4);
constexpr int IT4 = (NQ4 + NT - 1) / NT;
constexpr int RPW = (ROWS + NWARP - 1) / NWARP;

template <int NF>
__device__ __forceinline__ void stage(Box* const (&b)[NF], const float* const (&f)[NF], const int* const (&zbase)[NF],
                                      const Idx& ix, int tid, bool vec4) {
  if (vec4) {
    float4 v[NF][IT4];
#pragma unroll
    for (int q = 0; q < IT4; ++q) {
      const int t = tid + q * NT;
      if (t < NQ4) {
        const int r = t / (BX3 / 4), c4 = t - r * (BX3 / 4);
        const int lz = r / BY3, ly = r - lz * BY3;
#pragma unroll
        for (int n = 0; n < NF; ++n)
          v[n][q] = __ldg(reinterpret_cast<const float4*>(f[n] + zbase[n][lz] + ix.y[ly] + ix.x[4 * c4]));
      }
    }
#pragma unroll
    for (int q = 0; q < IT4; ++q) {
      const int t = tid + q * NT;
      if (t < NQ4) {
        const int r = t / (BX3 / 4), c4 = t - r * (BX3 / 4);
        const int lz = r / BY3, ly = r - lz * BY3;
#pragma unroll
        for (int n = 0; n < NF; ++n) *reinterpret_cast<float4*>(&(*b[n])[lz][ly][4 * c4]) = v[n][q];
      }
    }
  } else {
    const int lane = tid & 31, warp = tid >> 5;
    const int xa = ix.x[lane];
    const bool tail = lane < BX3 - 32;
    const int xb = tail ? ix.x[32 + lane] : 0;
    float va[NF][RPW], vb[NF][RPW];
#pragma unroll
    for (int q = 0; q < RPW; ++q) {
      const int r = warp + q * NWARP;
      if (r < ROWS) {
        const int lz = r / BY3, ly = r - lz * BY3;
#pragma unroll
        for (int n = 0; n < NF; ++n) {
          const int base = zbase[n][lz] + ix.y[ly];
          va[n][q] = LD(f[n], base + xa);
          vb[n][q] = tail ? LD(f[n], base + xb) : 0.f;
        }
      }
    }
#pragma unroll
    for (int q = 0; q < RPW; ++q) {
      const int r = warp + q * NWARP;
      if (r < ROWS) {
        const int lz = r / BY3, ly = r - lz * BY3;
#pragma unroll
        for (int n = 0; n < NF; ++n) {
          (*b[n])[lz][ly][lane] = va[n][q];
          if (tail) (*b[n])[lz][ly][32 + lane] = vb[n][q];
        }
      }
    }
  }
}

// face value through column face H (between entries H-1 and H of an n-entry column), given
// s(H-3..H+2); entries outside 0..n-1 are never used; zero on the end faces.  Near-boundary
// rules of vertical_flux_scalar2 and friends (advection.py:327-406).
__device__ __forceinline__ float vflux6(float m, float sm3, float sm2, float sm1, float s0, float sp1, float sp2, int H,
                                        int n, float eps) {
  if (H <= 0 || H >= n) return 0.f;
  const bool up = m >= 0.f;
  float r;
  if (H >= 3 && H <= n - 3) {
    r = weno5(up ? sm3 : sp2, up ? sm2 : sp1, up ? sm1 : s0, up ? s0 : sm1, up ? sp1 : sm2, eps);
  } else if (up) {
    if (H == 1)
      r = 0.5f * (sm1 + s0);
    else if (H == 2 || H == n - 1)
      r = weno3(sm2, sm1, s0, eps);
    else  // H == n-2
      r = weno5(sm3, sm2, sm1, s0, sp1, eps);
  } else {
    if (H == n - 1)
      r = 0.5f * (s0 + sm1);
    else if (H == 1 || H == n - 2)
      r = weno3(sp1, s0, sm1, eps);
    else  // H == 2
      r = weno5(sp2, sp1, s0, sm1, sm2, eps);
  }
  return m * r;
}

// WENO face fluxes of a staged field at box coordinates (lx, ly, lz) of the point right of /
// above the face
__device__ __forceinline__ float wx(const Box& b, int lx, int ly, int lz, float m, float eps) {
  return weno_flux(m, b[lz][ly][lx - 3], b[lz][ly][lx - 2], b[lz][ly][lx - 1], b[lz][ly][lx], b[lz][ly][lx + 1],
                   b[lz][ly][lx + 2], eps);
}
__device__ __forceinline__ float wy(const Box& b, int lx, int ly, int lz, float m, float eps) {
  return weno_flux(m, b[lz][ly - 3][lx], b[lz][ly - 2][lx], b[lz][ly - 1][lx], b[lz][ly][lx], b[lz][ly + 1][lx],
                   b[lz][ly + 2][lx], eps);
}
__device__ __forceinline__ float wz(const Box& b, int lx, int ly, int lz, float m, int H, int n, float eps) {
  return vflux6(m, b[lz - 3][ly][lx], b[lz - 2][ly][lx], b[lz - 1][ly][lx], b[lz][ly][lx], b[lz + 1][ly][lx],
                b[lz + 2][ly][lx], H, n, eps);
}

// Edge faces: warps 0-3 the north faces of layer `warp`, warps 4-7 the top faces of row warp-4,
// warp 8 (16 lanes) the east faces of (row, layer) = (lane % TY, lane / TY).
struct EdgeFace {
  int which;       // -1 none, 0 x, 1 y, 2 z
  int lx, ly, lz;  // box coordinates of the point right of / above the face
  int fi, fj, fk;  // slot in the flux arrays
};

__device__ __forceinline__ EdgeFace edge_face(int warp, int lane) {
  EdgeFace e{-1, 0, 0, 0, 0, 0, 0};
  if (warp < 4) {
    e = EdgeFace{1, lane + HX, TY + HALO, warp + HALO, lane, TY, warp};
  } else if (warp < 8) {
    e = EdgeFace{2, lane + HX, warp - 4 + HALO, TZ + HALO, lane, warp - 4, TZ};
  } else if (warp == 8 && lane < TY * TZ) {
    e = EdgeFace{0, TX + HX, lane % TY + HALO, lane / TY + HALO, TX, lane % TY, lane / TY};
  }
  return e;
}

// ================================================================================================
// theta and qv
// ================================================================================================
struct ScalarArgs {
  const float* div;
  const float* T0;  // values at the start of the big step (may alias the outputs)
  const float* q0;
  const float* sgsT;
  const float* sgsQ;
  float* Tn;
  float* qn;
  float* recT;
  float* recQ;
  float dts;
  float* div_out;   // vertical march only: when set, div(rho0 u) and theta_rho of the state are computed
  float* trho_out;  // here (div then unused as an input) and written out
};

// theta and qv share every mass flux, so they are staged interleaved as (theta, qv) pairs and
// each face's two reconstructions run together on the packed FP32x2 pipe.
typedef float2 Box2[BZ3][BY3][BX3];

__device__ __forceinline__ float2 vflux6x2(float m, float2 sm3, float2 sm2, float2 sm1, float2 s0, float2 sp1,
                                           float2 sp2, int H, int n, float2 eps) {
  if (H <= 0 || H >= n) return f2(0.f);
  const bool up = m >= 0.f;
  float2 r;
  if (H >= 3 && H <= n - 3) {
    r = weno5x2(sel2(up, sm3, sp2), sel2(up, sm2, sp1), sel2(up, sm1, s0), sel2(up, s0, sm1), sel2(up, sp1, sm2), eps);
  } else if (up) {
    if (H == 1)
      r = mul2(f2(0.5f), add2(sm1, s0));
    else if (H == 2 || H == n - 1)
      r = weno3x2(sm2, sm1, s0, eps);
    else  // H == n-2
      r = weno5x2(sm3, sm2, sm1, s0, sp1, eps);
  } else {
    if (H == n - 1)
      r = mul2(f2(0.5f), add2(s0, sm1));
    else if (H == 1 || H == n - 2)
      r = weno3x2(sp1, s0, sm1, eps);
    else  // H == 2
      r = weno5x2(sp2, sp1, s0, sm1, sm2, eps);
  }
  return mul2(f2(m), r);
}

__device__ __forceinline__ float2 wx2(const Box2& b, int lx, int ly, int lz, float m, float2 eps) {
  return weno_flux_x2(m, b[lz][ly][lx - 3], b[lz][ly][lx - 2], b[lz][ly][lx - 1], b[lz][ly][lx], b[lz][ly][lx + 1],
                      b[lz][ly][lx + 2], eps);
}
__device__ __forceinline__ float2 wy2(const Box2& b, int lx, int ly, int lz, float m, float2 eps) {
  return weno_flux_x2(m, b[lz][ly - 3][lx], b[lz][ly - 2][lx], b[lz][ly - 1][lx], b[lz][ly][lx], b[lz][ly + 1][lx],
                      b[lz][ly + 2][lx], eps);
}
__device__ __forceinline__ float2 wz2(const Box2& b, int lx, int ly, int lz, float m, int H, int n, float2 eps) {
  return vflux6x2(m, b[lz - 3][ly][lx], b[lz - 2][ly][lx], b[lz - 1][ly][lx], b[lz][ly][lx], b[lz + 1][ly][lx],
                  b[lz + 2][ly][lx], H, n, eps);
}

// (theta, qv) staging: all loads in flight before the shared stores
__device__ __forceinline__ void stage_pair(Box2& b, const float* T, const float* q, const Idx& ix, int tid,
                                           bool vec4) {
  if (vec4) {
    float4 vt[IT4], vq[IT4];
#pragma unroll
    for (int r = 0; r < IT4; ++r) {
      const int t = tid + r * NT;
      if (t < NQ4) {
        const int row = t / (BX3 / 4), c4 = t - row * (BX3 / 4);
        const int lz = row / BY3, ly = row - lz * BY3;
        const int g = ix.zc[lz] + ix.y[ly] + ix.x[4 * c4];
        vt[r] = __ldg(reinterpret_cast<const float4*>(T + g));
        vq[r] = __ldg(reinterpret_cast<const float4*>(q + g));
      }
    }
#pragma unroll
    for (int r = 0; r < IT4; ++r) {
      const int t = tid + r * NT;
      if (t < NQ4) {
        const int row = t / (BX3 / 4), c4 = t - row * (BX3 / 4);
        const int lz = row / BY3, ly = row - lz * BY3;
        float4* dst = reinterpret_cast<float4*>(&b[lz][ly][4 * c4]);
        dst[0] = make_float4(vt[r].x, vq[r].x, vt[r].y, vq[r].y);
        dst[1] = make_float4(vt[r].z, vq[r].z, vt[r].w, vq[r].w);
      }
    }
  } else {
    const int lane = tid & 31, warp = tid >> 5;
    const int xa = ix.x[lane];
    const bool tail = lane < BX3 - 32;
    const int xb = tail ? ix.x[32 + lane] : 0;
    float2 va[RPW], vb[RPW];
#pragma unroll
    for (int r = 0; r < RPW; ++r) {
      const int row = warp + r * NWARP;
      if (row < ROWS) {
        const int lz = row / BY3, ly = row - lz * BY3;
        const int base = ix.zc[lz] + ix.y[ly];
        va[r] = make_float2(LD(T, base + xa), LD(q, base + xa));
        vb[r] = tail ? make_float2(LD(T, base + xb), LD(q, base + xb)) : f2(0.f);
      }
    }
#pragma unroll
    for (int r = 0; r < RPW; ++r) {
      const int row = warp + r * NWARP;
      if (row < ROWS) {
        const int lz = row / BY3, ly = row - lz * BY3;
        b[lz][ly][lane] = va[r];
        if (tail) b[lz][ly][32 + lane] = vb[r];
      }
    }
  }
}

__global__ void __launch_bounds__(NT) k_weno_scalars(Dims d, Phys ph, Cols c, State s, ScalarArgs a) {
  __shared__ __align__(16) Box2 bTQ;
  __shared__ float2 xF[TZ][TY][TX + 1];
  __shared__ float2 yF[TZ][TY + 1][TX];
  __shared__ float2 zF[TZ + 1][TY][TX];
  __shared__ Idx ix;
  const int nx = d.nx, ny = d.ny, nz = d.nz, plane = d.plane();
  const int tx = threadIdx.x, ty = threadIdx.y, tz = threadIdx.z;
  const int tid = (tz * TY + ty) * TX + tx, warp = tid >> 5;
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY, k0 = blockIdx.z * TZ;
  build_idx(ix, tid, i0, j0, k0, d);
  __syncthreads();
  // ---- every global load of the block
  stage_pair(bTQ, s.T, s.q, ix, tid, (nx & 3) == 0);
  const int lx = tx + HX, ly = ty + HALO, lz = tz + HALO;
  const int k = k0 + tz;
  const bool inlev = k < nz;
  const bool own = (i0 + tx < nx) && (j0 + ty < ny) && inlev;
  const int id = (inlev ? k : 0) * plane + ix.y[ly] + ix.x[lx];
  // own faces: west (u of the own point), south (v), bottom (w at face k)
  float mx = 0.f, my = 0.f, mz = 0.f;
  if (inlev) {
    const float r = c.rho[k];
    mx = r * LD(s.u, id);
    my = r * LD(s.v, id);
    if (k >= 1) mz = c.rho_face[k] * LD(s.w, id);
  }
  const EdgeFace e = edge_face(warp, tx);
  float me = 0.f;
  int He = 0;
  if (e.which >= 0) {
    const int ke = k0 - HALO + e.lz;
    if (e.which == 0 && ke < nz) me = c.rho[ke] * LD(s.u, ke * plane + ix.y[e.ly] + ix.x[e.lx]);
    if (e.which == 1 && ke < nz) me = c.rho[ke] * LD(s.v, ke * plane + ix.y[e.ly] + ix.x[e.lx]);
    if (e.which == 2) {
      He = ke;
      if (He >= 1 && He < nz) me = c.rho_face[He] * LD(s.w, He * plane + ix.y[e.ly] + ix.x[e.lx]);
    }
  }
  float dv = 0.f, sT = 0.f, sQ = 0.f, T0 = 0.f, Q0 = 0.f;
  if (own) {
    dv = LD(a.div, id);
    if (a.sgsT) {
      sT = LD(a.sgsT, id);
      sQ = LD(a.sgsQ, id);
    }
    T0 = a.T0[id];  // may alias the output: plain loads, same thread
    Q0 = a.q0[id];
  }
  __syncthreads();
  // ---- face fluxes
  const float2 eps = make_float2(kWepsTheta, kWepsQv);
  if (inlev) {
    xF[tz][ty][tx] = wx2(bTQ, lx, ly, lz, mx, eps);
    yF[tz][ty][tx] = wy2(bTQ, lx, ly, lz, my, eps);
  }
  zF[tz][ty][tx] = wz2(bTQ, lx, ly, lz, mz, k, nz, eps);  // zero outside 1..nz-1 (surface flux 0, lid)
  if (e.which == 0)
    xF[e.fk][e.fj][e.fi] = wx2(bTQ, e.lx, e.ly, e.lz, me, eps);
  else if (e.which == 1)
    yF[e.fk][e.fj][e.fi] = wy2(bTQ, e.lx, e.ly, e.lz, me, eps);
  else if (e.which == 2)
    zF[e.fk][e.fj][e.fi] = wz2(bTQ, e.lx, e.ly, e.lz, me, He, nz, eps);
  __syncthreads();
  if (!own) return;
  const float r = c.rho[k];
  const float2 cv = fma2(sub2(zF[tz + 1][ty][tx], zF[tz][ty][tx]), f2(-ph.rdz),
                         fma2(sub2(yF[tz][ty + 1][tx], yF[tz][ty][tx]), f2(-ph.rdy),
                              mul2(sub2(xF[tz][ty][tx + 1], xF[tz][ty][tx]), f2(-ph.rdx))));
  const float2 own2 = bTQ[lz][ly][lx];
  const float aT = (cv.x + own2.x * dv) / r;
  const float aQ = (cv.y + own2.y * dv) / r;
  float Tn = T0 + aT * a.dts, Qn = Q0 + aQ * a.dts, rT = aT, rQ = aQ;
  if (a.sgsT) {
    Tn = Tn + sT * a.dts;
    Qn = Qn + sQ * a.dts;
    rT = rT + sT;
    rQ = rQ + sQ;
  }
  if (a.Tn) a.Tn[id] = Tn;
  if (a.qn) a.qn[id] = Qn;
  if (a.recT) a.recT[id] = rT;
  if (a.recQ) a.recQ[id] = rQ;
}

// ================================================================================================
// theta and qv, vertical march
//
// A block owns 32 x 8 columns (one thread each) and marches up a chunk of levels (as many chunks
// as make one wave of resident blocks: zm_chunk).  For the x and
// y faces of a level it stages that level's plane of theta and qv with a 3-cell halo (40 x 14
// values, x widened to 4-aligned 16-byte pieces) by cp.async into a two-slot ring, the next level's
// plane in flight while the current one is used; the vertical stencil of a thread's own column
// slides through registers (s(k-3) .. s(k+2)), so no z halo is staged.  Each face flux is evaluated
// once: a thread its point's west, south and bottom faces; warp 0 also the 8 east-edge x faces,
// (the mass-flux winds and the stencil's next column value are loaded one level ahead)
// warp 1 the 32 north-edge y faces.  The bottom face of level k+1 is the top face of level k, so a
// level's tendency is completed in the next iteration.  Same reconstructions, mass fluxes and
// expression order as k_weno_scalars.  Needs nx % 4 == 0.
// ================================================================================================
constexpr int ZX = 32, ZY = 8, ZHX = 4, ZHY = 3;
constexpr int ZPX = ZX + 2 * ZHX, ZPY = ZY + 2 * ZHY;   // staged plane 40 x 14
constexpr int ZNT = ZX * ZY;
constexpr int kScalarsZmBlocks = 3;   // resident blocks per SM the theta/qv march is compiled for (measured
                                      // 92 us at 3, 120 us at 4 for 192 x 192 x 96)

// resident blocks on the device (SMs x blocks per SM) of the momentum and theta/qv marches, set by
// init_weno_attributes
int g_zm_slots = 304, g_zs_slots = 608;

// levels per block of a vertical march: as many level chunks as make one wave of resident blocks
// (chunks of at least 8 levels)
inline int zm_chunk(const Dims& d, int slots) {
  const int tiles = ((d.nx + 31) / 32) * ((d.ny + 7) / 8);
  const int nch = max(1, min(slots / tiles, d.nz / 8));
  return (d.nz + nch - 1) / nch;
}
constexpr int ZCHUNKS = ZPY * (ZPX / 4);                 // 16-byte pieces of one field's plane

__device__ __forceinline__ void cp_async16(unsigned sa, const void* gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
constexpr unsigned kSlotBytes = ZPY * ZPX * sizeof(float);   // one staged plane
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// the per-point values a level needs beyond the staged plane (loaded one level ahead)
struct ZLevel {
  float u, v, w, ue, ve;
  float2 top;   // the column value three levels up, for the register stencil
};

// FUSED: also form div(rho0 u) and theta_rho of the state (a.div_out, a.trho_out) instead of reading a.div
template <bool FUSED>
__global__ void __launch_bounds__(ZNT, kScalarsZmBlocks) k_weno_scalars_zm(Dims d, Phys ph, Cols c, State s,
                                                                          ScalarArgs a, int zc) {
  __shared__ __align__(16) float pT[2][ZPY][ZPX];
  __shared__ __align__(16) float pQ[2][ZPY][ZPX];
  __shared__ float2 xF[ZY][ZX + 1];
  __shared__ float2 yF[ZY + 1][ZX];
  __shared__ float sMx[ZY][ZX + 1];  // FUSED: rho0 u on the west faces of the level's cells and the east edge
  __shared__ float sMy[ZY + 1][ZX];  //        rho0 v on the south faces and the north edge
  const int nx = d.nx, ny = d.ny, nz = d.nz, plane = d.plane();
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5, tid = threadIdx.x;
  const int i0 = blockIdx.x * ZX, j0 = blockIdx.y * ZY;
  const int kb = blockIdx.z * zc, ke = min(kb + zc, nz);
  constexpr bool fused = FUSED;
  const int i = i0 + tx, j = j0 + ty;
  const bool col_own = i < nx && j < ny;
  // wrapped coordinates by full modulo: a tile and its halo may reach several periods past a
  // narrow grid (nx, ny >= 4)
  const int ic = pmod(i, nx), jc = pmod(j, ny);   // in-range column for loads
  const int cidx = jc * nx + ic;
  const int eidx = pmod(j0 + tx, ny) * nx + pmod(i0 + ZX, nx);  // warp 0: row tx's east-edge face
  const int nidx = pmod(j0 + ZY, ny) * nx + pmod(i0 + tx, nx);  // warp 1: column tx's north-edge face
  const float2 eps = make_float2(kWepsTheta, kWepsQv);

  // staging: thread t < 140 copies 16-byte piece t (row t / 10, x piece t % 10) of each field's
  // plane, at the same in-plane offset on every level
  const bool stager = tid < ZCHUNKS;
  const int sr = stager ? tid / (ZPX / 4) : 0, sc = 4 * (tid % (ZPX / 4));
  const int soff = pmod(j0 - ZHY + sr, ny) * nx + pmod(i0 - ZHX + sc, nx);
  const unsigned aT = smem_addr(&pT[0][sr][sc]), aQ = smem_addr(&pQ[0][sr][sc]);
  auto stage = [&](int k, int b) {
    if (stager) {
      const size_t o = (size_t)k * plane + soff;
      cp_async16(aT + b * kSlotBytes, s.T + o);
      cp_async16(aQ + b * kSlotBytes, s.q + o);
    }
    cp_async_commit();
  };
  auto colv = [&](int k) {
    const size_t g = (size_t)clampi(k, 0, nz - 1) * plane + cidx;
    return make_float2(__ldg(s.T + g), __ldg(s.q + g));
  };
  // level k's loads (k <= ke; level ke only needs w and the stencil value)
  auto fetch = [&](int k) {
    ZLevel L{0.f, 0.f, 0.f, 0.f, 0.f, make_float2(0.f, 0.f)};
    const size_t base = (size_t)min(k, nz - 1) * plane;
    if (k < nz) {
      L.u = __ldg(s.u + base + cidx);
      L.v = __ldg(s.v + base + cidx);
      if (ty == 0 && tx < ZY) L.ue = __ldg(s.u + base + eidx);
      if (ty == 1) L.ve = __ldg(s.v + base + nidx);
    }
    // faces 0 and nz carry no mass flux but enter the divergence as stored (k_div_trho reads them too)
    if (col_own && (fused || (k >= 1 && k < nz))) L.w = __ldg(s.w + (size_t)k * plane + cidx);
    L.top = colv(k + 3);
    return L;
  };

  stage(kb, 0);
  float2 cl[6];
#pragma unroll
  for (int m = 0; m < 6; ++m) cl[m] = colv(kb - 3 + m);
  ZLevel cur = fetch(kb);
  float2 zprev = f2(0.f), inner = f2(0.f), own = f2(0.f);
  float dv = 0.f, sT = 0.f, sQ = 0.f, T0 = 0.f, Q0 = 0.f;
  for (int k = kb; k <= ke; ++k) {
    const bool lev = k < ke;
    const ZLevel nxt = lev ? fetch(k + 1) : cur;   // one level ahead
    // bottom face of level k (top face of level k-1)
    const float mz = (col_own && k >= 1 && k < nz) ? c.rho_face[k] * cur.w : 0.f;
    const float2 zf = vflux6x2(mz, cl[0], cl[1], cl[2], cl[3], cl[4], cl[5], k, nz, eps);
    if (k > kb && col_own) {  // level k-1 complete
      const int km = k - 1;
      const size_t id = (size_t)km * plane + cidx;
      const float ri = c.rho_inv[km];
      const float2 cv = fma2(sub2(zf, zprev), f2(-ph.rdz), inner);
      const float advT = (cv.x + own.x * dv) * ri;   // 1/rho0 as a correctly rounded column value
      const float advQ = (cv.y + own.y * dv) * ri;
      float Tn = T0 + advT * a.dts, Qn = Q0 + advQ * a.dts, rT = advT, rQ = advQ;
      if (a.sgsT) {
        Tn = Tn + sT * a.dts;
        Qn = Qn + sQ * a.dts;
        rT = rT + sT;
        rQ = rQ + sQ;
      }
      if (a.Tn) a.Tn[id] = Tn;
      if (a.qn) a.qn[id] = Qn;
      if (a.recT) a.recT[id] = rT;
      if (a.recQ) a.recQ[id] = rQ;
    }
    zprev = zf;
    if (!lev) break;
    // x and y faces of level k; threads past the grid's end (partial tiles) evaluate the wrapped
    // faces: their west / south face is the periodic east / north face of the last column / row
    const bool next = k + 1 < ke;
    if (next) stage(k + 1, (k + 1 - kb) & 1);
    const float r = c.rho[k];
    const float mx = r * cur.u, my = r * cur.v, mxe = r * cur.ue, mye = r * cur.ve;
    if (col_own) {  // used when the level is completed, in the next iteration
      const size_t id = (size_t)k * plane + cidx;
      if (!fused) dv = __ldg(a.div + id);
      if (a.sgsT) {
        sT = __ldg(a.sgsT + id);
        sQ = __ldg(a.sgsQ + id);
      }
      T0 = a.T0[id];  // may alias the output: plain loads, same thread, before its write
      Q0 = a.q0[id];
    }
    if (next) cp_async_wait<1>(); else cp_async_wait<0>();
    __syncthreads();
    const int b = (k - kb) & 1;
    const float(&PT)[ZPY][ZPX] = pT[b];
    const float(&PQ)[ZPY][ZPX] = pQ[b];
    auto v2 = [&](int ry, int rx) { return make_float2(PT[ry][rx], PQ[ry][rx]); };
    const int lx = tx + ZHX, ly = ty + ZHY;
    own = v2(ly, lx);
    float dvz = 0.f;
    if (fused) {
      sMx[ty][tx] = mx;
      sMy[ty][tx] = my;
      if (ty == 0 && tx < ZY) sMx[tx][ZX] = mxe;
      if (ty == 1) sMy[ZY][tx] = mye;
      dvz = (c.rho_face0[k + 1] * nxt.w - c.rho_face0[k] * cur.w) * ph.rdz;
    }
    xF[ty][tx] = weno_flux_x2(mx, v2(ly, lx - 3), v2(ly, lx - 2), v2(ly, lx - 1), v2(ly, lx), v2(ly, lx + 1),
                              v2(ly, lx + 2), eps);
    yF[ty][tx] = weno_flux_x2(my, v2(ly - 3, lx), v2(ly - 2, lx), v2(ly - 1, lx), v2(ly, lx), v2(ly + 1, lx),
                              v2(ly + 2, lx), eps);
    if (ty == 0 && tx < ZY) {  // east-edge x face of row tx
      const int ry = tx + ZHY, rx = ZX + ZHX;
      xF[tx][ZX] = weno_flux_x2(mxe, v2(ry, rx - 3), v2(ry, rx - 2), v2(ry, rx - 1), v2(ry, rx), v2(ry, rx + 1),
                                v2(ry, rx + 2), eps);
    }
    if (ty == 1) {  // north-edge y face of column tx
      const int ry = ZY + ZHY, rx = tx + ZHX;
      yF[ZY][tx] = weno_flux_x2(mye, v2(ry - 3, rx), v2(ry - 2, rx), v2(ry - 1, rx), v2(ry, rx), v2(ry + 1, rx),
                                v2(ry + 2, rx), eps);
    }
    __syncthreads();
    inner = fma2(sub2(yF[ty + 1][tx], yF[ty][tx]), f2(-ph.rdy), mul2(sub2(xF[ty][tx + 1], xF[ty][tx]), f2(-ph.rdx)));
    if (fused && col_own) {  // get_divergence (advection.py:200-226) and theta_rho, as k_div_trho forms them
      const float dvx = (sMx[ty][tx + 1] - sMx[ty][tx]) * ph.rdx;
      const float dvy = (sMy[ty + 1][tx] - sMy[ty][tx]) * ph.rdy;
      dv = dvx + dvy + dvz;
      const size_t id = (size_t)k * plane + cidx;
      a.div_out[id] = dv;
      a.trho_out[id] = theta_rho(own.x, own.y, ph.theta_ref);
    }
    // slide the column stencil up one level
#pragma unroll
    for (int m = 0; m < 5; ++m) cl[m] = cl[m + 1];
    cl[5] = cur.top;
    cur = nxt;
  }
}

// ================================================================================================
// u, v, w
// ================================================================================================
struct MomentumArgs {
  const float* div;
  const float* sgs_u;
  const float* sgs_v;
  const float* sgs_w;
  float* Ru;
  float* Rv;
  float* Rw;
  int wmode;
};

// Column values a face at level k needs (loaded before the reconstruction work).
struct LevelCols {
  float r, rm, rf;  // rho0(k), rho0(k-1), rho0 on face k
};

__device__ __forceinline__ LevelCols level_cols(const Cols& c, int k, int nz) {
  LevelCols l{0.f, 0.f, 0.f};
  if (k >= 0 && k < nz) l.r = c.rho[k];
  if (k >= 1 && k <= nz) l.rm = c.rho[k - 1];
  if (k >= 0 && k <= nz) l.rf = c.rho_face[k];
  return l;
}

// face fluxes of u, v and w through the faces (x: which 0, y: 1, z: 2) whose right/upper point
// is box (lx, ly, lz) at level k.  Mass fluxes: advection.py:678-767 (u), :933-1024 (v),
// :1186-1281 (w) and the vertical ones :561-676, :816-931, :1070-1184.
__device__ __forceinline__ void momentum_face(const Box& bu, const Box& bv, const Box& bw, int which, int lx, int ly,
                                              int lz, int k, const LevelCols& L, int nz, float& fu, float& fv,
                                              float& fw) {
  fu = 0.f;
  fv = 0.f;
  fw = 0.f;
  const float eps = kWepsMom;
  if (which == 0) {
    if (k >= 0 && k < nz) {
      const float r = L.r;
      fu = wx(bu, lx, ly, lz, 0.5f * (bu[lz][ly][lx - 1] + bu[lz][ly][lx]) * r, eps);  // cell between u's
      fv = wx(bv, lx, ly, lz, 0.5f * (r * bu[lz][ly - 1][lx] + r * bu[lz][ly][lx]), eps);  // corner
    }
    if (k >= 1 && k < nz) {  // w's lateral faces on interior face levels
      const float m = 0.5f * (L.rm * bu[lz - 1][ly][lx] + L.r * bu[lz][ly][lx]);
      fw = wx(bw, lx, ly, lz, m, eps);
    }
  } else if (which == 1) {
    if (k >= 0 && k < nz) {
      const float r = L.r;
      fu = wy(bu, lx, ly, lz, 0.5f * (r * bv[lz][ly][lx - 1] + r * bv[lz][ly][lx]), eps);  // corner
      fv = wy(bv, lx, ly, lz, 0.5f * (bv[lz][ly - 1][lx] + bv[lz][ly][lx]) * r, eps);      // cell between v's
    }
    if (k >= 1 && k < nz) {
      const float m = 0.5f * (L.rm * bv[lz - 1][ly][lx] + L.r * bv[lz][ly][lx]);
      fw = wy(bw, lx, ly, lz, m, eps);
    }
  } else {
    const int H = k;
    if (H >= 1 && H < nz) {  // u and v columns: faces between cell levels, zero at the ends
      const float rf = L.rf;
      fu = wz(bu, lx, ly, lz, 0.5f * (rf * bw[lz][ly][lx - 1] + rf * bw[lz][ly][lx]), H, nz, eps);
      fv = wz(bv, lx, ly, lz, 0.5f * (rf * bw[lz][ly - 1][lx] + rf * bw[lz][ly][lx]), H, nz, eps);
    }
    if (H >= 1 && H <= nz) {  // w column: its face H is the cell H-1
      fw = wz(bw, lx, ly, lz, 0.5f * (bw[lz - 1][ly][lx] + bw[lz][ly][lx]) * L.rm, H, nz + 1, eps);
    }
  }
}

// 70 KB of shared memory: above the 48 KB static limit, so it is carved from dynamic shared
// memory (opted in once per process by init_weno_attributes).
struct MomentumSmem {
  __align__(16) Box bu;
  __align__(16) Box bv;
  __align__(16) Box bw;
  FluxX xu, xv, xw;
  FluxY yu, yv, yw;
  FluxZ zu, zv, zw;
  Idx ix;
};

__global__ void __launch_bounds__(NT) k_weno_momentum(Dims d, Phys ph, Cols c, State s, MomentumArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  MomentumSmem& S = *reinterpret_cast<MomentumSmem*>(smem_raw);
  Box &bu = S.bu, &bv = S.bv, &bw = S.bw;
  Idx& ix = S.ix;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const int plane = d.plane();
  const int tx = threadIdx.x, ty = threadIdx.y, tz = threadIdx.z;
  const int tid = (tz * TY + ty) * TX + tx, warp = tid >> 5;
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY, k0 = blockIdx.z * TZ;
  build_idx(ix, tid, i0, j0, k0, d);
  __syncthreads();
  {
    Box* const boxes[3] = {&bu, &bv, &bw};
    const float* const src[3] = {s.u, s.v, s.w};
    const int* const zb[3] = {ix.zc, ix.zc, ix.zw};
    stage<3>(boxes, src, zb, ix, tid, (nx & 3) == 0);
  }
  const int lx = tx + HX, ly = ty + HALO, lz = tz + HALO;
  const int k = k0 + tz;
  const bool own = (i0 + tx < nx) && (j0 + ty < ny) && (k <= nz);
  const bool cell = own && k < nz;  // u and v live on cell levels only
  const int col = ix.x[lx], row = ix.y[ly];
  const int id = (k <= nz ? k : 0) * plane + row + col;
  const LevelCols Lown = level_cols(c, k, nz);
  const EdgeFace e = edge_face(warp, tx);
  const int ke = k0 - HALO + e.lz;
  const LevelCols Ledge = level_cols(c, ke, nz);
  float dc = 0.f, dxm = 0.f, dym = 0.f, dzm = 0.f, su = 0.f, sv = 0.f, sw = 0.f;
  if (cell) {
    dc = LD(a.div, id);
    dxm = LD(a.div, k * plane + row + ix.x[lx - 1]);
    dym = LD(a.div, k * plane + ix.y[ly - 1] + col);
    if (a.sgs_u) {
      su = LD(a.sgs_u, id);
      sv = LD(a.sgs_v, id);
    }
  }
  if (own && k >= 1 && k < nz) dzm = LD(a.div, id - plane);
  if (own && a.sgs_w) sw = LD(a.sgs_w, id);
  __syncthreads();
  momentum_face(bu, bv, bw, 0, lx, ly, lz, k, Lown, nz, S.xu[tz][ty][tx], S.xv[tz][ty][tx], S.xw[tz][ty][tx]);
  momentum_face(bu, bv, bw, 1, lx, ly, lz, k, Lown, nz, S.yu[tz][ty][tx], S.yv[tz][ty][tx], S.yw[tz][ty][tx]);
  momentum_face(bu, bv, bw, 2, lx, ly, lz, k, Lown, nz, S.zu[tz][ty][tx], S.zv[tz][ty][tx], S.zw[tz][ty][tx]);
  if (e.which == 0) {
    momentum_face(bu, bv, bw, 0, e.lx, e.ly, e.lz, ke, Ledge, nz, S.xu[e.fk][e.fj][e.fi], S.xv[e.fk][e.fj][e.fi],
                  S.xw[e.fk][e.fj][e.fi]);
  } else if (e.which == 1) {
    momentum_face(bu, bv, bw, 1, e.lx, e.ly, e.lz, ke, Ledge, nz, S.yu[e.fk][e.fj][e.fi], S.yv[e.fk][e.fj][e.fi],
                  S.yw[e.fk][e.fj][e.fi]);
  } else if (e.which == 2) {
    momentum_face(bu, bv, bw, 2, e.lx, e.ly, e.lz, ke, Ledge, nz, S.zu[e.fk][e.fj][e.fi], S.zv[e.fk][e.fj][e.fi],
                  S.zw[e.fk][e.fj][e.fi]);
  }
  __syncthreads();
  if (!own) return;
  if (cell) {
    const float r = Lown.r;
    const float cu = -((S.xu[tz][ty][tx + 1] - S.xu[tz][ty][tx]) * ph.rdx +
                       (S.yu[tz][ty + 1][tx] - S.yu[tz][ty][tx]) * ph.rdy +
                       (S.zu[tz + 1][ty][tx] - S.zu[tz][ty][tx]) * ph.rdz);
    const float cv = -((S.xv[tz][ty][tx + 1] - S.xv[tz][ty][tx]) * ph.rdx +
                       (S.yv[tz][ty + 1][tx] - S.yv[tz][ty][tx]) * ph.rdy +
                       (S.zv[tz + 1][ty][tx] - S.zv[tz][ty][tx]) * ph.rdz);
    float Ru = (cu + bu[lz][ly][lx] * (0.5f * (dxm + dc))) / r;
    float Rv = (cv + bv[lz][ly][lx] * (0.5f * (dym + dc))) / r;
    if (ph.cor_opt) {  // f v at u points, f u at v points (4-point averages)
      const float fv = ph.f_cor * 0.25f * (bv[lz][ly][lx - 1] + bv[lz][ly + 1][lx - 1] + bv[lz][ly][lx] +
                                           bv[lz][ly + 1][lx]);
      float fu = 0.25f * (bu[lz][ly - 1][lx] + bu[lz][ly][lx] + bu[lz][ly - 1][lx + 1] + bu[lz][ly][lx + 1]);
      fu = ph.cor_opt == 2 ? ph.f_cor * (fu - 1.0f) : ph.f_cor * fu;
      Ru = Ru + fv;
      Rv = Rv - fu;
    }
    if (a.sgs_u) {
      Ru = Ru + su;
      Rv = Rv + sv;
    }
    a.Ru[id] = Ru;
    a.Rv[id] = Rv;
  }
  // w on face k
  float adv = 0.f;
  if (k >= 1 && k < nz) {
    const float cw = -((S.xw[tz][ty][tx + 1] - S.xw[tz][ty][tx]) * ph.rdx +
                       (S.yw[tz][ty + 1][tx] - S.yw[tz][ty][tx]) * ph.rdy +
                       (S.zw[tz + 1][ty][tx] - S.zw[tz][ty][tx]) * ph.rdz);
    adv = (cw + bw[lz][ly][lx] * (0.5f * (dzm + dc))) / (0.5f * (Lown.rm + Lown.r));
  }
  if (a.wmode == 1) {
    a.Rw[id] = adv;
    return;
  }
  auto b = [&](int kk) {
    const int q = kk * plane + row + col;
    return buoyancy_at(LD(s.T, q), LD(s.q, q), kk, c);
  };
  float b8w;
  if (k == 0)
    b8w = 1.875f * b(0) - 1.25f * b(1) + 0.375f * b(2);
  else if (k == nz)
    b8w = 1.875f * b(nz - 1) - 1.25f * b(nz - 2) + 0.375f * b(nz - 3);
  else
    b8w = 0.5f * (b(k - 1) + b(k));
  if (a.wmode == 2) {
    a.Rw[id] = b8w;
    return;
  }
  float R = adv + b8w;
  if (a.sgs_w) R = R + sw;
  a.Rw[id] = R;
}

}  // namespace

// ================================================================================================
// u, v and w, vertical march
//
// The tiling of k_weno_scalars_zm: a block owns 32 x 8 columns (one thread each) and marches up a
// chunk of levels.  Level k stages the planes of u and v at cell level k and of w at face level k
// (40 x 14 with halo, cp.async, two-slot ring; the next level's planes in flight while the current
// ones are used); the own columns of u, v and w slide through registers for the vertical stencils.
// Per thread and level: the x and y faces of u, of v and of w as three packed FP32x2 pairs (x face,
// y face, each upwinded by its own mass flux), the bottom faces of u and v as one more pair and the
// bottom face of w alone.  Edge faces: warp 0 the east x faces of u and v, warp 1 the north y faces
// of u and v, warp 2 the north y faces of w, warp 3 the east x faces of w.  Level k-1's tendencies
// are completed once the bottom faces of level k are known; the chunk at the lid adds w's face nz
// (no advection there).  Mass fluxes, reconstructions and output expressions as k_weno_momentum.
// Needs nx % 4 == 0.
// ================================================================================================
__device__ __forceinline__ float2 sel2m(bool p, bool q, float2 a, float2 b) {
  return make_float2(p ? a.x : b.x, q ? a.y : b.y);
}

// (m.x * upwind WENO5 of stencil .x, m.y * upwind WENO5 of stencil .y): two faces with mass fluxes of
// their own
__device__ __forceinline__ float2 weno_flux_2m(float2 m, float2 sm3, float2 sm2, float2 sm1, float2 s0, float2 sp1,
                                               float2 sp2, float2 eps) {
  const bool p = m.x >= 0.f, q = m.y >= 0.f;
  return mul2(m, weno5x2(sel2m(p, q, sm3, sp2), sel2m(p, q, sm2, sp1), sel2m(p, q, sm1, s0), sel2m(p, q, s0, sm1),
                         sel2m(p, q, sp1, sm2), eps));
}

// vflux6 for two columns at the same face H: packed away from the ends, where each column's
// direction picks its own near-boundary rule
__device__ __forceinline__ float2 vflux6_2m(float2 m, float2 sm3, float2 sm2, float2 sm1, float2 s0, float2 sp1,
                                            float2 sp2, int H, int n, float eps) {
  if (H <= 0 || H >= n) return f2(0.f);
  if (H >= 3 && H <= n - 3) return weno_flux_2m(m, sm3, sm2, sm1, s0, sp1, sp2, f2(eps));
  return make_float2(vflux6(m.x, sm3.x, sm2.x, sm1.x, s0.x, sp1.x, sp2.x, H, n, eps),
                     vflux6(m.y, sm3.y, sm2.y, sm1.y, s0.y, sp1.y, sp2.y, H, n, eps));
}


__global__ void __launch_bounds__(ZNT, 3) k_weno_momentum_zm(Dims d, Phys ph, Cols c, State s, MomentumArgs a,
                                                              int zc) {
  __shared__ __align__(16) float pU[2][ZPY][ZPX];
  __shared__ __align__(16) float pV[2][ZPY][ZPX];
  __shared__ __align__(16) float pW[2][ZPY][ZPX];
  __shared__ float2 xUV[ZY][ZX + 1];   // x faces of (u, v)
  __shared__ float2 yUV[ZY + 1][ZX];   // y faces of (u, v)
  __shared__ float xW[ZY][ZX + 1];
  __shared__ float yW[ZY + 1][ZX];
  const int nx = d.nx, ny = d.ny, nz = d.nz, plane = d.plane();
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5, tid = threadIdx.x;
  const int i0 = blockIdx.x * ZX, j0 = blockIdx.y * ZY;
  const int kb = blockIdx.z * zc, ke = min(kb + zc, nz);
  const int i = i0 + tx, j = j0 + ty;
  const bool col_own = i < nx && j < ny;
  const int cidx = pmod(j, ny) * nx + pmod(i, nx);     // threads past the grid's end: the wrapped column
  const int xmidx = pmod(j, ny) * nx + pmod(i - 1, nx);
  const int ymidx = pmod(j - 1, ny) * nx + pmod(i, nx);
  const int eidx = pmod(j0 + tx, ny) * nx + pmod(i0 + ZX, nx);  // warp 3: row tx's east point
  const int nidx = pmod(j0 + ZY, ny) * nx + pmod(i0 + tx, nx);  // warp 2: column tx's north point
  const float eps = kWepsMom;
  // staging: thread t < 140 copies 16-byte piece t of each field's plane (as in k_weno_scalars_zm)
  const bool stager = tid < ZCHUNKS;
  const int sr = stager ? tid / (ZPX / 4) : 0, sc = 4 * (tid % (ZPX / 4));
  const int soff = pmod(j0 - ZHY + sr, ny) * nx + pmod(i0 - ZHX + sc, nx);
  const unsigned sU = smem_addr(&pU[0][sr][sc]), sV = smem_addr(&pV[0][sr][sc]), sW = smem_addr(&pW[0][sr][sc]);
  // stage level k into slot b: u and v at cell level k (the lid's level for k = nz), w at face k
  auto stage = [&](int k, int b) {
    if (stager) {
      const size_t ouv = (size_t)min(k, nz - 1) * plane + soff, ow = (size_t)k * plane + soff;
      cp_async16(sU + b * kSlotBytes, s.u + ouv);
      cp_async16(sV + b * kSlotBytes, s.v + ouv);
      cp_async16(sW + b * kSlotBytes, s.w + ow);
    }
    cp_async_commit();
  };
  auto col = [&](const float* f, int k, int top) { return __ldg(f + (size_t)clampi(k, 0, top) * plane + cidx); };
  auto bq = [&](int k) {
    const size_t q = (size_t)k * plane + cidx;
    return buoyancy_at(__ldg(s.T + q), __ldg(s.q + q), k, c);
  };

  stage(kb, 0);
  float su[6], sv[6], sw[6];   // own columns: levels k-3 .. k+2 (u, v) and faces k-3 .. k+2 (w)
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    su[m] = col(s.u, kb - 3 + m, nz - 1);
    sv[m] = col(s.v, kb - 3 + m, nz - 1);
    sw[m] = col(s.w, kb - 3 + m, nz);
  }
  // edge lanes of w's faces: the level below's u at the east point (warp 3), v at the north point (warp 2)
  float eprev = 0.f;
  if (kb >= 1 && ty == 3 && tx < ZY) eprev = __ldg(s.u + (size_t)(kb - 1) * plane + eidx);
  if (kb >= 1 && ty == 2) eprev = __ldg(s.v + (size_t)(kb - 1) * plane + nidx);
  // the level being completed: x + y flux differences, Coriolis, div (own, i-1, j-1), the level
  // below's div, SGS, buoyancy (and the level below's)
  float2 inUV = f2(0.f);
  float inW = 0.f, corU = 0.f, corV = 0.f, dcC = 0.f, dxC = 0.f, dyC = 0.f, dzC = 0.f;
  float sgU = 0.f, sgV = 0.f, sgW = 0.f, bC = 0.f, bP = 0.f;
  if (kb >= 1 && col_own) {
    dcC = __ldg(a.div + (size_t)(kb - 1) * plane + cidx);
    if (a.wmode != 1) bC = bq(kb - 1);
  }
  float2 zpUV = f2(0.f);   // bottom faces of the level being completed
  float zpW = 0.f;
  const int lx = tx + ZHX, ly = ty + ZHY;
  for (int k = kb; k <= ke; ++k) {
    const bool lev = k < ke;
    const bool more = k + 1 <= ke;
    // the stencils' next column values and this level's per-point inputs, loaded ahead of their use
    const float tu = col(s.u, k + 3, nz - 1), tv = col(s.v, k + 3, nz - 1), tw = col(s.w, k + 3, nz);
    if (more) stage(k + 1, (k + 1 - kb) & 1);
    float dcN = 0.f, dxN = 0.f, dyN = 0.f, sgUN = 0.f, sgVN = 0.f, sgWN = 0.f, TN = 0.f, QN = 0.f;
    if (lev && col_own) {
      const size_t o = (size_t)k * plane;
      dcN = __ldg(a.div + o + cidx);
      dxN = __ldg(a.div + o + xmidx);
      dyN = __ldg(a.div + o + ymidx);
      if (a.sgs_u) {
        sgUN = __ldg(a.sgs_u + o + cidx);
        sgVN = __ldg(a.sgs_v + o + cidx);
      }
      if (a.sgs_w) sgWN = __ldg(a.sgs_w + o + cidx);
      if (a.wmode != 1) {
        TN = __ldg(s.T + o + cidx);
        QN = __ldg(s.q + o + cidx);
      }
    }
    if (more) cp_async_wait<1>(); else cp_async_wait<0>();
    __syncthreads();
    const int b = (k - kb) & 1;
    const float(&PU)[ZPY][ZPX] = pU[b];
    const float(&PV)[ZPY][ZPX] = pV[b];
    const float(&PW)[ZPY][ZPX] = pW[b];
    // bottom faces of level k: u and v through the face between cells k-1 and k (mass flux from w
    // on face k), w through cell k-1
    float2 zUV = f2(0.f);
    if (k >= 1 && k < nz) {
      const float rf = c.rho_face[k];
      const float2 m = make_float2(0.5f * (rf * PW[ly][lx - 1] + rf * PW[ly][lx]),
                                   0.5f * (rf * PW[ly - 1][lx] + rf * PW[ly][lx]));
      zUV = vflux6_2m(m, make_float2(su[0], sv[0]), make_float2(su[1], sv[1]), make_float2(su[2], sv[2]),
                      make_float2(su[3], sv[3]), make_float2(su[4], sv[4]), make_float2(su[5], sv[5]), k, nz, eps);
    }
    const float zW = (k >= 1) ? vflux6(0.5f * (sw[2] + sw[3]) * c.rho[k - 1], sw[0], sw[1], sw[2], sw[3], sw[4],
                                       sw[5], k, nz + 1, eps)
                              : 0.f;
    if (k > kb && col_own) {  // level k-1 complete
      const int kk = k - 1;
      const size_t id = (size_t)kk * plane + cidx;
      const float ri = c.rho_inv[kk];   // 1/rho0, 1/rho0 on the face: correctly rounded column values
      const float2 cuv = fma2(sub2(zUV, zpUV), f2(-ph.rdz), inUV);
      float Ru = (cuv.x + su[2] * (0.5f * (dxC + dcC))) * ri;
      float Rv = (cuv.y + sv[2] * (0.5f * (dyC + dcC))) * ri;
      if (ph.cor_opt) {
        Ru = Ru + corU;
        Rv = Rv - corV;
      }
      if (a.sgs_u) {
        Ru = Ru + sgU;
        Rv = Rv + sgV;
      }
      a.Ru[id] = Ru;
      a.Rv[id] = Rv;
      float adv = 0.f;   // w on face kk
      if (kk >= 1) {
        const float cw = fmaf(zW - zpW, -ph.rdz, inW);
        adv = (cw + sw[2] * (0.5f * (dzC + dcC))) * c.rho_w_inv[kk];
      }
      float Rw = adv;
      if (a.wmode != 1) {
        const float b8w = kk == 0 ? 1.875f * bq(0) - 1.25f * bq(1) + 0.375f * bq(2) : 0.5f * (bP + bC);
        if (a.wmode == 2) {
          Rw = b8w;
        } else {
          Rw = adv + b8w;
          if (a.sgs_w) Rw = Rw + sgW;
        }
      }
      a.Rw[id] = Rw;
    }
    zpUV = zUV;
    zpW = zW;
    if (!lev) break;
    // x and y faces of level k
    const float r = c.rho[k], rm = k >= 1 ? c.rho[k - 1] : 0.f;
    auto xs = [&](const float(&P)[ZPY][ZPX], int ry, int rx, int o) { return P[ry][rx + o]; };
    {
      const float2 mu = make_float2(0.5f * (PU[ly][lx - 1] + PU[ly][lx]) * r,          // cell between u's
                                    0.5f * (r * PV[ly][lx - 1] + r * PV[ly][lx]));     // corner
      const float2 fu = weno_flux_2m(mu, make_float2(PU[ly][lx - 3], PU[ly - 3][lx]),
                                     make_float2(PU[ly][lx - 2], PU[ly - 2][lx]),
                                     make_float2(PU[ly][lx - 1], PU[ly - 1][lx]), make_float2(PU[ly][lx], PU[ly][lx]),
                                     make_float2(PU[ly][lx + 1], PU[ly + 1][lx]),
                                     make_float2(PU[ly][lx + 2], PU[ly + 2][lx]), f2(eps));
      const float2 mv = make_float2(0.5f * (r * PU[ly - 1][lx] + r * PU[ly][lx]),      // corner
                                    0.5f * (PV[ly - 1][lx] + PV[ly][lx]) * r);         // cell between v's
      const float2 fv = weno_flux_2m(mv, make_float2(PV[ly][lx - 3], PV[ly - 3][lx]),
                                     make_float2(PV[ly][lx - 2], PV[ly - 2][lx]),
                                     make_float2(PV[ly][lx - 1], PV[ly - 1][lx]), make_float2(PV[ly][lx], PV[ly][lx]),
                                     make_float2(PV[ly][lx + 1], PV[ly + 1][lx]),
                                     make_float2(PV[ly][lx + 2], PV[ly + 2][lx]), f2(eps));
      xUV[ty][tx] = make_float2(fu.x, fv.x);
      yUV[ty][tx] = make_float2(fu.y, fv.y);
    }
    if (k >= 1 && k < nz) {  // w's lateral faces on interior face levels
      const float2 mw = make_float2(0.5f * (rm * su[2] + r * su[3]), 0.5f * (rm * sv[2] + r * sv[3]));
      const float2 fw = weno_flux_2m(mw, make_float2(PW[ly][lx - 3], PW[ly - 3][lx]),
                                     make_float2(PW[ly][lx - 2], PW[ly - 2][lx]),
                                     make_float2(PW[ly][lx - 1], PW[ly - 1][lx]), make_float2(PW[ly][lx], PW[ly][lx]),
                                     make_float2(PW[ly][lx + 1], PW[ly + 1][lx]),
                                     make_float2(PW[ly][lx + 2], PW[ly + 2][lx]), f2(eps));
      xW[ty][tx] = fw.x;
      yW[ty][tx] = fw.y;
    } else {
      xW[ty][tx] = 0.f;
      yW[ty][tx] = 0.f;
    }
    float corUN = 0.f, corVN = 0.f;
    if (ph.cor_opt) {  // f v at u points, f u at v points (4-point averages)
      corUN = ph.f_cor * 0.25f * (PV[ly][lx - 1] + PV[ly + 1][lx - 1] + PV[ly][lx] + PV[ly + 1][lx]);
      const float fu = 0.25f * (PU[ly - 1][lx] + PU[ly][lx] + PU[ly - 1][lx + 1] + PU[ly][lx + 1]);
      corVN = ph.cor_opt == 2 ? ph.f_cor * (fu - 1.0f) : ph.f_cor * fu;
    }
    if (ty == 0 && tx < ZY) {  // east x faces of u and v, row tx
      const int ry = tx + ZHY, rx = ZX + ZHX;
      const float2 m = make_float2(0.5f * (PU[ry][rx - 1] + PU[ry][rx]) * r,
                                   0.5f * (r * PU[ry - 1][rx] + r * PU[ry][rx]));
      xUV[tx][ZX] = weno_flux_2m(m, make_float2(xs(PU, ry, rx, -3), xs(PV, ry, rx, -3)),
                                 make_float2(xs(PU, ry, rx, -2), xs(PV, ry, rx, -2)),
                                 make_float2(xs(PU, ry, rx, -1), xs(PV, ry, rx, -1)),
                                 make_float2(xs(PU, ry, rx, 0), xs(PV, ry, rx, 0)),
                                 make_float2(xs(PU, ry, rx, 1), xs(PV, ry, rx, 1)),
                                 make_float2(xs(PU, ry, rx, 2), xs(PV, ry, rx, 2)), f2(eps));
    } else if (ty == 1) {  // north y faces of u and v, column tx
      const int ry = ZY + ZHY, rx = tx + ZHX;
      const float2 m = make_float2(0.5f * (r * PV[ry][rx - 1] + r * PV[ry][rx]),
                                   0.5f * (PV[ry - 1][rx] + PV[ry][rx]) * r);
      yUV[ZY][tx] = weno_flux_2m(m, make_float2(PU[ry - 3][rx], PV[ry - 3][rx]),
                                 make_float2(PU[ry - 2][rx], PV[ry - 2][rx]),
                                 make_float2(PU[ry - 1][rx], PV[ry - 1][rx]), make_float2(PU[ry][rx], PV[ry][rx]),
                                 make_float2(PU[ry + 1][rx], PV[ry + 1][rx]),
                                 make_float2(PU[ry + 2][rx], PV[ry + 2][rx]), f2(eps));
    } else if (ty == 2) {  // north y faces of w, column tx
      const int ry = ZY + ZHY, rx = tx + ZHX;
      float f = 0.f;
      if (k >= 1 && k < nz)
        f = weno_flux(0.5f * (rm * eprev + r * PV[ry][rx]), PW[ry - 3][rx], PW[ry - 2][rx], PW[ry - 1][rx],
                      PW[ry][rx], PW[ry + 1][rx], PW[ry + 2][rx], eps);
      yW[ZY][tx] = f;
      eprev = PV[ry][rx];
    } else if (ty == 3 && tx < ZY) {  // east x faces of w, row tx
      const int ry = tx + ZHY, rx = ZX + ZHX;
      float f = 0.f;
      if (k >= 1 && k < nz)
        f = weno_flux(0.5f * (rm * eprev + r * PU[ry][rx]), PW[ry][rx - 3], PW[ry][rx - 2], PW[ry][rx - 1],
                      PW[ry][rx], PW[ry][rx + 1], PW[ry][rx + 2], eps);
      xW[tx][ZX] = f;
      eprev = PU[ry][rx];
    }
    __syncthreads();
    inUV = fma2(sub2(yUV[ty + 1][tx], yUV[ty][tx]), f2(-ph.rdy), mul2(sub2(xUV[ty][tx + 1], xUV[ty][tx]), f2(-ph.rdx)));
    inW = fmaf(yW[ty + 1][tx] - yW[ty][tx], -ph.rdy, (xW[ty][tx + 1] - xW[ty][tx]) * -ph.rdx);
    corU = corUN;
    corV = corVN;
    dzC = dcC;
    dcC = dcN;
    dxC = dxN;
    dyC = dyN;
    sgU = sgUN;
    sgV = sgVN;
    sgW = sgWN;
    bP = bC;
    if (a.wmode != 1 && col_own) bC = buoyancy_at(TN, QN, k, c);
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      su[m] = su[m + 1];
      sv[m] = sv[m + 1];
      sw[m] = sw[m + 1];
    }
    su[5] = tu;
    sv[5] = tv;
    sw[5] = tw;
  }
  if (ke == nz && col_own) {  // w on the lid: no advection
    const size_t id = (size_t)nz * plane + cidx;
    float Rw = 0.f;
    if (a.wmode != 1) {
      const float b8w = 1.875f * bq(nz - 1) - 1.25f * bq(nz - 2) + 0.375f * bq(nz - 3);
      Rw = b8w;
      if (a.wmode == 0) {
        Rw = 0.f + b8w;
        if (a.sgs_w) Rw = Rw + __ldg(a.sgs_w + id);
      }
    }
    a.Rw[id] = Rw;
  }
}

cudaError_t launch_adv_scalars(const Dims& d, const Phys& ph, const Cols& c, State in, const float* div,
                               const float* T0, const float* q0, Sgs sgs, float dts, SlowOut out, cudaStream_t st,
                               float* div_out, float* trho_out) {
  ScalarArgs a{div, T0, q0, sgs.T, sgs.q, out.T_next, out.q_next, out.dT, out.dq, dts, nullptr, nullptr};
  if (div_out && d.nx % 4 != 0) {  // no vertical march: the divergence and theta_rho first
    cudaError_t e = launch_div_trho(d, ph, c, in, div_out, trho_out, st);
    if (e != cudaSuccess) return e;
    a.div = div_out;
  } else if (div_out) {
    a.div_out = div_out;
    a.trho_out = trho_out;
  }
  if (d.nx % 4 == 0) {  // the vertical march (16-byte plane pieces need nx % 4 == 0)
    const int zc = zm_chunk(d, g_zs_slots);
    dim3 g((d.nx + ZX - 1) / ZX, (d.ny + ZY - 1) / ZY, (d.nz + zc - 1) / zc);
    if (a.div_out)
      k_weno_scalars_zm<true><<<g, ZNT, 0, st>>>(d, ph, c, in, a, zc);
    else
      k_weno_scalars_zm<false><<<g, ZNT, 0, st>>>(d, ph, c, in, a, zc);
    return cudaGetLastError();
  }
  dim3 g((d.nx + TX - 1) / TX, (d.ny + TY - 1) / TY, (d.nz + TZ - 1) / TZ);
  k_weno_scalars<<<g, dim3(TX, TY, TZ), 0, st>>>(d, ph, c, in, a);
  return cudaGetLastError();
}

cudaError_t launch_adv_momentum(const Dims& d, const Phys& ph, const Cols& c, State in, const float* div, Sgs sgs,
                                float* Ru, float* Rv, float* Rw, int wmode, cudaStream_t st) {
  MomentumArgs a{div, sgs.u, sgs.v, sgs.w, Ru, Rv, Rw, wmode};
  if (d.nx % 4 == 0) {  // the vertical march
    const int zc = zm_chunk(d, g_zm_slots);
    dim3 gz((d.nx + ZX - 1) / ZX, (d.ny + ZY - 1) / ZY, (d.nz + zc - 1) / zc);
    k_weno_momentum_zm<<<gz, ZNT, 0, st>>>(d, ph, c, in, a, zc);
    return cudaGetLastError();
  }
  dim3 g((d.nx + TX - 1) / TX, (d.ny + TY - 1) / TY, (d.nz + 1 + TZ - 1) / TZ);
  k_weno_momentum<<<g, dim3(TX, TY, TZ), sizeof(MomentumSmem), st>>>(d, ph, c, in, a);
  return cudaGetLastError();
}

cudaError_t init_weno_attributes() {
  cudaError_t e = cudaFuncSetAttribute(k_weno_momentum, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)sizeof(MomentumSmem));
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0, nb = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_weno_momentum_zm, ZNT, 0)) != cudaSuccess) return e;
  g_zm_slots = sms * max(nb, 1);
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_weno_scalars_zm<true>, ZNT, 0)) != cudaSuccess)
    return e;
  g_zs_slots = sms * max(nb, 1);
  return cudaSuccess;
}

}  // namespace lexgb
