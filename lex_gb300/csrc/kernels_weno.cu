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

cudaError_t launch_adv_scalars(const Dims& d, const Phys& ph, const Cols& c, State in, const float* div,
                               const float* T0, const float* q0, Sgs sgs, float dts, SlowOut out, cudaStream_t st) {
  ScalarArgs a{div, T0, q0, sgs.T, sgs.q, out.T_next, out.q_next, out.dT, out.dq, dts};
  dim3 g((d.nx + TX - 1) / TX, (d.ny + TY - 1) / TY, (d.nz + TZ - 1) / TZ);
  k_weno_scalars<<<g, dim3(TX, TY, TZ), 0, st>>>(d, ph, c, in, a);
  return cudaGetLastError();
}

cudaError_t launch_adv_momentum(const Dims& d, const Phys& ph, const Cols& c, State in, const float* div, Sgs sgs,
                                float* Ru, float* Rv, float* Rw, int wmode, cudaStream_t st) {
  MomentumArgs a{div, sgs.u, sgs.v, sgs.w, Ru, Rv, Rw, wmode};
  dim3 g((d.nx + TX - 1) / TX, (d.ny + TY - 1) / TY, (d.nz + 1 + TZ - 1) / TZ);
  k_weno_momentum<<<g, dim3(TX, TY, TZ), sizeof(MomentumSmem), st>>>(d, ph, c, in, a);
  return cudaGetLastError();
}

cudaError_t init_weno_attributes() {
  return cudaFuncSetAttribute(k_weno_momentum, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)sizeof(MomentumSmem));
}

}  // namespace lexgb
