// kernels_acoustic.cu - one forward-backward acoustic sub-step (sound_rk_step0/1/2,
// one_step_integration.py:519-556, :638-675, :757-794):
//
//   u,v,w <- u,v,w + dtau (PGF(pi') + rhs)        pressure_gradient_force, pressure_gradient_coriolis.py:7-37
//   w = 0 on the bottom and lid faces             set_w_bc, boundary_conditions.py:104-109
//   pi'   <- pi' + 1.1 dtau (-(Rd/Cv)(pi0 + pi'_s) div(u) + adv_pi)
//                                                 get_divergence2 / advection_pi, advection.py:152-236
//
// One thread per cell computes the new pi' of its cell and the new winds on the cell's west,
// south and bottom faces; the winds on the east, north and top faces that its divergence needs
// are recomputed from the same inputs, so one launch is one whole sub-step.  Inputs and outputs
// are distinct buffers (the caller ping-pongs).
#include "lexgb_internal.cuh"

namespace lexgb {

namespace {

constexpr int BX = 32, BY = 4, BZ = 2;
#define LD(p, idx) __ldg((p) + (idx))

// x points per thread of the vectorised sub-step kernel
#ifndef ACOUSTIC_VEC
#define ACOUSTIC_VEC 4
#endif

constexpr float kHalfCp = (float)(0.5 * kCp);
constexpr float kRdCv = (float)(kRd / kCv);

// -Cp * 0.5*(trho_a + trho_b) * ((p_a - p_b) * rd)
__device__ __forceinline__ float pgf(float tra, float trb, float pa, float pb, float rd) {
  return -kHalfCp * (tra + trb) * ((pa - pb) * rd);
}

// new u on the west face of cell (i, j, k), i.e. u(i)
__device__ __forceinline__ float u_new(const Dims& d, const Phys& ph, const AcousticIn& a, int i, int j, int k,
                                       float dtau) {
  const int im = wrap(i - 1, d.nx);
  const int c0 = d.at(i, j, k), cm = d.at(im, j, k);
  const float f = pgf(LD(a.trho, c0), LD(a.trho, cm), LD(a.p, c0), LD(a.p, cm), ph.rdx);
  return LD(a.u, c0) + (f + LD(a.Ru, c0)) * dtau;
}

__device__ __forceinline__ float v_new(const Dims& d, const Phys& ph, const AcousticIn& a, int i, int j, int k,
                                       float dtau) {
  const int jm = wrap(j - 1, d.ny);
  const int c0 = d.at(i, j, k), cm = d.at(i, jm, k);
  const float f = pgf(LD(a.trho, c0), LD(a.trho, cm), LD(a.p, c0), LD(a.p, cm), ph.rdy);
  return LD(a.v, c0) + (f + LD(a.Rv, c0)) * dtau;
}

// new w on face f (0..nz); zero on the bottom and the lid
__device__ __forceinline__ float w_new(const Dims& d, const Phys& ph, const AcousticIn& a, int i, int j, int f,
                                       float dtau) {
  if (f <= 0 || f >= d.nz) return 0.f;
  const int c0 = d.at(i, j, f), cm = d.at(i, j, f - 1);
  const float g = pgf(LD(a.trho, c0), LD(a.trho, cm), LD(a.p, c0), LD(a.p, cm), ph.rdz);
  return LD(a.w, c0) + (g + LD(a.Rw, c0)) * dtau;
}

// advection_pi at cell (i, j, k) given the face winds around it and pi'_s (advection.py:152-197)
__device__ __forceinline__ float adv_pi(const Dims& d, const Phys& ph, const Cols& c, const float* __restrict__ ps,
                                        int i, int j, int k, float uw, float ue, float vs, float vn, float wb,
                                        float wt) {
  const int im = wrap(i - 1, d.nx), ip = wrap(i + 1, d.nx);
  const int jm = wrap(j - 1, d.ny), jp = wrap(j + 1, d.ny);
  const float p0 = LD(ps, d.at(i, j, k));
  const float gxw = (p0 - LD(ps, d.at(im, j, k))) * ph.rdx;
  const float gxe = (LD(ps, d.at(ip, j, k)) - p0) * ph.rdx;
  const float gys = (p0 - LD(ps, d.at(i, jm, k))) * ph.rdy;
  const float gyn = (LD(ps, d.at(i, jp, k)) - p0) * ph.rdy;
  // w * dpi/dz on the bounding faces, zero on the bottom and the lid
  const float wzb = (k == 0) ? 0.f : wb * (c.dpi0dz[k] + (p0 - LD(ps, d.at(i, j, k - 1))) * ph.rdz);
  const float wzt = (k + 1 >= d.nz) ? 0.f : wt * (c.dpi0dz[k + 1] + (LD(ps, d.at(i, j, k + 1)) - p0) * ph.rdz);
  return -(0.5f * (ue * gxe + uw * gxw) + 0.5f * (vn * gyn + vs * gys) +
           (0.5f * wzb * c.rho_face[k] + 0.5f * wzt * c.rho_face[k + 1]) / c.rho[k]);
}

__global__ void __launch_bounds__(BX* BY* BZ) k_acoustic(Dims d, Phys ph, Cols c, AcousticIn a, AcousticOut o,
                                                       float dtau) {
  const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y, k = blockIdx.z * BZ + threadIdx.z;
  if (i >= d.nx || j >= d.ny || k >= d.nz) return;
  const int ip = wrap(i + 1, d.nx), jp = wrap(j + 1, d.ny);
  const float uw = u_new(d, ph, a, i, j, k, dtau);
  const float ue = u_new(d, ph, a, ip, j, k, dtau);
  const float vs = v_new(d, ph, a, i, j, k, dtau);
  const float vn = v_new(d, ph, a, i, jp, k, dtau);
  const float wb = w_new(d, ph, a, i, j, k, dtau);
  const float wt = w_new(d, ph, a, i, j, k + 1, dtau);
  const float div = (ue - uw) * ph.rdx + (vn - vs) * ph.rdy + (wt - wb) * ph.rdz;
  const int id = d.at(i, j, k);
  const float ap = adv_pi(d, ph, c, a.ps, i, j, k, uw, ue, vs, vn, wb, wt);
  const float dpdt = -kRdCv * ((c.pi0[k] + LD(a.ps, id)) * div) + ap;
  o.p[id] = LD(a.p, id) + (kDivDamp * dpdt) * dtau;
  o.u[id] = uw;
  o.v[id] = vs;
  o.w[id] = wb;
  if (k == d.nz - 1) o.w[d.at(i, j, d.nz)] = 0.f;
}

// Vectorised sub-step: each thread owns V (4 or 2) consecutive x points of one (j, k) row and
// moves every field with V-wide loads/stores (needs nx % V == 0).  Same arithmetic as k_acoustic.
template <int V>
struct VecT;
template <>
struct VecT<4> {
  typedef float4 T;
};
template <>
struct VecT<2> {
  typedef float2 T;
};

template <int V>
__device__ __forceinline__ void ldv(const float* __restrict__ p, int idx, float (&o)[V]) {
  typedef typename VecT<V>::T T;
  const T t = __ldg(reinterpret_cast<const T*>(p + idx));
  const float* f = reinterpret_cast<const float*>(&t);
#pragma unroll
  for (int l = 0; l < V; ++l) o[l] = f[l];
}

template <int V>
__device__ __forceinline__ void stv(float* p, int idx, const float (&v)[V]) {
  typedef typename VecT<V>::T T;
  T t;
  float* f = reinterpret_cast<float*>(&t);
#pragma unroll
  for (int l = 0; l < V; ++l) f[l] = v[l];
  *reinterpret_cast<T*>(p + idx) = t;
}

template <int V>
__device__ __forceinline__ void zero(float (&o)[V]) {
#pragma unroll
  for (int l = 0; l < V; ++l) o[l] = 0.f;
}

template <int V>
__global__ void __launch_bounds__(256) k_acoustic_vec(Dims d, Phys ph, Cols c, AcousticIn a, AcousticOut o,
                                                      float dtau) {
  const int nq = d.nx / V;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (q >= nq || j >= d.ny) return;
  const int nx = d.nx, nz = d.nz;
  const int i0 = q * V;
  const int iw = wrap(i0 - 1, nx), ie = wrap(i0 + V, nx);
  const int jm = wrap(j - 1, d.ny), jp = wrap(j + 1, d.ny);
  const int r0 = (k * d.ny + j) * nx;
  const int rs = (k * d.ny + jm) * nx, rn = (k * d.ny + jp) * nx;
  const int rb = r0 - d.plane(), rt = r0 + d.plane();
  const bool has_b = k > 0, has_t = k + 1 < nz;
  float P[V], TR[V], U[V], RU[V], Vv[V], RV[V], PS[V], TS[V], VN[V], RVN[V], PN[V], TN[V];
  float W[V], RW[V], PB[V], TB[V], WT[V], RWT[V], PT[V], TT[V], S0[V], SS[V], SN[V], SB[V], ST[V];
  // centre row
  ldv<V>(a.p, r0 + i0, P);
  ldv<V>(a.trho, r0 + i0, TR);
  ldv<V>(a.u, r0 + i0, U);
  ldv<V>(a.Ru, r0 + i0, RU);
  const float pW = __ldg(a.p + r0 + iw), pE = __ldg(a.p + r0 + ie);
  const float tW = __ldg(a.trho + r0 + iw), tE = __ldg(a.trho + r0 + ie);
  const float uE = __ldg(a.u + r0 + ie), ruE = __ldg(a.Ru + r0 + ie);
  // south / north rows
  ldv<V>(a.v, r0 + i0, Vv);
  ldv<V>(a.Rv, r0 + i0, RV);
  ldv<V>(a.p, rs + i0, PS);
  ldv<V>(a.trho, rs + i0, TS);
  ldv<V>(a.v, rn + i0, VN);
  ldv<V>(a.Rv, rn + i0, RVN);
  ldv<V>(a.p, rn + i0, PN);
  ldv<V>(a.trho, rn + i0, TN);
  // bottom / top levels
  if (has_b) {
    ldv<V>(a.w, r0 + i0, W);
    ldv<V>(a.Rw, r0 + i0, RW);
    ldv<V>(a.p, rb + i0, PB);
    ldv<V>(a.trho, rb + i0, TB);
    ldv<V>(a.ps, rb + i0, SB);
  } else {
    zero<V>(W); zero<V>(RW); zero<V>(PB); zero<V>(TB); zero<V>(SB);
  }
  if (has_t) {
    ldv<V>(a.w, rt + i0, WT);
    ldv<V>(a.Rw, rt + i0, RWT);
    ldv<V>(a.p, rt + i0, PT);
    ldv<V>(a.trho, rt + i0, TT);
    ldv<V>(a.ps, rt + i0, ST);
  } else {
    zero<V>(WT); zero<V>(RWT); zero<V>(PT); zero<V>(TT); zero<V>(ST);
  }
  // pi'_s for advection_pi
  ldv<V>(a.ps, r0 + i0, S0);
  ldv<V>(a.ps, rs + i0, SS);
  ldv<V>(a.ps, rn + i0, SN);
  const float sW = __ldg(a.ps + r0 + iw), sE = __ldg(a.ps + r0 + ie);

  float un[V + 1];
  {
    float pc[V + 2], tc[V + 2], uc[V + 1], rc[V + 1];
    pc[0] = pW;
    tc[0] = tW;
    pc[V + 1] = pE;
    tc[V + 1] = tE;
    uc[V] = uE;
    rc[V] = ruE;
#pragma unroll
    for (int l = 0; l < V; ++l) {
      pc[l + 1] = P[l];
      tc[l + 1] = TR[l];
      uc[l] = U[l];
      rc[l] = RU[l];
    }
#pragma unroll
    for (int l = 0; l <= V; ++l) un[l] = uc[l] + (pgf(tc[l + 1], tc[l], pc[l + 1], pc[l], ph.rdx) + rc[l]) * dtau;
  }
  float sc[V + 2];
  sc[0] = sW;
  sc[V + 1] = sE;
#pragma unroll
  for (int l = 0; l < V; ++l) sc[l + 1] = S0[l];
  const float rho = c.rho[k], rfb = c.rho_face[k], rft = c.rho_face[k + 1];
  const float dzb = c.dpi0dz[k], dzt = c.dpi0dz[k + 1], pi0 = c.pi0[k];
  float outp[V], outv[V], outw[V], outu[V];
#pragma unroll
  for (int l = 0; l < V; ++l) {
    const float p0 = P[l], t0 = TR[l];
    const float vs = Vv[l] + (pgf(t0, TS[l], p0, PS[l], ph.rdy) + RV[l]) * dtau;
    const float vn = VN[l] + (pgf(TN[l], t0, PN[l], p0, ph.rdy) + RVN[l]) * dtau;
    const float wb = has_b ? W[l] + (pgf(t0, TB[l], p0, PB[l], ph.rdz) + RW[l]) * dtau : 0.f;
    const float wt = has_t ? WT[l] + (pgf(TT[l], t0, PT[l], p0, ph.rdz) + RWT[l]) * dtau : 0.f;
    const float div = (un[l + 1] - un[l]) * ph.rdx + (vn - vs) * ph.rdy + (wt - wb) * ph.rdz;
    const float s0 = sc[l + 1];
    const float gxw = (s0 - sc[l]) * ph.rdx, gxe = (sc[l + 2] - s0) * ph.rdx;
    const float gys = (s0 - SS[l]) * ph.rdy, gyn = (SN[l] - s0) * ph.rdy;
    const float wzb = has_b ? wb * (dzb + (s0 - SB[l]) * ph.rdz) : 0.f;
    const float wzt = has_t ? wt * (dzt + (ST[l] - s0) * ph.rdz) : 0.f;
    const float ap = -(0.5f * (un[l + 1] * gxe + un[l] * gxw) + 0.5f * (vn * gyn + vs * gys) +
                       (0.5f * wzb * rfb + 0.5f * wzt * rft) / rho);
    const float dpdt = -kRdCv * ((pi0 + s0) * div) + ap;
    outp[l] = p0 + (kDivDamp * dpdt) * dtau;
    outv[l] = vs;
    outw[l] = wb;
    outu[l] = un[l];
  }
  stv<V>(o.p, r0 + i0, outp);
  stv<V>(o.u, r0 + i0, outu);
  stv<V>(o.v, r0 + i0, outv);
  stv<V>(o.w, r0 + i0, outw);
  if (k == nz - 1) {
    float z[V];
    zero<V>(z);
    stv<V>(o.w, rt + i0, z);
  }
}

// ================================================================================================
// Two sub-steps per launch (temporal blocking).
//
// A block owns a 32 x 4 x 4 tile T of cells.  The first sub-step is evaluated on T grown by one
// cell on every side (E), which is exactly what the second sub-step reads, so the two sub-steps
// need their inputs once: pi', theta_rho and pi'_s on T grown by two cells (boxes), and the
// winds and slow tendencies on the faces of E.  Each field crosses DRAM once per two sub-steps.
//
// Phases (one __syncthreads between each):
//   0  stage the boxes; every thread also loads the old winds and R of the faces it owns
//   1  winds after sub-step 1 on all faces of E               -> uf / vf / wf
//   2  pi' after sub-step 1 on the cells of E                 -> pm
//   3  winds after sub-step 2 on the faces of T (in place in uf / vf / wf; own faces stored)
//   4  pi' after sub-step 2 on T (stored)
// ================================================================================================
namespace tb {
constexpr int TX = 32, TY = 4, TZ = 4, NT = TX * TY * TZ;
constexpr int EX = TX + 2, EY = TY + 2, EZ = TZ + 2;  // E: cells i0-1 .. i0+TX
constexpr int HBX = TX + 4, HBY = TY + 4, HBZ = TZ + 4;  // boxes: cells i0-2 .. i0+TX+1
constexpr int NU = (EX + 1) * EY * EZ;                // x faces of E
constexpr int NV = EX * (EY + 1) * EZ;                // y faces of E
constexpr int NW = EX * EY * (EZ + 1);                // z faces of E
constexpr int IU = (NU + NT - 1) / NT, IV = (NV + NT - 1) / NT, IW = (NW + NT - 1) / NT;
constexpr int NB = HBX * HBY * HBZ;
constexpr int IB = (NB + NT - 1) / NT;

struct Smem {
  float P[HBZ][HBY][HBX], TR[HBZ][HBY][HBX], PS[HBZ][HBY][HBX];
  float uf[EZ][EY][EX + 1];  // u on x faces i0-1+f
  float vf[EZ][EY + 1][EX];  // v on y faces j0-1+f
  float wf[EZ + 1][EY][EX];  // w on z faces k0-1+f
  float pm[EZ][EY][EX];      // pi' after sub-step 1 on E
  int gx[HBX];                // x index of box column (i0-2+b), wrapped
  int gy[HBY];                // (j0-2+b) wrapped, times nx
  int gz[HBZ];                // (k0-2+b) clamped to 0..nz-1, times nx*ny
};
}  // namespace tb

__global__ void __launch_bounds__(tb::NT) k_acoustic_pair(Dims d, Phys ph, Cols c, AcousticIn a, AcousticOut o,
                                                        float dtau) {
  using namespace tb;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Smem& S = *reinterpret_cast<Smem*>(smem_raw);
  const int nx = d.nx, ny = d.ny, nz = d.nz, plane = d.plane();
  const int tid = threadIdx.x;
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY, k0 = blockIdx.z * TZ;
  if (tid < HBX) {
    int i = (i0 - 2 + tid) % nx;
    S.gx[tid] = i < 0 ? i + nx : i;
  } else if (tid < HBX + HBY) {
    int j = (j0 - 2 + (tid - HBX)) % ny;
    S.gy[tid - HBX] = (j < 0 ? j + ny : j) * nx;
  } else if (tid < HBX + HBY + HBZ) {
    S.gz[tid - HBX - HBY] = clampi(k0 - 2 + (tid - HBX - HBY), 0, nz - 1) * plane;
  }
  __syncthreads();

  // ---------------------------------------------------------------- phase 0: loads
  float stP[IB], stT[IB], stS[IB];
#pragma unroll
  for (int q = 0; q < IB; ++q) {
    const int t = tid + q * NT;
    if (t < NB) {
      const int bx = t % HBX, by = (t / HBX) % HBY, bz = t / (HBX * HBY);
      const int g = S.gz[bz] + S.gy[by] + S.gx[bx];
      stP[q] = __ldg(a.p + g);
      stT[q] = __ldg(a.trho + g);
      stS[q] = __ldg(a.ps + g);
    }
  }
  // owned faces: x face item t -> (f, ey, ez) with global face i0-1+f, row j0-1+ey, level k0-1+ez
  float u0[IU], ru[IU], v0[IV], rv[IV], w0[IW], rw[IW];
#pragma unroll
  for (int q = 0; q < IU; ++q) {
    const int t = tid + q * NT;
    u0[q] = ru[q] = 0.f;
    if (t < NU) {
      const int f = t % (EX + 1), ey = (t / (EX + 1)) % EY, ez = t / ((EX + 1) * EY);
      const int k = k0 - 1 + ez;
      if (k >= 0 && k < nz) {
        const int g = S.gz[ez + 1] + S.gy[ey + 1] + S.gx[f + 1];
        u0[q] = __ldg(a.u + g);
        ru[q] = __ldg(a.Ru + g);
      }
    }
  }
#pragma unroll
  for (int q = 0; q < IV; ++q) {
    const int t = tid + q * NT;
    v0[q] = rv[q] = 0.f;
    if (t < NV) {
      const int ex = t % EX, f = (t / EX) % (EY + 1), ez = t / (EX * (EY + 1));
      const int k = k0 - 1 + ez;
      if (k >= 0 && k < nz) {
        const int g = S.gz[ez + 1] + S.gy[f + 1] + S.gx[ex + 1];
        v0[q] = __ldg(a.v + g);
        rv[q] = __ldg(a.Rv + g);
      }
    }
  }
#pragma unroll
  for (int q = 0; q < IW; ++q) {
    const int t = tid + q * NT;
    w0[q] = rw[q] = 0.f;
    if (t < NW) {
      const int ex = t % EX, ey = (t / EX) % EY, f = t / (EX * EY);
      const int kf = k0 - 1 + f;  // face level
      if (kf > 0 && kf < nz) {
        const int g = kf * plane + S.gy[ey + 1] + S.gx[ex + 1];
        w0[q] = __ldg(a.w + g);
        rw[q] = __ldg(a.Rw + g);
      }
    }
  }
#pragma unroll
  for (int q = 0; q < IB; ++q) {
    const int t = tid + q * NT;
    if (t < NB) {
      (&S.P[0][0][0])[t] = stP[q];
      (&S.TR[0][0][0])[t] = stT[q];
      (&S.PS[0][0][0])[t] = stS[q];
    }
  }
  __syncthreads();

  // ---------------------------------------------------------------- phase 1: winds after sub-step 1 on E
#pragma unroll
  for (int q = 0; q < IU; ++q) {
    const int t = tid + q * NT;
    if (t < NU) {
      const int f = t % (EX + 1), ey = (t / (EX + 1)) % EY, ez = t / ((EX + 1) * EY);
      const int bx = f + 1, by = ey + 1, bz = ez + 1;  // box cell right of the face
      const float g = pgf(S.TR[bz][by][bx], S.TR[bz][by][bx - 1], S.P[bz][by][bx], S.P[bz][by][bx - 1], ph.rdx);
      (&S.uf[0][0][0])[t] = u0[q] + (g + ru[q]) * dtau;
    }
  }
#pragma unroll
  for (int q = 0; q < IV; ++q) {
    const int t = tid + q * NT;
    if (t < NV) {
      const int ex = t % EX, f = (t / EX) % (EY + 1), ez = t / (EX * (EY + 1));
      const int bx = ex + 1, by = f + 1, bz = ez + 1;
      const float g = pgf(S.TR[bz][by][bx], S.TR[bz][by - 1][bx], S.P[bz][by][bx], S.P[bz][by - 1][bx], ph.rdy);
      (&S.vf[0][0][0])[t] = v0[q] + (g + rv[q]) * dtau;
    }
  }
#pragma unroll
  for (int q = 0; q < IW; ++q) {
    const int t = tid + q * NT;
    if (t < NW) {
      const int ex = t % EX, ey = (t / EX) % EY, f = t / (EX * EY);
      const int kf = k0 - 1 + f;
      float wn = 0.f;
      if (kf > 0 && kf < nz) {
        const int bx = ex + 1, by = ey + 1, bz = f + 1;
        const float g = pgf(S.TR[bz][by][bx], S.TR[bz - 1][by][bx], S.P[bz][by][bx], S.P[bz - 1][by][bx], ph.rdz);
        wn = w0[q] + (g + rw[q]) * dtau;
      }
      (&S.wf[0][0][0])[t] = wn;
    }
  }
  __syncthreads();

  // ---------------------------------------------------------------- phase 2: pi' after sub-step 1 on E
  constexpr int NE = EX * EY * EZ;
  for (int t = tid; t < NE; t += NT) {
    const int ex = t % EX, ey = (t / EX) % EY, ez = t / (EX * EY);
    const int k = k0 - 1 + ez;
    if (k < 0 || k >= nz) continue;
    const int bx = ex + 1, by = ey + 1, bz = ez + 1;
    const float uw = S.uf[ez][ey][ex], ue = S.uf[ez][ey][ex + 1];
    const float vs = S.vf[ez][ey][ex], vn = S.vf[ez][ey + 1][ex];
    const float wb = S.wf[ez][ey][ex], wt = S.wf[ez + 1][ey][ex];
    const float div = (ue - uw) * ph.rdx + (vn - vs) * ph.rdy + (wt - wb) * ph.rdz;
    const float s0 = S.PS[bz][by][bx];
    const float gxw = (s0 - S.PS[bz][by][bx - 1]) * ph.rdx, gxe = (S.PS[bz][by][bx + 1] - s0) * ph.rdx;
    const float gys = (s0 - S.PS[bz][by - 1][bx]) * ph.rdy, gyn = (S.PS[bz][by + 1][bx] - s0) * ph.rdy;
    const float wzb = (k == 0) ? 0.f : wb * (c.dpi0dz[k] + (s0 - S.PS[bz - 1][by][bx]) * ph.rdz);
    const float wzt = (k + 1 >= nz) ? 0.f : wt * (c.dpi0dz[k + 1] + (S.PS[bz + 1][by][bx] - s0) * ph.rdz);
    const float ap = -(0.5f * (ue * gxe + uw * gxw) + 0.5f * (vn * gyn + vs * gys) +
                       (0.5f * wzb * c.rho_face[k] + 0.5f * wzt * c.rho_face[k + 1]) / c.rho[k]);
    const float dpdt = -kRdCv * ((c.pi0[k] + s0) * div) + ap;
    S.pm[ez][ey][ex] = S.P[bz][by][bx] + (kDivDamp * dpdt) * dtau;
  }
  __syncthreads();

  // ---------------------------------------------------------------- phase 3: winds after sub-step 2 on T
#pragma unroll
  for (int q = 0; q < IU; ++q) {
    const int t = tid + q * NT;
    if (t < NU) {
      const int f = t % (EX + 1), ey = (t / (EX + 1)) % EY, ez = t / ((EX + 1) * EY);
      if (f >= 1 && f <= TX + 1 && ey >= 1 && ey <= TY && ez >= 1 && ez <= TZ) {
        const int k = k0 - 1 + ez;
        if (k < nz) {
          const int bx = f + 1, by = ey + 1, bz = ez + 1;
          const float g = pgf(S.TR[bz][by][bx], S.TR[bz][by][bx - 1], S.pm[ez][ey][f], S.pm[ez][ey][f - 1], ph.rdx);
          const float un = S.uf[ez][ey][f] + (g + ru[q]) * dtau;
          S.uf[ez][ey][f] = un;
          const int i = i0 - 1 + f, j = j0 - 1 + ey;
          if (f <= TX && i < nx && j < ny) o.u[k * plane + j * nx + i] = un;
        }
      }
    }
  }
#pragma unroll
  for (int q = 0; q < IV; ++q) {
    const int t = tid + q * NT;
    if (t < NV) {
      const int ex = t % EX, f = (t / EX) % (EY + 1), ez = t / (EX * (EY + 1));
      if (ex >= 1 && ex <= TX && f >= 1 && f <= TY + 1 && ez >= 1 && ez <= TZ) {
        const int k = k0 - 1 + ez;
        if (k < nz) {
          const int bx = ex + 1, by = f + 1, bz = ez + 1;
          const float g = pgf(S.TR[bz][by][bx], S.TR[bz][by - 1][bx], S.pm[ez][f][ex], S.pm[ez][f - 1][ex], ph.rdy);
          const float vn = S.vf[ez][f][ex] + (g + rv[q]) * dtau;
          S.vf[ez][f][ex] = vn;
          const int i = i0 - 1 + ex, j = j0 - 1 + f;
          if (f <= TY && i < nx && j < ny) o.v[k * plane + j * nx + i] = vn;
        }
      }
    }
  }
#pragma unroll
  for (int q = 0; q < IW; ++q) {
    const int t = tid + q * NT;
    if (t < NW) {
      const int ex = t % EX, ey = (t / EX) % EY, f = t / (EX * EY);
      if (ex >= 1 && ex <= TX && ey >= 1 && ey <= TY && f >= 1 && f <= TZ + 1) {
        const int kf = k0 - 1 + f;
        float wn = 0.f;
        if (kf > 0 && kf < nz) {
          const int bx = ex + 1, by = ey + 1, bz = f + 1;
          const float g = pgf(S.TR[bz][by][bx], S.TR[bz - 1][by][bx], S.pm[f][ey][ex], S.pm[f - 1][ey][ex], ph.rdz);
          wn = S.wf[f][ey][ex] + (g + rw[q]) * dtau;
        }
        S.wf[f][ey][ex] = wn;
        const int i = i0 - 1 + ex, j = j0 - 1 + ey;
        if (i < nx && j < ny && kf <= nz && (f <= TZ || kf == nz)) o.w[kf * plane + j * nx + i] = wn;
      }
    }
  }
  __syncthreads();

  // ---------------------------------------------------------------- phase 4: pi' after sub-step 2 on T
  {
    const int tx = tid % TX, ty = (tid / TX) % TY, tz = tid / (TX * TY);
    const int i = i0 + tx, j = j0 + ty, k = k0 + tz;
    if (i >= nx || j >= ny || k >= nz) return;
    const int ex = tx + 1, ey = ty + 1, ez = tz + 1;
    const int bx = tx + 2, by = ty + 2, bz = tz + 2;
    const float uw = S.uf[ez][ey][ex], ue = S.uf[ez][ey][ex + 1];
    const float vs = S.vf[ez][ey][ex], vn = S.vf[ez][ey + 1][ex];
    const float wb = S.wf[ez][ey][ex], wt = S.wf[ez + 1][ey][ex];
    const float div = (ue - uw) * ph.rdx + (vn - vs) * ph.rdy + (wt - wb) * ph.rdz;
    const float s0 = S.PS[bz][by][bx];
    const float gxw = (s0 - S.PS[bz][by][bx - 1]) * ph.rdx, gxe = (S.PS[bz][by][bx + 1] - s0) * ph.rdx;
    const float gys = (s0 - S.PS[bz][by - 1][bx]) * ph.rdy, gyn = (S.PS[bz][by + 1][bx] - s0) * ph.rdy;
    const float wzb = (k == 0) ? 0.f : wb * (c.dpi0dz[k] + (s0 - S.PS[bz - 1][by][bx]) * ph.rdz);
    const float wzt = (k + 1 >= nz) ? 0.f : wt * (c.dpi0dz[k + 1] + (S.PS[bz + 1][by][bx] - s0) * ph.rdz);
    const float ap = -(0.5f * (ue * gxe + uw * gxw) + 0.5f * (vn * gyn + vs * gys) +
                       (0.5f * wzb * c.rho_face[k] + 0.5f * wzt * c.rho_face[k + 1]) / c.rho[k]);
    const float dpdt = -kRdCv * ((c.pi0[k] + s0) * div) + ap;
    o.p[k * plane + j * nx + i] = S.pm[ez][ey][ex] + (kDivDamp * dpdt) * dtau;
  }
}

__global__ void k_diag_pgf(Dims d, Phys ph, Cols c, const float* __restrict__ p, const float* __restrict__ trho,
                           float* pu, float* pv, float* pw) {
  const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y, f = blockIdx.z * BZ + threadIdx.z;
  if (i >= d.nx || j >= d.ny || f > d.nz) return;
  if (f < d.nz) {
    const int c0 = d.at(i, j, f);
    const int cw = d.at(wrap(i - 1, d.nx), j, f), cs = d.at(i, wrap(j - 1, d.ny), f);
    pu[c0] = pgf(LD(trho, c0), LD(trho, cw), LD(p, c0), LD(p, cw), ph.rdx);
    pv[c0] = pgf(LD(trho, c0), LD(trho, cs), LD(p, c0), LD(p, cs), ph.rdy);
  }
  float g = 0.f;
  if (f > 0 && f < d.nz) {
    const int c0 = d.at(i, j, f), cb = d.at(i, j, f - 1);
    g = pgf(LD(trho, c0), LD(trho, cb), LD(p, c0), LD(p, cb), ph.rdz);
  }
  pw[d.at(i, j, f)] = g;
}

__global__ void k_diag_advpi(Dims d, Phys ph, Cols c, const float* __restrict__ ps, const float* __restrict__ u,
                             const float* __restrict__ v, const float* __restrict__ w, float* out) {
  const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y, k = blockIdx.z * BZ + threadIdx.z;
  if (i >= d.nx || j >= d.ny || k >= d.nz) return;
  const int ip = wrap(i + 1, d.nx), jp = wrap(j + 1, d.ny);
  const float wb = (k == 0) ? 0.f : LD(w, d.at(i, j, k));
  const float wt = (k + 1 >= d.nz) ? 0.f : LD(w, d.at(i, j, k + 1));
  out[d.at(i, j, k)] = adv_pi(d, ph, c, ps, i, j, k, LD(u, d.at(i, j, k)), LD(u, d.at(ip, j, k)),
                              LD(v, d.at(i, j, k)), LD(v, d.at(i, jp, k)), wb, wt);
}

}  // namespace

cudaError_t launch_acoustic(const Dims& d, const Phys& ph, const Cols& c, AcousticIn in, AcousticOut out, float dtau,
                            cudaStream_t st) {
  constexpr int VW = ACOUSTIC_VEC;
  if (d.nx % VW == 0) {
    const int nq = d.nx / VW;
    dim3 b(VW == 4 ? 16 : 32, VW == 4 ? 16 : 8, 1);
    dim3 g((nq + b.x - 1) / b.x, (d.ny + b.y - 1) / b.y, d.nz);
    k_acoustic_vec<VW><<<g, b, 0, st>>>(d, ph, c, in, out, dtau);
    return cudaGetLastError();
  }
  dim3 g((d.nx + BX - 1) / BX, (d.ny + BY - 1) / BY, (d.nz + BZ - 1) / BZ);
  k_acoustic<<<g, dim3(BX, BY, BZ), 0, st>>>(d, ph, c, in, out, dtau);
  return cudaGetLastError();
}

cudaError_t launch_acoustic_pair(const Dims& d, const Phys& ph, const Cols& c, AcousticIn in, AcousticOut out,
                                 float dtau, cudaStream_t st) {
  dim3 g((d.nx + tb::TX - 1) / tb::TX, (d.ny + tb::TY - 1) / tb::TY, (d.nz + tb::TZ - 1) / tb::TZ);
  k_acoustic_pair<<<g, tb::NT, sizeof(tb::Smem), st>>>(d, ph, c, in, out, dtau);
  return cudaGetLastError();
}

cudaError_t init_acoustic_attributes() {
  return cudaFuncSetAttribute(k_acoustic_pair, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(tb::Smem));
}

cudaError_t launch_diag_pgf(const Dims& d, const Phys& ph, const Cols& c, const float* p, const float* trho,
                            float* pu, float* pv, float* pw, cudaStream_t st) {
  dim3 g((d.nx + BX - 1) / BX, (d.ny + BY - 1) / BY, (d.nz + 1 + BZ - 1) / BZ);
  k_diag_pgf<<<g, dim3(BX, BY, BZ), 0, st>>>(d, ph, c, p, trho, pu, pv, pw);
  return cudaGetLastError();
}

cudaError_t launch_diag_advpi(const Dims& d, const Phys& ph, const Cols& c, const float* ps, const float* u,
                              const float* v, const float* w, float* out, cudaStream_t st) {
  dim3 g((d.nx + BX - 1) / BX, (d.ny + BY - 1) / BY, (d.nz + BZ - 1) / BZ);
  k_diag_advpi<<<g, dim3(BX, BY, BZ), 0, st>>>(d, ph, c, ps, u, v, w, out);
  return cudaGetLastError();
}

}  // namespace lexgb
