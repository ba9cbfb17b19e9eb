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
// levels per thread of the vertical-march sub-step kernel (0: one level per thread)
#ifndef ACOUSTIC_ZMARCH
#define ACOUSTIC_ZMARCH 0
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
           (0.5f * wzb * c.rho_face[k] + 0.5f * wzt * c.rho_face[k + 1]) * c.rho_inv[k]);
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
                                                      float dtau, int rev) {
  const int nq = d.nx / V;
  // rev: blocks walk the grid in reverse order, so that a sub-step following one in forward order
  // starts on the fields its predecessor wrote last (still in L2)
  const int bx = rev ? gridDim.x - 1 - blockIdx.x : blockIdx.x;
  const int by = rev ? gridDim.y - 1 - blockIdx.y : blockIdx.y;
  const int q = bx * blockDim.x + threadIdx.x;
  const int j = by * blockDim.y + threadIdx.y;
  const int k = rev ? gridDim.z - 1 - blockIdx.z : blockIdx.z;
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
  const float rho = c.rho[k], rhoi = c.rho_inv[k], rfb = c.rho_face[k], rft = c.rho_face[k + 1];
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
                       (0.5f * wzb * rfb + 0.5f * wzt * rft) * rhoi);
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

// Vertical-march sub-step: each thread owns V consecutive x points of row j and walks the levels
// kb .. kb+kc-1.  pi', theta_rho and pi'_s of the level above and the new w on the top face are
// carried to the next level (the new w on face k+1 is the next level's bottom wind, same
// operands), so each level loads 17 vectors instead of 25.  Same arithmetic as k_acoustic_vec.
template <int V>
__global__ void __launch_bounds__(256) k_acoustic_zm(Dims d, Phys ph, Cols c, AcousticIn a, AcousticOut o,
                                                     float dtau, int kc) {
  const int nq = d.nx / V;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (q >= nq || j >= d.ny) return;
  const int nx = d.nx, nz = d.nz, plane = d.plane();
  const int kb = blockIdx.z * kc, ke = min(kb + kc, nz);
  const int i0 = q * V;
  const int iw = wrap(i0 - 1, nx), ie = wrap(i0 + V, nx);
  const int rc = j * nx, rs = wrap(j - 1, d.ny) * nx, rn = wrap(j + 1, d.ny) * nx;
  float P[V], TR[V], S0[V], PB[V], TB[V], SB[V], WB[V];
  ldv<V>(a.p, kb * plane + rc + i0, P);
  ldv<V>(a.trho, kb * plane + rc + i0, TR);
  ldv<V>(a.ps, kb * plane + rc + i0, S0);
  if (kb > 0) {
    const int rb = (kb - 1) * plane + rc + i0;
    float W[V], RW[V];
    ldv<V>(a.p, rb, PB);
    ldv<V>(a.trho, rb, TB);
    ldv<V>(a.ps, rb, SB);
    ldv<V>(a.w, kb * plane + rc + i0, W);
    ldv<V>(a.Rw, kb * plane + rc + i0, RW);
#pragma unroll
    for (int l = 0; l < V; ++l) WB[l] = W[l] + (pgf(TR[l], TB[l], P[l], PB[l], ph.rdz) + RW[l]) * dtau;
  } else {
    zero<V>(PB); zero<V>(TB); zero<V>(SB); zero<V>(WB);
  }
  for (int k = kb; k < ke; ++k) {
    const int r0 = k * plane;
    const bool has_b = k > 0, has_t = k + 1 < nz;
    float U[V], RU[V], Vv[V], RV[V], VN[V], RVN[V], PS[V], TS[V], SS[V], PN[V], TN[V], SN[V];
    float PT[V], TT[V], ST[V], WT[V], RWT[V];
    ldv<V>(a.u, r0 + rc + i0, U);
    ldv<V>(a.Ru, r0 + rc + i0, RU);
    ldv<V>(a.v, r0 + rc + i0, Vv);
    ldv<V>(a.Rv, r0 + rc + i0, RV);
    ldv<V>(a.v, r0 + rn + i0, VN);
    ldv<V>(a.Rv, r0 + rn + i0, RVN);
    ldv<V>(a.p, r0 + rs + i0, PS);
    ldv<V>(a.trho, r0 + rs + i0, TS);
    ldv<V>(a.ps, r0 + rs + i0, SS);
    ldv<V>(a.p, r0 + rn + i0, PN);
    ldv<V>(a.trho, r0 + rn + i0, TN);
    ldv<V>(a.ps, r0 + rn + i0, SN);
    const float pW = __ldg(a.p + r0 + rc + iw), pE = __ldg(a.p + r0 + rc + ie);
    const float tW = __ldg(a.trho + r0 + rc + iw), tE = __ldg(a.trho + r0 + rc + ie);
    const float uE = __ldg(a.u + r0 + rc + ie), ruE = __ldg(a.Ru + r0 + rc + ie);
    const float sW = __ldg(a.ps + r0 + rc + iw), sE = __ldg(a.ps + r0 + rc + ie);
    if (has_t) {
      const int rt = r0 + plane + rc + i0;
      ldv<V>(a.p, rt, PT);
      ldv<V>(a.trho, rt, TT);
      ldv<V>(a.ps, rt, ST);
      ldv<V>(a.w, rt, WT);
      ldv<V>(a.Rw, rt, RWT);
    } else {
      zero<V>(PT); zero<V>(TT); zero<V>(ST); zero<V>(WT); zero<V>(RWT);
    }
    float un[V + 1];
    {
      float pc[V + 2], tc[V + 2], uc[V + 1], rcu[V + 1];
      pc[0] = pW;
      tc[0] = tW;
      pc[V + 1] = pE;
      tc[V + 1] = tE;
      uc[V] = uE;
      rcu[V] = ruE;
#pragma unroll
      for (int l = 0; l < V; ++l) {
        pc[l + 1] = P[l];
        tc[l + 1] = TR[l];
        uc[l] = U[l];
        rcu[l] = RU[l];
      }
#pragma unroll
      for (int l = 0; l <= V; ++l) un[l] = uc[l] + (pgf(tc[l + 1], tc[l], pc[l + 1], pc[l], ph.rdx) + rcu[l]) * dtau;
    }
    float sc[V + 2];
    sc[0] = sW;
    sc[V + 1] = sE;
#pragma unroll
    for (int l = 0; l < V; ++l) sc[l + 1] = S0[l];
    const float rho = c.rho[k], rhoi = c.rho_inv[k], rfb = c.rho_face[k], rft = c.rho_face[k + 1];
    const float dzb = c.dpi0dz[k], dzt = c.dpi0dz[k + 1], pi0 = c.pi0[k];
    float outp[V], outv[V], wt[V];
#pragma unroll
    for (int l = 0; l < V; ++l) {
      const float p0 = P[l], t0 = TR[l];
      const float vs = Vv[l] + (pgf(t0, TS[l], p0, PS[l], ph.rdy) + RV[l]) * dtau;
      const float vn = VN[l] + (pgf(TN[l], t0, PN[l], p0, ph.rdy) + RVN[l]) * dtau;
      const float wb = WB[l];
      wt[l] = has_t ? WT[l] + (pgf(TT[l], t0, PT[l], p0, ph.rdz) + RWT[l]) * dtau : 0.f;
      const float div = (un[l + 1] - un[l]) * ph.rdx + (vn - vs) * ph.rdy + (wt[l] - wb) * ph.rdz;
      const float s0 = sc[l + 1];
      const float gxw = (s0 - sc[l]) * ph.rdx, gxe = (sc[l + 2] - s0) * ph.rdx;
      const float gys = (s0 - SS[l]) * ph.rdy, gyn = (SN[l] - s0) * ph.rdy;
      const float wzb = has_b ? wb * (dzb + (s0 - SB[l]) * ph.rdz) : 0.f;
      const float wzt = has_t ? wt[l] * (dzt + (ST[l] - s0) * ph.rdz) : 0.f;
      const float ap = -(0.5f * (un[l + 1] * gxe + un[l] * gxw) + 0.5f * (vn * gyn + vs * gys) +
                         (0.5f * wzb * rfb + 0.5f * wzt * rft) * rhoi);
      const float dpdt = -kRdCv * ((pi0 + s0) * div) + ap;
      outp[l] = p0 + (kDivDamp * dpdt) * dtau;
      outv[l] = vs;
    }
    float outu[V];
#pragma unroll
    for (int l = 0; l < V; ++l) outu[l] = un[l];
    stv<V>(o.p, r0 + rc + i0, outp);
    stv<V>(o.u, r0 + rc + i0, outu);
    stv<V>(o.v, r0 + rc + i0, outv);
    stv<V>(o.w, r0 + rc + i0, WB);
    if (k == nz - 1) {
      float z[V];
      zero<V>(z);
      stv<V>(o.w, r0 + plane + rc + i0, z);
    }
#pragma unroll
    for (int l = 0; l < V; ++l) {
      PB[l] = P[l]; TB[l] = TR[l]; SB[l] = S0[l];
      P[l] = PT[l]; TR[l] = TT[l]; S0[l] = ST[l];
      WB[l] = wt[l];
    }
  }
}

// ================================================================================================
// Two sub-steps per launch (temporal blocking in 2.5-D).
//
// A block owns a 32 x 16 tile of columns O and a chunk kb .. ke-1 of levels, and walks the
// chunk upwards.  Sub-step 1 is evaluated on O grown by one column on every side (E), which is
// what sub-step 2 on O reads; sub-step 2 runs one level behind sub-step 1 (its top-face wind
// needs sub-step 1's pi' one level up).  Each input field crosses DRAM once per two sub-steps.
//
// Iteration n (three barriers):
//   X  sub-step 1 winds of level n on E: u on west faces, v on south faces, w on the top face
//      n+1, and the east / north edge faces                   -> U1 / V1 / W1 rings
//      sub-step 2 pi' of level n-2 on O and the stores of level n-2's outputs
//   Y  sub-step 1 pi' of level n on E                         -> P1 ring
//   Z  sub-step 2 winds of level n-1 on O (top face only at level kb-1) -> U2 / V2 / W2
// The input planes (pi', theta_rho, pi'_s on O grown by two columns; u, v, w and the slow
// tendencies on E's faces) move with cp.async as aligned 16-byte row pieces into shared-memory
// rings: level n+2's cell planes are issued before X, level n+1's face planes before Y, and
// both are waited for at the end of the iteration.  Sub-step 2's own slow tendencies and pi'_s
// values are loaded into registers one iteration before use.
// Needs nx % 4 == 0.  Sub-step 1 runs on levels kb-1 .. ke (within 0 .. nz-1).
// ================================================================================================
namespace tb {
constexpr int OX = 32, OY = 16, NT = OX * OY;     // owned columns (one thread each)
constexpr int EX = OX + 2, EY = OY + 2, NE = EX * EY;
constexpr int RWD = 40, NG = RWD / 4;            // staged row: x = i0-4 .. i0+35, 10 groups of 4
constexpr int RY = OY + 4;                       // cell-plane rows: y = j0-2 .. j0+OY+1
constexpr int FU = OY + 2, FV = OY + 3;          // rows of the u / w / R planes (E rows), v planes (j0-1 .. j0+OY+1)
constexpr int Q_CELL = RY * NG, Q_U = FU * NG, Q_V = FV * NG;
constexpr int N1A = NE + EY + EX;                // sub-step 1 wind items: E cells + east + north edge faces
constexpr int N2A = NT + OY + OX;                // sub-step 2 wind items: O cells + east + north edge faces
static_assert(NT <= NE && NE + EY + EX <= 2 * NT, "each thread owns one E cell and at most one more item");

struct Smem {
  float P0[3][RY][RWD], TR[4][RY][RWD], PS[4][RY][RWD];
  float U0[FU][RWD], RU[FU][RWD], W0[FU][RWD], RW[FU][RWD], V0[FV][RWD], RV[FV][RWD];
  float U1[2][EY][EX + 1];  // u after sub-step 1 on x faces i0-1+f, E rows (ring by level)
  float V1[2][EY + 1][EX];  // v after sub-step 1 on y faces j0-1+f, E columns
  float W1[2][EY][EX];      // w after sub-step 1 (ring by face level)
  float P1[2][EY][EX];      // pi' after sub-step 1 (ring by level)
  float U2[OY][OX + 1], V2[OY + 1][OX], W2[2][OY][OX];
  int gx[NG];               // wrapped x of group g (i0-4+4g)
  int gy[RY];               // wrapped y of cell-plane row r (j0-2+r), times nx
};

__device__ __forceinline__ int pmod(int i, int n) {
  i %= n;
  return i < 0 ? i + n : i;
}

__device__ __forceinline__ void cp16(void* dst, const void* src) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

constexpr int ROWS_CELL = 3 * RY;                  // staged rows per level: cell planes
constexpr int ROWS_FACE = 4 * FU + 2 * FV;         // face planes

__device__ __forceinline__ void copy_row(float* dst, const float* src_row, const int* gx) {
#pragma unroll
  for (int g = 0; g < NG; ++g) cp16(dst + 4 * g, src_row + gx[g]);
}

// pi', theta_rho, pi'_s of level lc into their ring slots: one thread per staged row
__device__ __forceinline__ void stage_cells(Smem& S, const AcousticIn& a, int plane, int lc, int tid) {
  if (tid < ROWS_CELL) {
    const int f = tid / RY, row = tid - f * RY;
    const float* src = f == 0 ? a.p : (f == 1 ? a.trho : a.ps);
    float* dst = f == 0 ? S.P0[lc % 3][row] : (f == 1 ? S.TR[lc % 4][row] : S.PS[lc % 4][row]);
    copy_row(dst, src + lc * plane + S.gy[row], S.gx);
  }
}

// u, R_u, v, R_v of level lf and w, R_w of face level lw (lw < 0: skipped); threads from 64 up
__device__ __forceinline__ void stage_faces(Smem& S, const AcousticIn& a, int plane, int lf, int lw, int tid) {
  const int q = tid - 64;
  if (q < 0 || q >= ROWS_FACE) return;
  int f, row;
  if (q < 4 * FU) {
    f = q / FU;
    row = q - f * FU;
  } else {
    f = 4 + (q - 4 * FU) / FV;
    row = q - 4 * FU - (f - 4) * FV;
  }
  const int lev = (f == 2 || f == 3) ? lw : lf;
  if (lev < 0) return;
  const float* src;
  float* dst;
  switch (f) {
    case 0: src = a.u; dst = S.U0[row]; break;
    case 1: src = a.Ru; dst = S.RU[row]; break;
    case 2: src = a.w; dst = S.W0[row]; break;
    case 3: src = a.Rw; dst = S.RW[row]; break;
    case 4: src = a.v; dst = S.V0[row]; break;
    default: src = a.Rv; dst = S.RV[row]; break;
  }
  copy_row(dst, src + lev * plane + S.gy[row + 1], S.gx);  // these planes start at y = j0-1
}
}  // namespace tb

__global__ void __launch_bounds__(tb::NT, 2) k_acoustic_pair(Dims d, Phys ph, Cols c, AcousticIn a, AcousticOut o,
                                                           float dtau, int kc) {
  using namespace tb;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Smem& S = *reinterpret_cast<Smem*>(smem_raw);
  const int nx = d.nx, ny = d.ny, nz = d.nz, plane = d.plane();
  const int tid = threadIdx.x;
  const int i0 = blockIdx.x * OX, j0 = blockIdx.y * OY;
  const int kb = blockIdx.z * kc, ke = min(kb + kc, nz);
  const int n0 = max(kb - 1, 0), n1 = min(ke, nz - 1);
  const float rdx = ph.rdx, rdy = ph.rdy, rdz = ph.rdz;
  if (tid < NG) S.gx[tid] = pmod(i0 - 4 + 4 * tid, nx);
  if (tid >= 32 && tid < 32 + RY) S.gy[tid - 32] = pmod(j0 - 2 + (tid - 32), ny) * nx;
  // ---- loop-invariant per-thread offsets
  // sub-step 2: owned column (ox, oy) and its wrapped neighbours
  const int ox = tid % OX, oy = tid / OX;
  const int gxo = pmod(i0 + ox, nx), gxm = pmod(i0 + ox - 1, nx), gxp = pmod(i0 + ox + 1, nx);
  const int gyo = pmod(j0 + oy, ny) * nx, gym = pmod(j0 + oy - 1, ny) * nx, gyp = pmod(j0 + oy + 1, ny) * nx;
  const bool valid = (i0 + ox < nx) && (j0 + oy < ny);
  const int o_t = (oy + 2) * RWD + ox + 4;           // cell planes
  const int o_e = (oy + 1) * EX + ox + 1;            // E planes (P1, W1)
  const int o_u1 = (oy + 1) * (EX + 1) + ox + 1;     // U1
  const int o_v1 = (oy + 1) * EX + ox + 1;           // V1
  const int o_u2 = oy * (OX + 1) + ox, o_v2 = oy * OX + ox, o_w2 = oy * OX + ox;
  // second sub-step-2 wind item (east / north edge faces of O)
  const int gxe2 = tid < OY ? pmod(i0 + OX, nx) : pmod(i0 + (tid - OY), nx);
  const int gye2 = tid < OY ? pmod(j0 + tid, ny) * nx : pmod(j0 + OY, ny) * nx;
  const int e2y = tid < OY ? tid : OY, e2x = tid < OY ? OX : tid - OY;   // O-relative face position
  const int o2_t = (e2y + 2) * RWD + e2x + 4, o2_e = (e2y + 1) * EX + e2x + 1;
  const int o2_u1 = (e2y + 1) * (EX + 1) + e2x + 1, o2_v1 = (e2y + 1) * EX + e2x + 1;
  // sub-step 1 items: E cell tid, then E cell / east edge face / north edge face tid+NT
  const int ex0 = tid % EX, ey0 = tid / EX;
  const int e1 = tid + NT;
  const int kind1 = e1 < NE ? 0 : (e1 < NE + EY ? 1 : (e1 < N1A ? 2 : 3));
  const int ex1 = kind1 == 0 ? e1 % EX : (kind1 == 1 ? EX : e1 - NE - EY);
  const int ey1 = kind1 == 0 ? e1 / EX : (kind1 == 1 ? e1 - NE : EY);
  const int c0 = (ey0 + 1) * RWD + ex0 + 3, f0 = ey0 * RWD + ex0 + 3;   // cell / face plane offsets
  const int u0o = ey0 * (EX + 1) + ex0, e0o = ey0 * EX + ex0;           // U1 / (V1, W1, P1) offsets
  const int c1 = (ey1 + 1) * RWD + ex1 + 3, f1 = ey1 * RWD + ex1 + 3;
  const int u1o = ey1 * (EX + 1) + ex1, e1o = ey1 * EX + ex1;
  __syncthreads();
  // ---- prologue: cell planes of levels n0-1 .. n0+1, face planes of level n0 / face n0+1
  if (n0 >= 1) stage_cells(S, a, plane, n0 - 1, tid);
  stage_cells(S, a, plane, n0, tid);
  if (n0 + 1 < nz) stage_cells(S, a, plane, n0 + 1, tid);
  stage_faces(S, a, plane, n0, n0 + 1 < nz ? n0 + 1 : -1, tid);
  cp_commit();
  if (kb == 0)
    for (int t = tid; t < OX * OY; t += NT) S.W2[0][t / OX][t % OX] = 0.f;
  cp_wait_all();
  __syncthreads();
  // sub-step 1 w on the bottom face n0 of E
  for (int e = tid; e < NE; e += NT) {
    const int ex = e % EX, ey = e / EX;
    float w = 0.f;
    if (n0 > 0) {
      const int cx = ex + 3, ry = ey + 1;
      const int g = n0 * plane + S.gy[ry] + pmod(i0 - 1 + ex, nx);
      w = __ldg(a.w + g) + (pgf(S.TR[n0 % 4][ry][cx], S.TR[(n0 - 1) % 4][ry][cx], S.P0[n0 % 3][ry][cx],
                                S.P0[(n0 - 1) % 3][ry][cx], rdz) +
                            __ldg(a.Rw + g)) *
                               dtau;
    }
    S.W1[n0 % 2][ey][ex] = w;
  }
  // registers: pi'_s around this thread's column at the level whose sub-step-2 pi' is due next
  float q0 = 0.f, qW = 0.f, qE = 0.f, qS = 0.f, qN = 0.f, qB = 0.f, qT = 0.f;
  __syncthreads();

  const float* U0 = &S.U0[0][0];
  const float* RU = &S.RU[0][0];
  const float* V0 = &S.V0[0][0];
  const float* RV = &S.RV[0][0];
  const float* W0 = &S.W0[0][0];
  const float* RWp = &S.RW[0][0];
  for (int n = n0; n <= ke + 1; ++n) {
    const bool s1 = n <= n1;
    const int L2 = n - 1;  // sub-step 2 winds this iteration (Z)
    const bool s2a = L2 >= 0 && L2 >= kb - 1 && L2 < ke;
    const int LB = n - 2;  // sub-step 2 pi' this iteration (X)
    const bool s2b = LB >= kb && LB < ke;
    // ring planes of this iteration
    const int m3 = n % 3, m4 = n % 4, m2 = n & 1;
    const float* P0c = &S.P0[m3][0][0];
    const float* P0u = &S.P0[m3 == 2 ? 0 : m3 + 1][0][0];
    const float* TRc = &S.TR[m4][0][0];
    const float* TRu = &S.TR[(m4 + 1) & 3][0][0];
    const float* TRm = &S.TR[(m4 + 3) & 3][0][0];
    const float* PSc = &S.PS[m4][0][0];
    const float* PSu = &S.PS[(m4 + 1) & 3][0][0];
    const float* PSb = &S.PS[(m4 + 3) & 3][0][0];
    float* U1c = &S.U1[m2][0][0];
    float* V1c = &S.V1[m2][0][0];
    float* W1c = &S.W1[m2][0][0];       // face n
    float* W1u = &S.W1[m2 ^ 1][0][0];   // face n+1
    float* P1c = &S.P1[m2][0][0];
    const float* U1m = &S.U1[m2 ^ 1][0][0];
    const float* V1m = &S.V1[m2 ^ 1][0][0];
    const float* P1m = &S.P1[m2 ^ 1][0][0];
    float* W2n = &S.W2[m2][0][0];       // face n  (= face n-2's slot)
    float* W2m = &S.W2[m2 ^ 1][0][0];   // face n-1
    // ---- cell planes of level n+2 (cp.async) and this iteration's sub-step-2 slow tendencies
    if (n + 1 <= n1 && n + 2 < nz) stage_cells(S, a, plane, n + 2, tid);
    cp_commit();
    float ru = 0.f, rv = 0.f, rw = 0.f, r2 = 0.f;
    if (s2a) {
      const int lp = L2 * plane;
      if (L2 >= kb) {
        ru = __ldg(a.Ru + lp + gyo + gxo);
        rv = __ldg(a.Rv + lp + gyo + gxo);
        if (tid < OY) r2 = __ldg(a.Ru + lp + gye2 + gxe2);
        else if (tid < OY + OX) r2 = __ldg(a.Rv + lp + gye2 + gxe2);
      }
      if (L2 + 1 < nz) rw = __ldg(a.Rw + lp + plane + gyo + gxo);
    }
    // ---- X: sub-step 2 pi' of level n-2, sub-step 1 winds of level n
    if (s2b && valid) {
      const int L = LB;
      const bool has_b = L > 0, has_t = L + 1 < nz;
      const int id = L * plane + gyo + gxo;
      const float uw = S.U2[0][o_u2], ue = S.U2[0][o_u2 + 1];
      const float vs = S.V2[0][o_v2], vn = S.V2[0][o_v2 + OX];
      const float wb = W2n[o_w2], wt = W2m[o_w2];
      const float div = (ue - uw) * rdx + (vn - vs) * rdy + (wt - wb) * rdz;
      const float gxw = (q0 - qW) * rdx, gxe = (qE - q0) * rdx;
      const float gys = (q0 - qS) * rdy, gyn = (qN - q0) * rdy;
      const float wzb = has_b ? wb * (c.dpi0dz[L] + (q0 - qB) * rdz) : 0.f;
      const float wzt = has_t ? wt * (c.dpi0dz[L + 1] + (qT - q0) * rdz) : 0.f;
      const float ap = -(0.5f * (ue * gxe + uw * gxw) + 0.5f * (vn * gyn + vs * gys) +
                         (0.5f * wzb * c.rho_face[L] + 0.5f * wzt * c.rho_face[L + 1]) * c.rho_inv[L]);
      const float dpdt = -kRdCv * ((c.pi0[L] + q0) * div) + ap;
      o.p[id] = P1c[o_e] + (kDivDamp * dpdt) * dtau;  // P1 of level n-2 shares level n's slot
      o.u[id] = uw;
      o.v[id] = vs;
      o.w[id] = wb;
      if (L == nz - 1) o.w[id + plane] = 0.f;
    }
    {  // pi'_s for the next sub-step-2 pi' (level n-1, used in the next iteration's X)
      const int L = n - 1;
      if (L >= kb && L < ke && valid) {
        const int lp = L * plane;
        q0 = __ldg(a.ps + lp + gyo + gxo);
        qW = __ldg(a.ps + lp + gyo + gxm);
        qE = __ldg(a.ps + lp + gyo + gxp);
        qS = __ldg(a.ps + lp + gym + gxo);
        qN = __ldg(a.ps + lp + gyp + gxo);
        qB = L > 0 ? __ldg(a.ps + lp - plane + gyo + gxo) : 0.f;
        qT = L + 1 < nz ? __ldg(a.ps + lp + plane + gyo + gxo) : 0.f;
      }
    }
    if (s1) {
      const bool has_t = n + 1 < nz;
      auto cell = [&](int cc, int ff, int uo, int eo) {
        const float p0 = P0c[cc], t0 = TRc[cc];
        U1c[uo] = U0[ff] + (pgf(t0, TRc[cc - 1], p0, P0c[cc - 1], rdx) + RU[ff]) * dtau;
        V1c[eo] = V0[ff] + (pgf(t0, TRc[cc - RWD], p0, P0c[cc - RWD], rdy) + RV[ff]) * dtau;
        W1u[eo] = has_t ? W0[ff] + (pgf(TRu[cc], t0, P0u[cc], p0, rdz) + RWp[ff]) * dtau : 0.f;
      };
      cell(c0, f0, u0o, e0o);
      if (kind1 == 0) {
        cell(c1, f1, u1o, e1o);
      } else if (kind1 == 1) {  // u on the east face of E's last column
        U1c[u1o] = U0[f1] + (pgf(TRc[c1], TRc[c1 - 1], P0c[c1], P0c[c1 - 1], rdx) + RU[f1]) * dtau;
      } else if (kind1 == 2) {  // v on the north face of E's last row
        V1c[e1o] = V0[f1] + (pgf(TRc[c1], TRc[c1 - RWD], P0c[c1], P0c[c1 - RWD], rdy) + RV[f1]) * dtau;
      }
    }
    __syncthreads();
    // ---- face planes of level n+1 / face n+2 (the ones X just read)
    if (n + 1 <= n1) stage_faces(S, a, plane, n + 1, n + 2 < nz ? n + 2 : -1, tid);
    cp_commit();
    // ---- Y: sub-step 1 pi' of level n
    if (s1) {
      const bool has_b = n > 0, has_t = n + 1 < nz;
      const float rho = c.rho[n], rhoi = c.rho_inv[n], rfb = c.rho_face[n], rft = c.rho_face[n + 1];
      const float dzb = c.dpi0dz[n], dzt = c.dpi0dz[n + 1], pi0 = c.pi0[n];
      auto cell = [&](int cc, int uo, int eo) {
        const float uw = U1c[uo], ue = U1c[uo + 1];
        const float vs = V1c[eo], vn = V1c[eo + EX];
        const float wb = W1c[eo], wt = W1u[eo];
        const float div = (ue - uw) * rdx + (vn - vs) * rdy + (wt - wb) * rdz;
        const float s0 = PSc[cc];
        const float gxw = (s0 - PSc[cc - 1]) * rdx, gxe = (PSc[cc + 1] - s0) * rdx;
        const float gys = (s0 - PSc[cc - RWD]) * rdy, gyn = (PSc[cc + RWD] - s0) * rdy;
        const float wzb = has_b ? wb * (dzb + (s0 - PSb[cc]) * rdz) : 0.f;
        const float wzt = has_t ? wt * (dzt + (PSu[cc] - s0) * rdz) : 0.f;
        const float ap = -(0.5f * (ue * gxe + uw * gxw) + 0.5f * (vn * gyn + vs * gys) +
                           (0.5f * wzb * rfb + 0.5f * wzt * rft) * rhoi);
        const float dpdt = -kRdCv * ((pi0 + s0) * div) + ap;
        P1c[eo] = P0c[cc] + (kDivDamp * dpdt) * dtau;
      };
      cell(c0, u0o, e0o);
      if (kind1 == 0) cell(c1, u1o, e1o);
    }
    __syncthreads();
    // ---- Z: sub-step 2 winds of level n-1 (top face only at level kb-1)
    if (s2a) {
      const bool top_only = L2 < kb;
      const bool has_t = L2 + 1 < nz;
      const float p1 = P1m[o_e];
      const float t0 = TRm[o_t];
      if (!top_only) {
        S.U2[0][o_u2] = U1m[o_u1] + (pgf(t0, TRm[o_t - 1], p1, P1m[o_e - 1], rdx) + ru) * dtau;
        S.V2[0][o_v2] = V1m[o_v1] + (pgf(t0, TRm[o_t - RWD], p1, P1m[o_e - EX], rdy) + rv) * dtau;
        if (tid < OY)  // u on the east face of O's last column
          S.U2[0][tid * (OX + 1) + OX] =
              U1m[o2_u1] + (pgf(TRm[o2_t], TRm[o2_t - 1], P1m[o2_e], P1m[o2_e - 1], rdx) + r2) * dtau;
        else if (tid < OY + OX)  // v on the north face of O's last row
          S.V2[0][OY * OX + (tid - OY)] =
              V1m[o2_v1] + (pgf(TRm[o2_t], TRm[o2_t - RWD], P1m[o2_e], P1m[o2_e - EX], rdy) + r2) * dtau;
      }
      W2n[o_w2] = has_t ? W1c[o_e] + (pgf(TRc[o_t], t0, P1c[o_e], p1, rdz) + rw) * dtau : 0.f;
    }
    cp_wait_all();
    __syncthreads();
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
                            cudaStream_t st, int rev, const cudaAccessPolicyWindow* win) {
  constexpr int VW = ACOUSTIC_VEC;
#if ACOUSTIC_ZMARCH > 0
  if (d.nx % VW == 0) {
    const int nq = d.nx / VW, kc = ACOUSTIC_ZMARCH;
    dim3 b(16, 16, 1);
    dim3 g((nq + b.x - 1) / b.x, (d.ny + b.y - 1) / b.y, (d.nz + kc - 1) / kc);
    k_acoustic_zm<VW><<<g, b, 0, st>>>(d, ph, c, in, out, dtau, kc);
    return cudaGetLastError();
  }
#endif
  if (d.nx % VW == 0) {
    const int nq = d.nx / VW;
    dim3 b(VW == 4 ? 16 : 32, VW == 4 ? 16 : 8, 1);
    dim3 g((nq + b.x - 1) / b.x, (d.ny + b.y - 1) / b.y, d.nz);
    if (win) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = g;
      cfg.blockDim = b;
      cfg.stream = st;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeAccessPolicyWindow;
      at[0].val.accessPolicyWindow = *win;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      return cudaLaunchKernelEx(&cfg, k_acoustic_vec<VW>, d, ph, c, in, out, dtau, rev);
    }
    k_acoustic_vec<VW><<<g, b, 0, st>>>(d, ph, c, in, out, dtau, rev);
    return cudaGetLastError();
  }
  dim3 g((d.nx + BX - 1) / BX, (d.ny + BY - 1) / BY, (d.nz + BZ - 1) / BZ);
  k_acoustic<<<g, dim3(BX, BY, BZ), 0, st>>>(d, ph, c, in, out, dtau);
  return cudaGetLastError();
}

// Levels per block: enough chunks that the grid fills two blocks per SM.
static int pair_chunk(const Dims& d) {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      sms = 152;
  }
  const int cols = ((d.nx + tb::OX - 1) / tb::OX) * ((d.ny + tb::OY - 1) / tb::OY);
  int chunks = (2 * sms) / cols;
  chunks = chunks < 1 ? 1 : (chunks > d.nz ? d.nz : chunks);
  return (d.nz + chunks - 1) / chunks;
}

cudaError_t launch_acoustic_pair(const Dims& d, const Phys& ph, const Cols& c, AcousticIn in, AcousticOut out,
                                 float dtau, cudaStream_t st) {
  if (d.nx % 4 != 0) return cudaErrorInvalidValue;  // staged rows move as float4
  const int kc = pair_chunk(d);
  dim3 g((d.nx + tb::OX - 1) / tb::OX, (d.ny + tb::OY - 1) / tb::OY, (d.nz + kc - 1) / kc);
  k_acoustic_pair<<<g, tb::NT, sizeof(tb::Smem), st>>>(d, ph, c, in, out, dtau, kc);
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
